// host_upload.cu -- host image lists (one pointer per image, as the
// reference's callers pass them) into device stacks.
//
// Pageable memory goes through pinned staging.  The copy engine can read
// pageable memory on a GB300 with its Grace host, and does so at link speed
// once the pages are mapped for the device, but the first copy of a buffer
// pays for that mapping: measured 55-170 ms for the 1.16 GB stack of 50,000
// 76x76 images (growing with the processes a box has run), against 6 ms for
// the same copy repeated -- and the caller's arrays are new to the device at
// every call.  Host threads copying into pinned memory run at the host's
// memory bandwidth every time (1.16 GB in 10 ms with 16 threads, 84 ms with
// one), and the DMA out of pinned memory (5.5 ms) overlaps them.
//
// The destination stack is cut into pieces of kSlotBytes; worker t takes
// pieces t, t + T, ... into its own two pinned slots in turn, gathering the
// piece from the caller's image pointers, and queues the slot's copy on the
// caller's stream; a slot is refilled once its previous copy has left (an
// event per slot).  A source that is one contiguous run of pinned memory is
// copied directly.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstring>
#include <mutex>
#include <thread>
#include <vector>

#include "host_geometry.h"

namespace gpuisac {
namespace {

constexpr size_t kSlotBytes = 2u << 20;
constexpr unsigned kMaxWorkers = 16;

struct Staging {
    std::mutex mu;
    unsigned char* h = nullptr;
    size_t bytes = 0;
} g_stage;

} // namespace

void release_upload_staging()
{
    std::lock_guard<std::mutex> lk(g_stage.mu);
    if (g_stage.h)
        cudaFreeHost(g_stage.h);
    g_stage.h = nullptr;
    g_stage.bytes = 0;
}

cudaError_t upload_host_images(const float* const* imgs, unsigned n, size_t img_elems, float* dst,
                               cudaStream_t stream, unsigned* bad)
{
    for (unsigned i = 0; i < n; i++)
        if (!imgs[i]) {
            if (bad)
                *bad = i;
            return cudaErrorInvalidValue;
        }
    const size_t bytes = img_elems * sizeof(float);
    const size_t total = (size_t)n * bytes;
    if (total == 0)
        return cudaSuccess;

    // one contiguous run of pinned memory: straight copy
    bool contiguous = true;
    for (unsigned i = 1; i < n && contiguous; i++)
        contiguous = imgs[i] == imgs[i - 1] + img_elems;
    if (contiguous) {
        cudaPointerAttributes a{};
        if (cudaPointerGetAttributes(&a, imgs[0]) == cudaSuccess && a.type == cudaMemoryTypeHost) {
            cudaError_t e = cudaMemcpyAsync(dst, imgs[0], total, cudaMemcpyHostToDevice, stream);
            return e != cudaSuccess ? e : cudaStreamSynchronize(stream);
        }
        (void)cudaGetLastError(); // pageable pointers may report an error on older drivers
    }

    const size_t n_pieces = (total + kSlotBytes - 1) / kSlotBytes;
    unsigned hw = std::thread::hardware_concurrency();
    const unsigned T = (unsigned)std::min<size_t>(std::min(kMaxWorkers, std::max(1u, hw)), n_pieces);

    std::lock_guard<std::mutex> lk(g_stage.mu);
    const size_t need = (size_t)2 * T * kSlotBytes;
    if (g_stage.bytes < need) {
        if (g_stage.h)
            cudaFreeHost(g_stage.h);
        g_stage.h = nullptr;
        g_stage.bytes = 0;
        cudaError_t e = cudaMallocHost(&g_stage.h, need);
        if (e != cudaSuccess)
            return e;
        g_stage.bytes = need;
    }
    std::vector<cudaEvent_t> ev(2 * T, nullptr);
    cudaError_t e = cudaSuccess;
    for (unsigned i = 0; i < 2 * T && e == cudaSuccess; i++)
        e = cudaEventCreateWithFlags(&ev[i], cudaEventDisableTiming);

    int dev = 0;
    if (e == cudaSuccess)
        e = cudaGetDevice(&dev);
    std::atomic<int> first_err{(int)e};
    unsigned char* d = reinterpret_cast<unsigned char*>(dst);
    auto fail = [&](cudaError_t r) {
        int expect = 0;
        first_err.compare_exchange_strong(expect, (int)r);
    };
    auto work = [&](unsigned t) {
        cudaError_t r0 = cudaSetDevice(dev); // a new thread starts on device 0
        if (r0 != cudaSuccess) {
            fail(r0);
            return;
        }
        size_t k = 0;
        for (size_t p = t; p < n_pieces && first_err.load(std::memory_order_relaxed) == 0; p += T, k++) {
            const unsigned slot = 2 * t + (unsigned)(k & 1);
            unsigned char* stage = g_stage.h + (size_t)slot * kSlotBytes;
            cudaError_t r = cudaEventSynchronize(ev[slot]); // the slot's previous copy has left
            const size_t x0 = p * kSlotBytes, x1 = std::min(total, x0 + kSlotBytes);
            if (r == cudaSuccess) {
                for (size_t x = x0; x < x1;) {
                    const size_t i = x / bytes, within = x - i * bytes;
                    const size_t len = std::min(bytes - within, x1 - x);
                    std::memcpy(stage + (x - x0), reinterpret_cast<const unsigned char*>(imgs[i]) + within, len);
                    x += len;
                }
                r = cudaMemcpyAsync(d + x0, stage, x1 - x0, cudaMemcpyHostToDevice, stream);
            }
            if (r == cudaSuccess)
                r = cudaEventRecord(ev[slot], stream);
            if (r != cudaSuccess) {
                fail(r);
                break;
            }
        }
        // this worker's copies have left its slots before it returns
        for (unsigned slot = 2 * t; slot < 2 * t + 2; slot++) {
            const cudaError_t r = cudaEventSynchronize(ev[slot]);
            if (r != cudaSuccess)
                fail(r);
        }
    };
    if (e == cudaSuccess) {
        std::vector<std::thread> pool;
        for (unsigned t = 1; t < T; t++)
            pool.emplace_back(work, t);
        work(0);
        for (auto& th : pool)
            th.join();
    }
    cudaError_t s = cudaStreamSynchronize(stream);
    for (cudaEvent_t x : ev)
        if (x)
            cudaEventDestroy(x);
    e = (cudaError_t)first_err.load();
    return e != cudaSuccess ? e : s;
}

} // namespace gpuisac
