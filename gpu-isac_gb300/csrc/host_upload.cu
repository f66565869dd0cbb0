// host_upload.cu -- host image lists (one pointer per image, as the
// reference's callers pass them) into device stacks.
//
// Runs of images that lie back to back in host memory (a numpy or EMData
// stack handed over as a pointer list) are copied straight from the caller's
// memory by the copy engine, which reads pageable memory at link speed on a
// GB300 with its Grace host (measured: 1.16 GB in 6-8 ms, against ~97 ms for
// one host thread copying it into pinned memory first).  Scattered images go through
// a double-buffered pinned staging area filled by several host threads.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <thread>
#include <vector>

#include "host_geometry.h"

namespace gpuisac {
namespace {

constexpr unsigned kMinRun = 8;         // shorter runs are staged
constexpr size_t kStageImages = 2048;   // images per staging half
constexpr unsigned kCopyThreads = 8;

struct Staging {
    std::mutex mu;
    float* h = nullptr;
    size_t n = 0; // floats
} g_stage;

} // namespace

void release_upload_staging()
{
    std::lock_guard<std::mutex> lk(g_stage.mu);
    if (g_stage.h)
        cudaFreeHost(g_stage.h);
    g_stage.h = nullptr;
    g_stage.n = 0;
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
    std::vector<unsigned> scattered;
    cudaError_t e = cudaSuccess;
    for (unsigned i = 0; i < n && e == cudaSuccess;) {
        unsigned j = i + 1;
        while (j < n && imgs[j] == imgs[j - 1] + img_elems)
            j++;
        if (j - i >= kMinRun)
            e = cudaMemcpyAsync(dst + (size_t)i * img_elems, imgs[i], (size_t)(j - i) * bytes, cudaMemcpyHostToDevice,
                                stream);
        else
            for (unsigned k = i; k < j; k++)
                scattered.push_back(k);
        i = j;
    }
    if (e != cudaSuccess || scattered.empty())
        return e != cudaSuccess ? e : cudaStreamSynchronize(stream);

    std::lock_guard<std::mutex> lk(g_stage.mu);
    const size_t half = std::min<size_t>(kStageImages, scattered.size());
    if (g_stage.n < 2 * half * img_elems) {
        if (g_stage.h)
            cudaFreeHost(g_stage.h);
        g_stage.h = nullptr;
        g_stage.n = 0;
        e = cudaMallocHost(&g_stage.h, 2 * half * img_elems * sizeof(float));
        if (e != cudaSuccess)
            return e;
        g_stage.n = 2 * half * img_elems;
    }
    cudaEvent_t done[2] = {nullptr, nullptr};
    e = cudaEventCreateWithFlags(&done[0], cudaEventDisableTiming);
    if (e == cudaSuccess)
        e = cudaEventCreateWithFlags(&done[1], cudaEventDisableTiming);
    for (size_t b0 = 0, h = 0; b0 < scattered.size() && e == cudaSuccess; b0 += half, h ^= 1) {
        const size_t m = std::min(half, scattered.size() - b0);
        float* stage = g_stage.h + h * half * img_elems;
        e = cudaEventSynchronize(done[h]); // this half's previous copies have left
        if (e != cudaSuccess)
            break;
        const unsigned nt = (unsigned)std::min<size_t>(kCopyThreads, (m + 63) / 64);
        auto copy_part = [&](unsigned t) {
            for (size_t q = m * t / nt; q < m * (t + 1) / nt; q++)
                std::memcpy(stage + q * img_elems, imgs[scattered[b0 + q]], bytes);
        };
        std::vector<std::thread> pool;
        for (unsigned t = 1; t < nt; t++)
            pool.emplace_back(copy_part, t);
        copy_part(0);
        for (auto& th : pool)
            th.join();
        // consecutive list entries are often consecutive slots: one copy per run
        for (size_t q = 0; q < m && e == cudaSuccess;) {
            size_t r = q + 1;
            while (r < m && scattered[b0 + r] == scattered[b0 + r - 1] + 1)
                r++;
            e = cudaMemcpyAsync(dst + (size_t)scattered[b0 + q] * img_elems, stage + q * img_elems, (r - q) * bytes,
                                cudaMemcpyHostToDevice, stream);
            q = r;
        }
        if (e == cudaSuccess)
            e = cudaEventRecord(done[h], stream);
    }
    cudaError_t s = cudaStreamSynchronize(stream);
    if (done[0])
        cudaEventDestroy(done[0]);
    if (done[1])
        cudaEventDestroy(done[1]);
    return e != cudaSuccess ? e : s;
}

} // namespace gpuisac
