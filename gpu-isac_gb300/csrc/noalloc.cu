// noalloc.cu -- gpuisac_multi_ref_align_device_noalloc: the device-resident
// alignment without any device memory allocation.
//
// Some callers cannot call cudaMalloc: a host program whose GPU memory is
// owned by another allocator (a framework's caching allocator that has
// reserved nearly all of the device, or a runtime that forbids allocation
// after start-up), or code that must not pay the implicit device-wide
// synchronisation cudaMalloc / cudaFree can cause in the middle of its stream
// work.  They pass their inputs and outputs; the work space this pipeline
// needs (the polar template, twiddles and shift tables, the reference
// spectra, and one chunk of particle spectra at a time) lives in one
// file-scope device array built into the library.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <mutex>
#include <vector>

#include "../../include/gpu_aln_pack.h"
#include "gpuisac_kernels.h"
#include "host_geometry.h"

using namespace gpuisac;

// 32 MiB of work space.  Every GPU that loads this library holds it until the
// process exits.  No region of it needs to start at zero: each call writes
// every part it reads before reading it, so what a previous call left behind
// is never used.
constexpr size_t kNoAllocScratchBytes = size_t(32) << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;                   // one call at a time: every call shares the array
unsigned char* g_noalloc_dev[kMaxDevices]; // device address of the array, per device

size_t up256(size_t b) { return (b + 255) & ~size_t(255); }

int fail(int code, const char* msg)
{
    record_error(code, msg);
    return code;
}

#define NA_CK(expr)                                                                     \
    do {                                                                                \
        cudaError_t e_ = (expr);                                                        \
        if (e_ != cudaSuccess) {                                                        \
            char m_[384];                                                               \
            snprintf(m_, sizeof(m_), "%s (%s) in the allocation-free entry point",      \
                     cudaGetErrorString(e_), #expr);                                    \
            return fail(1, m_);                                                         \
        }                                                                               \
    } while (0)

} // namespace

namespace {

// the array carved for one call: tables, reference spectra, then as many
// particles' spectra as fit
struct Carve {
    size_t off_err, off_tw, off_zero, off_tmpl, off_sf, off_si, off_ref, off_sbj, per_particle, need;
    unsigned chunk;
};

Carve carve(const HostGeometry& g)
{
    Carve c;
    const size_t row_bytes = (size_t)g.NR * kSlots * sizeof(float2); // one (image, shift) row
    c.off_err = 0;
    c.off_tw = c.off_err + 256;
    c.off_zero = c.off_tw + up256(kRingLen * sizeof(float2));
    c.off_tmpl = c.off_zero + up256(sizeof(int2));
    c.off_sf = c.off_tmpl + up256(g.tmpl.size() * sizeof(float2));
    c.off_si = c.off_sf + up256((size_t)g.S * sizeof(float2));
    c.off_ref = c.off_si + up256((size_t)g.S * sizeof(int2));
    c.off_sbj = c.off_ref + up256((size_t)g.R * row_bytes);
    c.per_particle = (size_t)g.S * row_bytes;
    c.need = c.off_sbj + c.per_particle;
    c.chunk = c.need > kNoAllocScratchBytes
                  ? 0u
                  : (unsigned)std::min<size_t>((kNoAllocScratchBytes - c.off_sbj) / c.per_particle, g.P);
    return c;
}

int enqueue_and_wait(const HostGeometry& g, const Carve& c, unsigned char* base, cudaStream_t st, const float* sbj,
                     const float* ref, const float* base_shift, float* d_out, float* peak_out, int dev);
} // namespace

extern "C" int gpuisac_multi_ref_align_device_noalloc(const AlignConfig* cfg, const float* sbj, const float* ref,
                                                      const float* base_shift, float* d_out, float* peak_out,
                                                      void* stream)
{
    HostGeometry g;
    int rc = host_geometry(cfg, g);
    if (rc)
        return rc;
    if (!sbj || !ref || !d_out || !peak_out)
        return fail(2, "NULL device pointer");
    if (g.P == 0 || g.R == 0)
        return 0;

    const Carve c = carve(g);
    if (c.chunk == 0) {
        char m[320];
        snprintf(m, sizeof(m),
                 "workload needs %zu bytes of work space (reference spectra + one particle's spectra); the "
                 "allocation-free entry point has %zu: use gpuisac_multi_ref_align_device",
                 c.need, kNoAllocScratchBytes);
        return fail(2, m);
    }

    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    int dev = 0;
    NA_CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices)
        return fail(2, "device index outside the allocation-free entry point's table");
    if (!g_noalloc_dev[dev]) {
        // set-up, once per device, with that device current: the array's
        // name is only a host-side stand-in; its device address comes from
        // the runtime
        void* p = nullptr;
        NA_CK(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        g_noalloc_dev[dev] = static_cast<unsigned char*>(p);
    }
    unsigned char* base = g_noalloc_dev[dev];

    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // From the first enqueue on, work on `st` reads and writes the shared
    // array: a failure returns only after that work has finished, so that
    // the next caller (another stream, once the lock is released) cannot
    // overwrite the array under it.
    const int rc2 = enqueue_and_wait(g, c, base, st, sbj, ref, base_shift, d_out, peak_out, dev);
    if (rc2)
        cudaStreamSynchronize(st); // its own error, if any, is already recorded
    return rc2;
}

namespace {

// enqueue the whole alignment on st and wait for it (the host tables and the
// shared array must outlive the work)
int enqueue_and_wait(const HostGeometry& g, const Carve& c, unsigned char* base, cudaStream_t st, const float* sbj,
                     const float* ref, const float* base_shift, float* d_out, float* peak_out, int dev)
{
    const unsigned chunk = c.chunk;
    unsigned* err = reinterpret_cast<unsigned*>(base + c.off_err);
    float2* tw = reinterpret_cast<float2*>(base + c.off_tw);
    int2* zero = reinterpret_cast<int2*>(base + c.off_zero);
    float2* tmpl = reinterpret_cast<float2*>(base + c.off_tmpl);
    float2* sf = reinterpret_cast<float2*>(base + c.off_sf);
    int2* si = reinterpret_cast<int2*>(base + c.off_si);
    float2* ref_sp = reinterpret_cast<float2*>(base + c.off_ref);
    float2* sbj_sp = reinterpret_cast<float2*>(base + c.off_sbj);

    const int2 zero_h = make_int2(0, 0);
    NA_CK(cudaMemsetAsync(err, 0, sizeof(unsigned), st));
    NA_CK(cudaMemcpyAsync(tw, g.tw.data(), kRingLen * sizeof(float2), cudaMemcpyHostToDevice, st));
    NA_CK(cudaMemcpyAsync(zero, &zero_h, sizeof(int2), cudaMemcpyHostToDevice, st));
    NA_CK(cudaMemcpyAsync(tmpl, g.tmpl.data(), g.tmpl.size() * sizeof(float2), cudaMemcpyHostToDevice, st));
    NA_CK(cudaMemcpyAsync(sf, g.shifts_f.data(), g.S * sizeof(float2), cudaMemcpyHostToDevice, st));
    NA_CK(cudaMemcpyAsync(si, g.shifts_i.data(), g.S * sizeof(int2), cudaMemcpyHostToDevice, st));

    const unsigned tex = texture_images(dev, g.D);
    const unsigned ref_batch = std::max(1u, std::min(g.R, 100u));
    if (ref_batch > tex)
        return fail(4, "reference batch exceeds one texture");
    StackDesc refs{ref, g.R, g.D, ref_batch, tex};
    StackDesc sbjs{sbj, g.P, g.D, g.sbj_batch, tex};
    const float2* bs = reinterpret_cast<const float2*>(base_shift);
    NA_CK(launch_polar_spectra(refs, tmpl, tw, g.NR, zero, 1, nullptr, 0, g.R, 1, ref_sp, st));
    for (unsigned p0 = 0; p0 < g.P; p0 += chunk) {
        const unsigned n = std::min(chunk, g.P - p0);
        NA_CK(launch_polar_spectra(sbjs, tmpl, tw, g.NR, si, g.S, bs, p0, n, 0, sbj_sp, st));
        NA_CK(launch_ccf_peak(sbj_sp, ref_sp, tw, g.NR, g.S, g.R, n, p0, g.P, sf, bs, d_out,
                              reinterpret_cast<float4*>(peak_out), err, st));
    }
    NA_CK(cudaStreamSynchronize(st));
    unsigned flag = 0;
    NA_CK(cudaMemcpy(&flag, err, sizeof(unsigned), cudaMemcpyDeviceToHost));
    if (flag)
        return fail(1, "a kernel timed out waiting for its own asynchronous copies");
    return 0;
}

} // namespace
