// align_abi.cu -- the C-ABI of libgpu_aln_pack.so: the reference's exports
// (include/gpu_aln_pack.h) on top of the GB300 kernels.
//
// Process-global state mirrors the reference's AlignmentResources singleton
// (cuda/gpu_aln_noref.cu:29-48): one configuration, one device, one
// host-writable AlignParam array per init/clear cycle.  Unlike the reference,
// CUDA failures never exit the process: they are recorded (gpuisac_last_error),
// printed to stderr, and the call returns.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/gpu_aln_pack.h"
#include "gpuisac_kernels.h"
#include "gpuisac_split.h"
#include "host_geometry.h"

using namespace gpuisac;

namespace {

// ---------------------------------------------------------------- errors
std::mutex g_err_mu;
int g_err_code = 0;
std::string g_err_msg;

void set_error(int code, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    {
        std::lock_guard<std::mutex> lk(g_err_mu);
        g_err_code = code;
        g_err_msg = buf;
    }
    fprintf(stderr, "gpuisac error %d: %s\n", code, buf);
}

enum ErrCode {
    E_CUDA = 1,
    E_ARG = 2,
    E_STATE = 3,
    E_UNSUPPORTED = 4,
    E_NOMEM = 5,
};

#define CK(expr)                                                                                  \
    do {                                                                                          \
        cudaError_t e_ = (expr);                                                                  \
        if (e_ != cudaSuccess) {                                                                  \
            set_error(E_CUDA, "%s (%s) at %s:%d", cudaGetErrorString(e_), #expr, __FILE__, __LINE__); \
            return E_CUDA;                                                                        \
        }                                                                                         \
    } while (0)

// ---------------------------------------------------------------- geometry
struct Geometry {
    unsigned P = 0, R = 0, D = 0, NR = 0, L = 0, S = 0;
    std::vector<float2> shifts_f; // the reference's float shift grid
    std::vector<int2> shifts_i;   // truncated to int as the resample kernel receives them
    std::vector<float2> tmpl;     // polar template [NR][L]
};

// Reference: generate_shift_array, cuda/gpu_aln_common.cu:64-86
std::vector<float2> shift_grid(float rx, float ry, float step)
{
    std::vector<float2> v;
    if (!(step > 0.f))
        return v;
    for (float sx = -rx; sx <= rx; sx += step)
        for (float sy = -ry; sy <= ry; sy += step) {
            v.push_back(make_float2(sx, sy));
            if (v.size() > kMaxShifts)
                return v;
        }
    return v;
}

// Reference: generate_polar_sampling_points, cuda/gpu_aln_common.cu:39-62
// (host libm, float products, same operation order)
std::vector<float2> polar_template(unsigned ring_num, unsigned ring_len)
{
    std::vector<float2> t((size_t)ring_num * ring_len);
    for (unsigned i = 0; i < ring_num; i++)
        for (unsigned j = 0; j < ring_len; j++) {
            volatile float angle = (float)((double)((float)j / (float)ring_len) * 3.14159265358979 * 2);
            volatile float cx = cosf(angle) * (float)(i + 1);
            volatile float sy = sinf(angle) * (float)(i + 1);
            volatile float ox = cx * (float)ring_num;
            volatile float oy = sy * (float)ring_num;
            t[(size_t)i * ring_len + j] = make_float2(ox / (float)ring_num, oy / (float)ring_num);
        }
    return t;
}

// ring_len: 256 everywhere; 512 where allow_l512 (the multi-reference calls,
// ring512.cu)
int validate(const AlignConfig* cfg, Geometry& g, bool need_type, bool allow_l512 = false)
{
    if (!cfg) {
        set_error(E_ARG, "AlignConfig is NULL");
        return E_ARG;
    }
    if (need_type && cfg->aln_type && std::strcmp(cfg->aln_type, "mref_aln") != 0) {
        set_error(E_UNSUPPORTED, "aln_type '%s' is not the multi-reference path ('mref_aln')", cfg->aln_type);
        return E_UNSUPPORTED;
    }
    if (cfg->ring_len != (unsigned)kRingLen && !(allow_l512 && cfg->ring_len == (unsigned)kRingLen512)) {
        set_error(E_UNSUPPORTED, "ring_len %u unsupported (256-sample rings%s)", cfg->ring_len,
                  allow_l512 ? "; 512 on the multi-reference path" : " on this entry point");
        return E_UNSUPPORTED;
    }
    if (cfg->ring_num == 0 || cfg->ring_num > kMaxRingNum) {
        set_error(E_UNSUPPORTED, "ring_num %u outside 1..%u", cfg->ring_num, kMaxRingNum);
        return E_UNSUPPORTED;
    }
    if (cfg->img_dim < 2 || cfg->img_dim > 4096) {
        set_error(E_ARG, "img_dim %u outside 2..4096", cfg->img_dim);
        return E_ARG;
    }
    if (!(cfg->shift_step > 0.f) || !(cfg->shift_rng_x >= 0.f) || !(cfg->shift_rng_y >= 0.f)) {
        set_error(E_ARG, "shift grid needs step > 0 and ranges >= 0");
        return E_ARG;
    }
    std::vector<float2> sf = shift_grid(cfg->shift_rng_x, cfg->shift_rng_y, cfg->shift_step);
    if (sf.empty() || sf.size() > kMaxShifts) {
        set_error(E_UNSUPPORTED, "shift grid has %zu entries (1..%u supported)", sf.size(), kMaxShifts);
        return E_UNSUPPORTED;
    }
    g.P = cfg->sbj_num;
    g.R = cfg->ref_num;
    g.D = cfg->img_dim;
    g.NR = cfg->ring_num;
    g.L = cfg->ring_len;
    g.S = (unsigned)sf.size();
    g.shifts_f = sf;
    g.shifts_i.resize(sf.size());
    for (size_t i = 0; i < sf.size(); i++)
        g.shifts_i[i] = make_int2((int)sf[i].x, (int)sf[i].y);
    g.tmpl = polar_template(g.NR, g.L);
    return 0;
}

// Reference subject batch size: the binary search of multi_ref_align
// (cuda/gpu_aln_noref.cu:433-440) against the cuFFT int32 guard of
// multi_ref_align_size_check (:238); the device-memory half of that check
// passes for any workload this library accepts on a GB300.
unsigned reference_sbj_batch(const AlignConfig* cfg)
{
    unsigned ref_b = std::min(cfg->ref_num, 100u);
    size_t shift_num = (size_t)((2 * (cfg->shift_rng_x / cfg->shift_step) + 1) *
                                (2 * (cfg->shift_rng_y / cfg->shift_step) + 1));
    unsigned bs = 0;
    if (cfg->sbj_num == 0)
        return 0;
    for (int i = (int)std::log2((double)cfg->sbj_num); i >= 0; i--) {
        unsigned split = (unsigned)std::pow(2.0, i);
        unsigned cand = std::min(bs + split, cfg->sbj_num);
        size_t entries = (size_t)cand * ref_b * (shift_num * 2) * (size_t)(cfg->ring_len + 2);
        if (entries <= (((size_t)1) << 31) - 1)
            bs = cand;
    }
    return bs;
}

unsigned texture_image_limit(int dev, unsigned dim)
{
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess)
        return 65000u / dim;
    return (unsigned)prop.maxTexture2DLinear[1] / dim;
}

// ---------------------------------------------------------------- device buffers
std::atomic<unsigned> g_fail_allocs{0};

template <typename T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    int ensure(size_t count)
    {
        if (count <= n)
            return 0;
        if (p)
            cudaFree(p);
        p = nullptr;
        n = 0;
        if (take_injected_alloc_failure()) {
            set_error(E_NOMEM, "cudaMalloc of %zu bytes failed: injected (gpuisac_test_fail_alloc)",
                      count * sizeof(T));
            return E_NOMEM;
        }
        cudaError_t e = cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T));
        if (e != cudaSuccess) {
            set_error(E_NOMEM, "cudaMalloc of %zu bytes failed: %s", count * sizeof(T), cudaGetErrorString(e));
            p = nullptr;
            return E_NOMEM;
        }
        n = count;
        return 0;
    }
    void release()
    {
        if (p)
            cudaFree(p);
        p = nullptr;
        n = 0;
    }
};

struct Workspace {
    // geometry currently uploaded (skip re-uploading an unchanged one)
    unsigned geo_D = 0, geo_NR = 0, geo_L = 0;
    std::vector<float2> geo_shifts;
    DevBuf<float2> tmpl, tw, tw512, shifts_f, ref_sp, sbj_sp, base;
    DevBuf<int2> shifts_i, zero_shift;
    DevBuf<unsigned> err; // device-side timeout flag of the kernels' bounded waits
    DevBuf<unsigned char> sop, rop; // BF16 hi/lo operands of the tensor-core contraction
    DevBuf<float2> zsp;             // its pair spectra
    TexStack ref_tex, sbj_tex; // the stacks as textures for the texture unit
    cudaStream_t copy_stream = nullptr; // results to the host, overlapping the next chunk
    cudaEvent_t chunk_done[2] = {nullptr, nullptr};
    // tensor-core path: contraction and FFT on a high-priority stream, the next
    // chunk's operand kernel on a low-priority one (events between them)
    cudaStream_t split_hi = nullptr, split_lo = nullptr;
    cudaEvent_t ops_done[2] = {nullptr, nullptr}, mma_done[2] = {nullptr, nullptr};
    cudaEvent_t split_entry = nullptr, split_exit = nullptr;
    void release()
    {
        for (int i = 0; i < 2; i++) {
            if (ops_done[i])
                cudaEventDestroy(ops_done[i]);
            if (mma_done[i])
                cudaEventDestroy(mma_done[i]);
            ops_done[i] = mma_done[i] = nullptr;
        }
        if (split_entry)
            cudaEventDestroy(split_entry);
        if (split_exit)
            cudaEventDestroy(split_exit);
        split_entry = split_exit = nullptr;
        if (split_hi)
            cudaStreamDestroy(split_hi);
        if (split_lo)
            cudaStreamDestroy(split_lo);
        split_hi = split_lo = nullptr;
        for (int i = 0; i < 2; i++) {
            if (chunk_done[i])
                cudaEventDestroy(chunk_done[i]);
            chunk_done[i] = nullptr;
        }
        if (copy_stream)
            cudaStreamDestroy(copy_stream);
        copy_stream = nullptr;
        err.release();
        sop.release();
        rop.release();
        zsp.release();
        ref_tex.release();
        sbj_tex.release();
        geo_D = geo_NR = geo_L = 0;
        geo_shifts.clear();
        zero_shift.release();
        tmpl.release();
        tw.release();
        tw512.release();
        shifts_f.release();
        ref_sp.release();
        sbj_sp.release();
        base.release();
        shifts_i.release();
    }
};

// forward twiddles e^(-2 pi i e / n), computed in double
std::vector<float2> twiddles(int n = kRingLen)
{
    std::vector<float2> t(n);
    for (int e = 0; e < n; e++) {
        double a = -2.0 * M_PI * (double)e / (double)n;
        t[e] = make_float2((float)std::cos(a), (float)std::sin(a));
    }
    return t;
}

int upload_geometry(const Geometry& g, Workspace& ws, cudaStream_t st)
{
    if (ws.geo_D == g.D && ws.geo_NR == g.NR && ws.geo_L == g.L && ws.geo_shifts.size() == g.shifts_f.size() &&
        ws.tmpl.p && std::memcmp(ws.geo_shifts.data(), g.shifts_f.data(), g.shifts_f.size() * sizeof(float2)) == 0)
        return 0;
    if (ws.tmpl.ensure(g.tmpl.size()) || ws.tw.ensure(kRingLen) || ws.tw512.ensure(kRingLen512) ||
        ws.shifts_f.ensure(g.S) || ws.shifts_i.ensure(g.S) || ws.zero_shift.ensure(1))
        return E_NOMEM;
    std::vector<float2> tw = twiddles(), tw512 = twiddles(kRingLen512);
    CK(cudaMemcpyAsync(ws.tw512.p, tw512.data(), tw512.size() * sizeof(float2), cudaMemcpyHostToDevice, st));
    const int2 zero = make_int2(0, 0);
    CK(cudaMemcpyAsync(ws.zero_shift.p, &zero, sizeof(int2), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(ws.tmpl.p, g.tmpl.data(), g.tmpl.size() * sizeof(float2), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(ws.tw.p, tw.data(), tw.size() * sizeof(float2), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(ws.shifts_f.p, g.shifts_f.data(), g.S * sizeof(float2), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(ws.shifts_i.p, g.shifts_i.data(), g.S * sizeof(int2), cudaMemcpyHostToDevice, st));
    // the host vectors die with this call: finish the copies first
    CK(cudaStreamSynchronize(st));
    ws.geo_D = g.D;
    ws.geo_NR = g.NR;
    ws.geo_L = g.L;
    ws.geo_shifts = g.shifts_f;
    return 0;
}

// after the stream has been synchronised: did a kernel give up a bounded wait?
int check_device_flag(Workspace& ws)
{
    if (!ws.err.p)
        return 0;
    unsigned h = 0;
    CK(cudaMemcpy(&h, ws.err.p, sizeof(unsigned), cudaMemcpyDeviceToHost));
    if (h) {
        set_error(E_CUDA, "a kernel timed out waiting for its own asynchronous copies (flag %u)", h);
        return E_CUDA;
    }
    return 0;
}

// ---------------------------------------------------------------- kernel timing
// Optional CUDA-event timing of every kernel launch of the pipeline, on the
// stream the kernel runs on (gpuisac_profile / gpuisac_kernel_time).
struct KernelTimer {
    bool on = false;
    struct Pending {
        int kind;
        cudaEvent_t a, b;
    };
    std::vector<Pending> pending;
    unsigned long long launches[4] = {0, 0, 0, 0};
    double ms[4] = {0.0, 0.0, 0.0, 0.0};
    cudaEvent_t begin(cudaStream_t st)
    {
        if (!on)
            return nullptr;
        cudaEvent_t e = nullptr;
        if (cudaEventCreate(&e) != cudaSuccess)
            return nullptr;
        cudaEventRecord(e, st);
        return e;
    }
    void end(int kind, cudaEvent_t a, cudaStream_t st)
    {
        if (!on || !a)
            return;
        cudaEvent_t b = nullptr;
        if (cudaEventCreate(&b) != cudaSuccess) {
            cudaEventDestroy(a);
            return;
        }
        cudaEventRecord(b, st);
        pending.push_back({kind, a, b});
    }
    // after the stream has been synchronised
    void collect()
    {
        for (auto& p : pending) {
            float t = 0.f;
            if (cudaEventElapsedTime(&t, p.a, p.b) == cudaSuccess) {
                launches[p.kind]++;
                ms[p.kind] += t;
            }
            cudaEventDestroy(p.a);
            cudaEventDestroy(p.b);
        }
        pending.clear();
    }
} g_timer;
enum { K_SPECTRA = 0, K_CCF = 1, K_MMA = 2, K_ZFFT = 3 };

// ---------------------------------------------------------------- contraction
// Arithmetic of the ring-summed contraction: FP32 on the CUDA cores (the
// drop-in default) or BF16 hi/lo split on the tensor cores.  The environment
// variable GPUISAC_CONTRACTION=bf16x3 selects the latter at load time, so an
// unchanged caller of the reference's entry points can opt in.
std::atomic<int> g_contraction{-1};
thread_local int t_contraction_forced = -1;

int contraction_mode()
{
    if (t_contraction_forced >= 0)
        return t_contraction_forced;
    int m = g_contraction.load();
    if (m < 0) {
        const char* e = getenv("GPUISAC_CONTRACTION");
        m = (e && std::strcmp(e, "bf16x3") == 0) ? GPUISAC_CONTRACTION_BF16X3 : GPUISAC_CONTRACTION_FP32;
        int expected = -1;
        g_contraction.compare_exchange_strong(expected, m);
        m = g_contraction.load();
    }
    return m;
}

// ---------------------------------------------------------------- the pipeline
// Host destinations of the results (the reference-facing call): d [R][pitch]
// and peak_list [R][4P] in the caller's memory.
struct HostOut {
    float* d = nullptr;
    unsigned d_pitch = 0;
    float* peak = nullptr;
};

// results of particles c0 .. c0 + cn - 1 to the host (copy stream, after the
// chunk's kernels: event ev)
int copy_chunk_back(const Geometry& g, Workspace& ws, const HostOut* host, const float* d_out, const float4* d_peak,
                    unsigned c0, unsigned cn, cudaEvent_t ev)
{
    CK(cudaStreamWaitEvent(ws.copy_stream, ev, 0));
    CK(cudaMemcpy2DAsync(host->d + c0, (size_t)host->d_pitch * sizeof(float), d_out + c0, (size_t)g.P * sizeof(float),
                         (size_t)cn * sizeof(float), g.R, cudaMemcpyDeviceToHost, ws.copy_stream));
    CK(cudaMemcpy2DAsync(host->peak + 4 * (size_t)c0, (size_t)g.P * sizeof(float4), d_peak + c0,
                         (size_t)g.P * sizeof(float4), (size_t)cn * sizeof(float4), g.R, cudaMemcpyDeviceToHost,
                         ws.copy_stream));
    return 0;
}

int prepare_copy_back(Workspace& ws)
{
    if (!ws.copy_stream)
        CK(cudaStreamCreateWithFlags(&ws.copy_stream, cudaStreamNonBlocking));
    for (int i = 0; i < 2; i++)
        if (!ws.chunk_done[i])
            CK(cudaEventCreateWithFlags(&ws.chunk_done[i], cudaEventDisableTiming));
    return 0;
}

// The same alignment with the contraction on the tensor cores: reference
// operands once, then per particle chunk the subject operands, the MMA kernel
// (pair spectra to HBM) and the inverse-FFT / peak kernel.
// the tensor-core path's streams and events (created once per workspace)
int prepare_split_streams(Workspace& ws)
{
    if (ws.split_hi)
        return 0;
    int least = 0, greatest = 0;
    CK(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    CK(cudaStreamCreateWithPriority(&ws.split_hi, cudaStreamNonBlocking, greatest));
    CK(cudaStreamCreateWithPriority(&ws.split_lo, cudaStreamNonBlocking, least));
    for (int i = 0; i < 2; i++) {
        CK(cudaEventCreateWithFlags(&ws.ops_done[i], cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&ws.mma_done[i], cudaEventDisableTiming));
    }
    CK(cudaEventCreateWithFlags(&ws.split_entry, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&ws.split_exit, cudaEventDisableTiming));
    return 0;
}

int run_alignment_split(const Geometry& g, Workspace& ws, const StackDesc& refs, const StackDesc& sbjs,
                        const unsigned long long* ref_tx, const unsigned long long* sbj_tx, const float2* d_base,
                        float* d_out, float4* d_peak, float mem_request, cudaStream_t st, const HostOut* host)
{
    SplitPlan pl;
    if (!split_plan(g.NR, g.S, g.R, pl)) {
        set_error(E_UNSUPPORTED, "the tensor-core contraction has no tile plan for %u rings, %u shifts, %u references",
                  g.NR, g.S, g.R);
        return E_UNSUPPORTED;
    }
    if (ws.rop.ensure(split_rop_bytes(pl)))
        return E_NOMEM;
    int rc = prepare_split_streams(ws);
    if (rc)
        return rc;
    // work of the call: the contraction and the FFT on `hi`, the particle
    // operands on `lo` -- a lower priority, so that one operand CTA shares each
    // SM with the contraction's persistent CTA instead of delaying it (575.7
    // -> 559.5 ms per 50,000 x 200 step) -- both after the caller's earlier
    // work on st, and st after both
    cudaStream_t hi = ws.split_hi, lo = ws.split_lo;
    CK(cudaEventRecord(ws.split_entry, st));
    CK(cudaStreamWaitEvent(hi, ws.split_entry, 0));
    CK(cudaStreamWaitEvent(lo, ws.split_entry, 0));
    cudaEvent_t ev = g_timer.begin(hi);
    CK(launch_polar_operands(refs, ws.tmpl.p, ws.tw.p, g.NR, ws.zero_shift.p, 1, nullptr, 0, g.R, 1,
                             split_ref_layout(pl, ws.rop.p), hi, ref_tx));
    g_timer.end(K_SPECTRA, ev, hi);
    // particle chunk: two operand buffers and the pair spectra of a particle
    // (4.2 + 19.6 MB at 76², 35 rings, 49 shifts, 200 references) within the
    // requested share of free memory, at most 2,048 particles
    size_t free_b = 0, total_b = 0;
    CK(cudaMemGetInfo(&free_b, &total_b));
    const double frac = (mem_request > 0.f && mem_request <= 1.f) ? mem_request : 0.9;
    const size_t budget = (size_t)((double)free_b * frac) / 2;
    const size_t per_part = 2 * split_sop_bytes(pl, 1) + split_z_bytes(pl, 1, g.R);
    size_t chunk = std::max<size_t>(1, std::min<size_t>(budget / per_part, 2048));
    chunk = std::min<size_t>(chunk, g.P);
    const size_t sop_bytes = split_sop_bytes(pl, (unsigned)chunk);
    if (ws.sop.ensure(2 * sop_bytes) || ws.zsp.ensure(split_z_bytes(pl, (unsigned)chunk, g.R) / sizeof(float2)) ||
        ws.err.ensure(1))
        return E_NOMEM;
    CK(cudaMemsetAsync(ws.err.p, 0, sizeof(unsigned), hi));
    if (host) {
        rc = prepare_copy_back(ws);
        if (rc)
            return rc;
    }
    unsigned prev_p0 = 0, prev_n = 0, slot = 0, c = 0;
    for (unsigned p0 = 0; p0 < g.P; p0 += (unsigned)chunk, c++) {
        const NvtxRange chunk_range("gpuisac:particle_chunk");
        const unsigned n = (unsigned)std::min<size_t>(chunk, g.P - p0);
        const unsigned buf = c & 1u;
        unsigned char* const sop = ws.sop.p + buf * sop_bytes;
        // operands of chunk c into buffer c mod 2, once the contraction of
        // chunk c - 2 has read it
        if (c >= 2)
            CK(cudaStreamWaitEvent(lo, ws.mma_done[buf], 0));
        ev = g_timer.begin(lo);
        CK(launch_polar_operands(sbjs, ws.tmpl.p, ws.tw.p, g.NR, ws.shifts_i.p, g.S, d_base, p0, n, 0,
                                 split_sbj_layout(pl, sop), lo, sbj_tx));
        g_timer.end(K_SPECTRA, ev, lo);
        CK(cudaEventRecord(ws.ops_done[buf], lo));
        CK(cudaStreamWaitEvent(hi, ws.ops_done[buf], 0));
        ev = g_timer.begin(hi);
        CK(launch_ccf_mma(pl, sop, ws.rop.p, ws.zsp.p, n, g.R, g.S, ws.err.p, hi));
        g_timer.end(K_MMA, ev, hi);
        CK(cudaEventRecord(ws.mma_done[buf], hi));
        ev = g_timer.begin(hi);
        CK(launch_zfft_peak(pl, ws.zsp.p, n, p0, g.P, g.R, g.S, ws.tw.p, ws.shifts_f.p, d_base, d_out, d_peak,
                            ws.err.p, hi));
        g_timer.end(K_ZFFT, ev, hi);
        if (host) {
            CK(cudaEventRecord(ws.chunk_done[slot], hi));
            if (prev_n) {
                rc = copy_chunk_back(g, ws, host, d_out, d_peak, prev_p0, prev_n, ws.chunk_done[slot ^ 1u]);
                if (rc)
                    return rc;
            }
        }
        prev_p0 = p0;
        prev_n = n;
        slot ^= 1u;
    }
    // every operand launch precedes a contraction on hi: hi's end is the call's end
    CK(cudaEventRecord(ws.split_exit, hi));
    CK(cudaStreamWaitEvent(st, ws.split_exit, 0));
    if (host && prev_n) {
        rc = copy_chunk_back(g, ws, host, d_out, d_peak, prev_p0, prev_n, ws.chunk_done[slot ^ 1u]);
        if (rc)
            return rc;
        CK(cudaStreamSynchronize(ws.copy_stream));
    }
    return 0;
}

// 512-sample rings (ring512.cu): FP32 contraction whatever the mode; chunks
// of particles bounded by the memory request, results copied to the host at
// the end when `host` is given
int run_alignment_l512(const Geometry& g, Workspace& ws, const StackDesc& refs, const StackDesc& sbjs,
                       const unsigned long long* ref_tx, const unsigned long long* sbj_tx, const float2* d_base,
                       float* d_out, float4* d_peak, float mem_request, cudaStream_t st, const HostOut* host)
{
    const size_t row_elems = (size_t)g.NR * kSlots512;
    if (ws.ref_sp.ensure(row_elems * std::max(g.R, 1u)))
        return E_NOMEM;
    cudaEvent_t ev = g_timer.begin(st);
    CK(launch_polar_spectra512(refs, ws.tmpl.p, ws.tw512.p, g.NR, ws.zero_shift.p, 1, nullptr, 0, g.R, 1,
                               ws.ref_sp.p, st, ref_tx));
    g_timer.end(K_SPECTRA, ev, st);
    size_t free_b = 0, total_b = 0;
    CK(cudaMemGetInfo(&free_b, &total_b));
    const double frac = (mem_request > 0.f && mem_request <= 1.f) ? mem_request : 0.9;
    const size_t budget = (size_t)((double)free_b * frac) / 2;
    const size_t per_part = row_elems * g.S * sizeof(float2);
    const size_t chunk = std::min<size_t>(std::max<size_t>(1, std::min<size_t>(budget / per_part, 2048)), g.P);
    if (ws.sbj_sp.ensure(per_part / sizeof(float2) * chunk))
        return E_NOMEM;
    for (unsigned p0 = 0; p0 < g.P; p0 += (unsigned)chunk) {
        const unsigned n = (unsigned)std::min<size_t>(chunk, g.P - p0);
        ev = g_timer.begin(st);
        CK(launch_polar_spectra512(sbjs, ws.tmpl.p, ws.tw512.p, g.NR, ws.shifts_i.p, g.S, d_base, p0, n, 0,
                                   ws.sbj_sp.p, st, sbj_tx));
        g_timer.end(K_SPECTRA, ev, st);
        ev = g_timer.begin(st);
        CK(launch_ccf_peak512(ws.sbj_sp.p, ws.ref_sp.p, ws.tw512.p, g.NR, g.S, g.R, n, p0, g.P, ws.shifts_f.p, d_base,
                              d_out, d_peak, st));
        g_timer.end(K_CCF, ev, st);
    }
    if (host) {
        CK(cudaMemcpy2DAsync(host->d, (size_t)host->d_pitch * sizeof(float), d_out, (size_t)g.P * sizeof(float),
                             (size_t)g.P * sizeof(float), g.R, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(host->peak, d_peak, (size_t)g.R * g.P * sizeof(float4), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
    }
    return 0;
}

int run_alignment(const AlignConfig* cfg, const Geometry& g, Workspace& ws, const float* d_sbj, const float* d_ref,
                  const float2* d_base, float* d_out, float4* d_peak, float mem_request, cudaStream_t st,
                  const HostOut* host = nullptr)
{
    int dev = 0;
    CK(cudaGetDevice(&dev));
    int rc = upload_geometry(g, ws, st);
    if (rc)
        return rc;
    const unsigned tex = std::max(1u, texture_image_limit(dev, g.D));
    const unsigned ref_batch = std::max(1u, std::min(g.R, 100u));
    if (ref_batch > tex) {
        set_error(E_UNSUPPORTED, "reference batch of %u images exceeds one texture (%u)", ref_batch, tex);
        return E_UNSUPPORTED;
    }
    StackDesc refs{d_ref, g.R, g.D, ref_batch, tex};
    StackDesc sbjs{d_sbj, g.P, g.D, std::max(1u, reference_sbj_batch(cfg)), tex};

    // both stacks as the reference's textures, sampled by the texture unit
    const unsigned long long *ref_tx = nullptr, *sbj_tx = nullptr;
    if (texture_unit_enabled()) {
        ref_tx = ws.ref_tex.try_build(refs, st);
        sbj_tx = ws.sbj_tex.try_build(sbjs, st);
    }
    if (g.L == (unsigned)kRingLen512)
        return run_alignment_l512(g, ws, refs, sbjs, ref_tx, sbj_tx, d_base, d_out, d_peak, mem_request, st, host);
    if (contraction_mode() == GPUISAC_CONTRACTION_BF16X3)
        return run_alignment_split(g, ws, refs, sbjs, ref_tx, sbj_tx, d_base, d_out, d_peak, mem_request, st, host);
    const size_t row_elems = (size_t)g.NR * kSlots; // float2 per (image, shift) row
    if (ws.ref_sp.ensure(row_elems * std::max(g.R, 1u)))
        return E_NOMEM;
    cudaEvent_t ev = g_timer.begin(st);
    CK(launch_polar_spectra(refs, ws.tmpl.p, ws.tw.p, g.NR, ws.zero_shift.p, 1, nullptr, 0,
                            g.R, 1, ws.ref_sp.p, st, nullptr, ref_tx));
    g_timer.end(K_SPECTRA, ev, st);

    // particle chunk: bounded by the requested share of free memory, and at
    // 8,192 particles (14 GB of spectra at 76², 35 rings, 49 shifts): larger
    // chunks gain nothing on the device, and the work space is allocated by
    // the call and freed by gpu_clear (16,384: 6 ms more per call end to end)
    size_t free_b = 0, total_b = 0;
    CK(cudaMemGetInfo(&free_b, &total_b));
    double frac = (mem_request > 0.f && mem_request <= 1.f) ? mem_request : 0.9;
    size_t budget = (size_t)((double)free_b * frac) / 2;
    size_t per_part = row_elems * g.S * sizeof(float2);
    size_t chunk = std::max<size_t>(1, std::min<size_t>(budget / per_part, 8192));
    chunk = std::min<size_t>(chunk, g.P);
    if (ws.sbj_sp.ensure(per_part / sizeof(float2) * chunk))
        return E_NOMEM;
    if (ws.err.ensure(2)) // the timeout flag and the CCF kernel's work counter
        return E_NOMEM;
    CK(cudaMemsetAsync(ws.err.p, 0, sizeof(unsigned), st));
    // a chunk's results to the host, on the copy stream after its kernels
    // (event chunk_done[slot], recorded right after the chunk's CCF launch)
    unsigned prev_p0 = 0, prev_n = 0, slot = 0;
    auto copy_back = [&](unsigned c0, unsigned cn, unsigned ev_slot) -> int {
        CK(cudaStreamWaitEvent(ws.copy_stream, ws.chunk_done[ev_slot], 0));
        CK(cudaMemcpy2DAsync(host->d + c0, (size_t)host->d_pitch * sizeof(float), d_out + c0, (size_t)g.P * sizeof(float),
                             (size_t)cn * sizeof(float), g.R, cudaMemcpyDeviceToHost, ws.copy_stream));
        CK(cudaMemcpy2DAsync(host->peak + 4 * (size_t)c0, (size_t)g.P * sizeof(float4), d_peak + c0,
                             (size_t)g.P * sizeof(float4), (size_t)cn * sizeof(float4), g.R, cudaMemcpyDeviceToHost,
                             ws.copy_stream));
        return 0;
    };
    if (host) {
        if (!ws.copy_stream)
            CK(cudaStreamCreateWithFlags(&ws.copy_stream, cudaStreamNonBlocking));
        for (int i = 0; i < 2; i++)
            if (!ws.chunk_done[i])
                CK(cudaEventCreateWithFlags(&ws.chunk_done[i], cudaEventDisableTiming));
    }
    for (unsigned p0 = 0; p0 < g.P; p0 += (unsigned)chunk) {
        unsigned n = (unsigned)std::min<size_t>(chunk, g.P - p0);
        ev = g_timer.begin(st);
        CK(launch_polar_spectra(sbjs, ws.tmpl.p, ws.tw.p, g.NR, ws.shifts_i.p, g.S, d_base, p0, n, 0, ws.sbj_sp.p,
                                st, nullptr, sbj_tx));
        g_timer.end(K_SPECTRA, ev, st);
        ev = g_timer.begin(st);
        CK(launch_ccf_peak(ws.sbj_sp.p, ws.ref_sp.p, ws.tw.p, g.NR, g.S, g.R, n, p0, g.P, ws.shifts_f.p, d_base, d_out,
                           d_peak, ws.err.p, st, kPeakMref, ws.err.p + 1));
        g_timer.end(K_CCF, ev, st);
        if (host)
            CK(cudaEventRecord(ws.chunk_done[slot], st));
        // the previous chunk's results leave while this one computes (a copy
        // to pageable memory returns when it is done, so it is issued after
        // this chunk's launches)
        if (host && prev_n) {
            int rc2 = copy_back(prev_p0, prev_n, slot ^ 1u);
            if (rc2)
                return rc2;
        }
        prev_p0 = p0;
        prev_n = n;
        slot ^= 1u;
    }
    if (host && prev_n) {
        int rc2 = copy_back(prev_p0, prev_n, slot ^ 1u);
        if (rc2)
            return rc2;
        CK(cudaStreamSynchronize(ws.copy_stream));
    }
    return 0;
}

// ---------------------------------------------------------------- global state
struct State {
    int device = -1;
    const AlignConfig* cfg = nullptr; // stored, not copied (as the reference does)
    AlignParam* params = nullptr;     // host-writable base shifts
    Geometry geo;
    Workspace ws;
    cudaStream_t stream = nullptr;
    float* d_sbj = nullptr;
    float* d_ref = nullptr;
    float* d_out = nullptr;
    float4* d_peak = nullptr;
    float2* d_base = nullptr;
} g_state;

std::mutex g_api_mu;

void free_call_buffers(State& s)
{
    if (s.d_sbj) cudaFree(s.d_sbj);
    if (s.d_ref) cudaFree(s.d_ref);
    if (s.d_out) cudaFree(s.d_out);
    if (s.d_peak) cudaFree(s.d_peak);
    if (s.d_base) cudaFree(s.d_base);
    s.d_sbj = s.d_ref = s.d_out = nullptr;
    s.d_peak = nullptr;
    s.d_base = nullptr;
}

// copy n host images (pointer list) into a device stack
int upload_images(State& s, const float** imgs, unsigned n, unsigned D, float* dst)
{
    unsigned bad = 0;
    cudaError_t e = upload_host_images(imgs, n, (size_t)D * D, dst, s.stream, &bad);
    if (e == cudaErrorInvalidValue) {
        set_error(E_ARG, "image pointer %u is NULL", bad);
        return E_ARG;
    }
    if (e != cudaSuccess) {
        set_error(E_CUDA, "image upload: %s", cudaGetErrorString(e));
        return E_CUDA;
    }
    return 0;
}

int do_multi_ref_align(State& s, const float** sbj_data, const float** ref_data, float* peak_list, float* d,
                       unsigned d_pitch, float mem_request)
{
    if (!s.cfg || s.device < 0) {
        set_error(E_STATE, "multi_ref_align called before multi_ref_align_init");
        return E_STATE;
    }
    Geometry& g = s.geo;
    const unsigned P = g.P, R = g.R, D = g.D;
    if (P == 0 || R == 0)
        return 0;
    if (!sbj_data || !ref_data || !peak_list || !d) {
        set_error(E_ARG, "NULL data or output pointer");
        return E_ARG;
    }
    if (d_pitch < P) {
        set_error(E_ARG, "isac_d_pitch %u smaller than sbj_num %u", d_pitch, P);
        return E_ARG;
    }
    CK(cudaSetDevice(s.device));
    if (!s.stream)
        CK(cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking));
    free_call_buffers(s);
    const size_t img_elems = (size_t)D * D;
    CK(cudaMalloc(&s.d_sbj, (size_t)P * img_elems * sizeof(float)));
    CK(cudaMalloc(&s.d_ref, (size_t)R * img_elems * sizeof(float)));
    CK(cudaMalloc(&s.d_out, (size_t)R * P * sizeof(float)));
    CK(cudaMalloc(&s.d_peak, (size_t)R * P * sizeof(float4)));
    CK(cudaMalloc(&s.d_base, (size_t)P * sizeof(float2)));

    int rc = upload_images(s, sbj_data, P, D, s.d_sbj);
    if (!rc)
        rc = upload_images(s, ref_data, R, D, s.d_ref);
    if (rc)
        return rc;
    std::vector<float2> base(P);
    for (unsigned i = 0; i < P; i++)
        base[i] = make_float2(s.params[i].shift_x, s.params[i].shift_y);
    CK(cudaMemcpyAsync(s.d_base, base.data(), P * sizeof(float2), cudaMemcpyHostToDevice, s.stream));

    HostOut host{d, d_pitch, peak_list};
    rc = run_alignment(s.cfg, g, s.ws, s.d_sbj, s.d_ref, s.d_base, s.d_out, s.d_peak, mem_request, s.stream, &host);
    if (rc)
        return rc;
    CK(cudaStreamSynchronize(s.stream));
    g_timer.collect();
    rc = check_device_flag(s.ws);
    if (rc)
        return rc;
    CK(cudaGetLastError());
    return 0;
}

void clear_state(State& s)
{
    if (s.device >= 0)
        cudaSetDevice(s.device);
    free_call_buffers(s);
    s.ws.release();
    if (s.stream)
        cudaStreamDestroy(s.stream);
    s.stream = nullptr;
    if (s.params)
        std::free(s.params);
    s.params = nullptr;
    s.cfg = nullptr;
    s.geo = Geometry();
    // the device choice persists like the reference's CUDA_DEVICE_ID
}

} // namespace

namespace gpuisac {

void contraction_force(int mode) { t_contraction_forced = mode; }

int host_geometry(const AlignConfig* cfg, HostGeometry& out)
{
    Geometry g;
    int rc = validate(cfg, g, false);
    if (rc)
        return rc;
    out.P = g.P;
    out.R = g.R;
    out.D = g.D;
    out.NR = g.NR;
    out.S = g.S;
    out.shifts_f = g.shifts_f;
    out.shifts_i = g.shifts_i;
    out.tmpl = g.tmpl;
    out.tw = twiddles();
    out.sbj_batch = std::max(1u, reference_sbj_batch(cfg));
    return 0;
}

unsigned reference_batch(const AlignConfig* cfg) { return std::max(1u, reference_sbj_batch(cfg)); }

unsigned texture_images(int dev, unsigned dim) { return std::max(1u, texture_image_limit(dev, std::max(dim, 1u))); }

void record_error(int code, const char* msg) { set_error(code, "%s", msg); }

std::vector<float2> shift_grid_of(float rx, float ry, float step) { return shift_grid(rx, ry, step); }

bool take_injected_alloc_failure()
{
    unsigned k = g_fail_allocs.load();
    while (k && !g_fail_allocs.compare_exchange_weak(k, k - 1)) {
    }
    return k != 0;
}

} // namespace gpuisac

// ====================================================================== C-ABI
extern "C" {

int gpuisac_last_error(char* buf, size_t n)
{
    std::lock_guard<std::mutex> lk(g_err_mu);
    if (buf && n) {
        std::strncpy(buf, g_err_msg.c_str(), n - 1);
        buf[n - 1] = 0;
    }
    return g_err_code;
}

void gpuisac_clear_error(void)
{
    std::lock_guard<std::mutex> lk(g_err_mu);
    g_err_code = 0;
    g_err_msg.clear();
}

const char* gpuisac_version(void) { return "gpuisac-gb300 0.1.0"; }

AlignParam* multi_ref_align_init(const AlignConfig* aln_cfg, unsigned int cuda_device_id)
{
    std::lock_guard<std::mutex> lk(g_api_mu);
    State& s = g_state;
    if (s.device >= 0 && s.device != (int)cuda_device_id) {
        set_error(E_STATE, "process already bound to device %d (asked for %u)", s.device, cuda_device_id);
        return nullptr;
    }
    Geometry geo;
    if (validate(aln_cfg, geo, true, true))
        return nullptr;
    cudaError_t e = cudaSetDevice((int)cuda_device_id);
    if (e != cudaSuccess) {
        set_error(E_CUDA, "cudaSetDevice(%u): %s", cuda_device_id, cudaGetErrorString(e));
        return nullptr;
    }
    clear_state(s);
    s.device = (int)cuda_device_id;
    s.cfg = aln_cfg;
    s.geo = geo;
    s.params = (AlignParam*)std::calloc(std::max(aln_cfg->sbj_num, 1u), sizeof(AlignParam));
    if (!s.params) {
        set_error(E_NOMEM, "AlignParam[%u] allocation failed", aln_cfg->sbj_num);
        return nullptr;
    }
    return s.params;
}

void multi_ref_align(const float** sbj_data, const float** ref_data, float* isac_peak_list, float* isac_d,
                     unsigned int isac_d_pitch, float cuda_mem_request)
{
    const NvtxRange range("gpuisac:multi_ref_align");
    std::lock_guard<std::mutex> lk(g_api_mu);
    State& s = g_state;
    // the configuration may have been edited between init and this call
    if (s.cfg) {
        Geometry geo;
        if (validate(s.cfg, geo, true, true))
            return;
        s.geo.P = geo.P;
        s.geo.R = geo.R;
        if (geo.D != s.geo.D || geo.NR != s.geo.NR || geo.L != s.geo.L)
            s.geo = geo;
    }
    do_multi_ref_align(s, sbj_data, ref_data, isac_peak_list, isac_d, isac_d_pitch, cuda_mem_request);
}

void gpu_clear(void)
{
    {
        std::lock_guard<std::mutex> lk(g_api_mu);
        clear_state(g_state);
    }
    gpuisac::prealign_clear();
    gpuisac::multigroup_clear();
    gpuisac::assign_clear();
    gpuisac::averages_clear();
    gpuisac::release_upload_staging();
}

void reset_shifts(float shift_range, float shift_step)
{
    // the pre-alignment and multigroup sessions, if open, take the new grid too
    const int pre = gpuisac::prealign_reset_shifts(shift_range, shift_step);
    const int mg = gpuisac::multigroup_reset_shifts(shift_range, shift_step);
    std::lock_guard<std::mutex> lk(g_api_mu);
    State& s = g_state;
    if (!s.cfg) {
        if (pre < 0 && mg < 0)
            set_error(E_STATE, "reset_shifts called before an init");
        return;
    }
    std::vector<float2> sf = shift_grid(shift_range, shift_range, shift_step);
    if (sf.size() != s.geo.shifts_f.size()) {
        set_error(E_ARG, "reset_shifts: grid size %zu differs from %zu", sf.size(), s.geo.shifts_f.size());
        return;
    }
    s.geo.shifts_f = sf;
    for (size_t i = 0; i < sf.size(); i++)
        s.geo.shifts_i[i] = make_int2((int)sf[i].x, (int)sf[i].y);
}

void print_gpu_info(unsigned int device_idx)
{
    int driver = 0, runtime = 0;
    cudaDriverGetVersion(&driver);
    cudaRuntimeGetVersion(&runtime);
    cudaDeviceProp p;
    cudaError_t e = cudaGetDeviceProperties(&p, (int)device_idx);
    if (e != cudaSuccess) {
        set_error(E_CUDA, "cudaGetDeviceProperties(%u): %s", device_idx, cudaGetErrorString(e));
        return;
    }
    printf("CUDA driver  version: %d.%d\n", driver / 1000, driver % 100 / 10);
    printf("CUDA runtime version: %d.%d\n", runtime / 1000, runtime % 100 / 10);
    printf("CUDA device[%u] info for %s:\n", device_idx, p.name);
    printf("Compute capability: %d.%d\n", p.major, p.minor);
    printf("No. of multiprocessors: %d\n", p.multiProcessorCount);
    printf("Total global memory: %.3f GB\n", (double)p.totalGlobalMem / (1024.0 * 1024 * 1024));
    printf("Shared memory per block (opt-in): %zu bytes\n", p.sharedMemPerBlockOptin);
    printf("Shared memory per multiprocessor: %zu bytes\n", p.sharedMemPerMultiprocessor);
    printf("L2 cache: %d bytes\n", p.l2CacheSize);
    printf("Max. 2D linear texture: %d x %d\n", p.maxTexture2DLinear[0], p.maxTexture2DLinear[1]);
    fflush(stdout);
}

int get_texture_limit(unsigned int img_dim)
{
    if (img_dim == 0) {
        set_error(E_ARG, "get_texture_limit: img_dim is 0");
        return 0;
    }
    int dev = 0;
    cudaGetDevice(&dev);
    return (int)texture_image_limit(dev, img_dim);
}

int gpuisac_shift_count(const AlignConfig* cfg)
{
    Geometry g;
    if (validate(cfg, g, false))
        return -1;
    return (int)g.S;
}

int gpuisac_multi_ref_align_device(const AlignConfig* cfg, const float* sbj, const float* ref,
                                   const float* base_shift, float* d_out, float* peak_out, void* stream)
{
    const NvtxRange range("gpuisac:multi_ref_align_device");
    Geometry g;
    int rc = validate(cfg, g, false, true);
    if (rc)
        return rc;
    if (!sbj || !ref || !d_out || !peak_out) {
        set_error(E_ARG, "NULL device pointer");
        return E_ARG;
    }
    if (g.P == 0 || g.R == 0)
        return 0;
    static Workspace ws; // persistent across calls; guarded by g_api_mu
    std::lock_guard<std::mutex> lk(g_api_mu);
    cudaStream_t st = (cudaStream_t)stream;
    rc = run_alignment(cfg, g, ws, sbj, ref, reinterpret_cast<const float2*>(base_shift), d_out,
                       reinterpret_cast<float4*>(peak_out), 0.9f, st);
    if (rc)
        return rc;
    CK(cudaStreamSynchronize(st));
    g_timer.collect();
    rc = check_device_flag(ws);
    if (rc)
        return rc;
    CK(cudaGetLastError());
    return 0;
}

int gpuisac_spectra_device_layout(const AlignConfig* cfg, const float* imgs, unsigned int n_img, int is_ref,
                                  const float* base_shift, unsigned int batch, unsigned int tex, float* out,
                                  void* stream)
{
    Geometry g;
    int rc = validate(cfg, g, false);
    if (rc)
        return rc;
    if (!imgs || !out || batch == 0 || tex == 0) {
        set_error(E_ARG, "NULL device pointer or empty layout");
        return E_ARG;
    }
    static Workspace ws;
    std::lock_guard<std::mutex> lk(g_api_mu);
    cudaStream_t st = (cudaStream_t)stream;
    rc = upload_geometry(g, ws, st);
    if (rc)
        return rc;
    StackDesc sd{imgs, n_img, g.D, std::min(batch, std::max(n_img, 1u)), tex};
    const unsigned long long* tx = nullptr;
    if (texture_unit_enabled() && n_img > 0)
        tx = ws.sbj_tex.try_build(sd, st);
    CK(launch_polar_spectra(sd, ws.tmpl.p, ws.tw.p, g.NR, is_ref ? ws.zero_shift.p : ws.shifts_i.p, is_ref ? 1 : g.S,
                            reinterpret_cast<const float2*>(base_shift), 0, n_img, is_ref,
                            reinterpret_cast<float2*>(out), st, nullptr, tx));
    CK(cudaStreamSynchronize(st));
    return 0;
}

int gpuisac_spectra_device(const AlignConfig* cfg, const float* imgs, unsigned int n_img, int is_ref,
                           const float* base_shift, float* out, void* stream)
{
    if (!cfg) {
        set_error(E_ARG, "AlignConfig is NULL");
        return E_ARG;
    }
    int dev = 0;
    CK(cudaGetDevice(&dev));
    const unsigned tex = std::max(1u, texture_image_limit(dev, std::max(cfg->img_dim, 1u)));
    const unsigned batch = is_ref ? std::max(1u, std::min(n_img, 100u)) : std::max(1u, reference_sbj_batch(cfg));
    return gpuisac_spectra_device_layout(cfg, imgs, n_img, is_ref, base_shift, batch, tex, out, stream);
}

int gpuisac_ccf_peak_device(const AlignConfig* cfg, const float* sbj_spectra, const float* ref_spectra,
                            const float* base_shift, unsigned int n_part, unsigned int p_global0, float* d_out,
                            float* peak_out, void* stream)
{
    Geometry g;
    int rc = validate(cfg, g, false);
    if (rc)
        return rc;
    if (!sbj_spectra || !ref_spectra || !d_out || !peak_out) {
        set_error(E_ARG, "NULL device pointer");
        return E_ARG;
    }
    if ((size_t)p_global0 + n_part > g.P) {
        set_error(E_ARG, "particles %u..%u outside sbj_num %u", p_global0, p_global0 + n_part, g.P);
        return E_ARG;
    }
    static Workspace ws;
    std::lock_guard<std::mutex> lk(g_api_mu);
    cudaStream_t st = (cudaStream_t)stream;
    rc = upload_geometry(g, ws, st);
    if (rc)
        return rc;
    if (ws.err.ensure(1))
        return E_NOMEM;
    rc = check_device_flag(ws); // a previous asynchronous call's timeout, if any
    CK(cudaMemsetAsync(ws.err.p, 0, sizeof(unsigned), st));
    if (rc)
        return rc;
    CK(launch_ccf_peak(reinterpret_cast<const float2*>(sbj_spectra), reinterpret_cast<const float2*>(ref_spectra),
                       ws.tw.p, g.NR, g.S, g.R, n_part, p_global0, g.P, ws.shifts_f.p,
                       reinterpret_cast<const float2*>(base_shift), d_out, reinterpret_cast<float4*>(peak_out),
                       ws.err.p, st));
    return 0;
}

unsigned long long gpuisac_launch_count(void) { return g_kernel_launches.load(); }

void gpuisac_test_fail_alloc(unsigned int n) { g_fail_allocs.store(n); }

int gpuisac_checked_failures(unsigned long long* first)
{
#ifdef GPUISAC_CHECKED
    void (*readers[])(unsigned&, unsigned long long&) = {checked_read_spectra, checked_read_split, checked_read_ccf,
                                                         checked_read_ring512, checked_read_averages};
    unsigned total = 0;
    unsigned long long f = 0;
    for (auto rd : readers) {
        unsigned c = 0;
        unsigned long long fi = 0;
        rd(c, fi);
        if (c && !total)
            f = fi;
        total += c;
    }
    if (first)
        *first = f;
    return (int)total;
#else
    if (first)
        *first = 0;
    return -1;
#endif
}

int gpuisac_set_contraction(int mode)
{
    if (mode != GPUISAC_CONTRACTION_FP32 && mode != GPUISAC_CONTRACTION_BF16X3) {
        set_error(E_ARG, "unknown contraction mode %d", mode);
        return -1;
    }
    std::lock_guard<std::mutex> lk(g_api_mu);
    const int forced = t_contraction_forced;
    t_contraction_forced = -1;
    const int prev = contraction_mode();
    t_contraction_forced = forced;
    g_contraction.store(mode);
    return prev;
}

int gpuisac_get_contraction(void)
{
    const int forced = t_contraction_forced;
    t_contraction_forced = -1;
    const int m = contraction_mode();
    t_contraction_forced = forced;
    return m;
}

int gpuisac_split_plan(unsigned int ring_num, unsigned int n_shift, unsigned int n_ref, unsigned int* fields,
                       unsigned int n_fields)
{
    SplitPlan p;
    if (!split_plan(ring_num, n_shift, n_ref, p)) {
        set_error(E_UNSUPPORTED, "no tensor-core tile plan for %u rings, %u shifts, %u references", ring_num, n_shift,
                  n_ref);
        return E_UNSUPPORTED;
    }
    const unsigned v[10] = {p.n_blocks, p.block, p.zw, p.kg, p.rga, p.rblock, p.n_rtiles, p.n_cols, p.n_stages,
                            p.fft_groups};
    for (unsigned i = 0; fields && i < n_fields && i < 10; i++)
        fields[i] = v[i];
    return 0;
}

void gpuisac_profile(int on)
{
    std::lock_guard<std::mutex> lk(g_api_mu);
    g_timer.on = on != 0;
    for (int i = 0; i < 4; i++) {
        g_timer.launches[i] = 0;
        g_timer.ms[i] = 0.0;
    }
}

int gpuisac_kernel_time(const char* kernel, unsigned long long* launches, double* total_ms)
{
    std::lock_guard<std::mutex> lk(g_api_mu);
    int k = -1;
    if (kernel && std::strcmp(kernel, "polar_spectra") == 0)
        k = K_SPECTRA;
    else if (kernel && std::strcmp(kernel, "ccf_peak") == 0)
        k = K_CCF;
    else if (kernel && std::strcmp(kernel, "ccf_mma") == 0)
        k = K_MMA;
    else if (kernel && std::strcmp(kernel, "zfft_peak") == 0)
        k = K_ZFFT;
    if (k < 0) {
        set_error(E_ARG, "unknown kernel name '%s'", kernel ? kernel : "(null)");
        return E_ARG;
    }
    if (launches)
        *launches = g_timer.launches[k];
    if (total_ms)
        *total_ms = g_timer.ms[k];
    return 0;
}

} // extern "C"
