// prealign.cu -- the pre-alignment path: every particle of a large stack
// against one reference (the running global average), over a shift grid
// that the caller narrows between rounds, the particles' shifts accumulating
// in the AlignParam array the caller reads.
//
// Reference: pre_align_size_check / pre_align_init / pre_align_fetch /
// pre_align_run (cuda/gpu_aln_noref.cu:565-769), reset_shifts (:117-137) and
// CcfResultTable::compute_alignment_param with cu_max_idx_silly and
// interpolate_angle (:2463-2513, 1624-1665, 2535-2577).  The same kernels as
// the multi-reference search run with one reference; the peak rule is the
// pre-alignment's (first strict maximum from 0 at index 0, angle from the
// parabola in double precision) and the host applies the reference's shift
// update (accumulate, clamp to +-(img_dim - ring_num - 2) in unsigned
// arithmetic).  The subject stack is one stacked-texture batch of
// cfg->sbj_num slots: slots past the last fetch keep the images an earlier
// fetch put there, as the reference's texture memory does.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/gpu_aln_pack.h"
#include "gpuisac_kernels.h"
#include "host_geometry.h"

using namespace gpuisac;

namespace {

enum { E_ARG = 2, E_STATE = 3 };

int fail(int code, const char* msg)
{
    record_error(code, msg);
    return code;
}

template <typename T>
struct DBuf {
    T* p = nullptr;
    size_t n = 0;
    cudaError_t ensure(size_t count)
    {
        if (count <= n)
            return cudaSuccess;
        if (p)
            cudaFree(p);
        p = nullptr;
        n = 0;
        cudaError_t e = cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T));
        if (e == cudaSuccess)
            n = count;
        return e;
    }
    void release()
    {
        if (p)
            cudaFree(p);
        p = nullptr;
        n = 0;
    }
};

struct PreState {
    std::mutex mu;
    bool active = false;
    int device = -1;
    const AlignConfig* cfg = nullptr; // kept, as the reference keeps it (the caller freezes it)
    unsigned capacity = 0, num_particles = 0, fetched = 0;
    bool ref_fetched = false;
    HostGeometry geo;
    AlignParam* params = nullptr; // host memory the caller reads and writes
    DBuf<float> sbj, ref;
    DBuf<float2> tw, tmpl, shifts_f, ref_sp, sbj_sp, base;
    DBuf<int2> shifts_i, zero;
    DBuf<float> d;
    DBuf<float4> peak;
    DBuf<unsigned> err;
    TexStack sbj_tex;
    std::vector<float4> h_peak;
    std::vector<float2> h_base;
} g_pre;

void clear_pre(PreState& s)
{
    s.sbj.release();
    s.ref.release();
    s.tw.release();
    s.tmpl.release();
    s.shifts_f.release();
    s.ref_sp.release();
    s.sbj_sp.release();
    s.base.release();
    s.shifts_i.release();
    s.zero.release();
    s.d.release();
    s.peak.release();
    s.err.release();
    s.sbj_tex.release();
    std::free(s.params);
    s.params = nullptr;
    s.active = false;
    s.cfg = nullptr;
    s.capacity = s.num_particles = s.fetched = 0;
    s.ref_fetched = false;
}

#define PRE_CK(expr)                                                                              \
    do {                                                                                          \
        cudaError_t e_ = (expr);                                                                  \
        if (e_ != cudaSuccess) {                                                                  \
            char m_[320];                                                                         \
            snprintf(m_, sizeof(m_), "%s (%s) in the pre-alignment", cudaGetErrorString(e_), #expr); \
            return fail(1, m_);                                                                   \
        }                                                                                         \
    } while (0)

int upload_shift_tables(PreState& s)
{
    PRE_CK(s.shifts_f.ensure(s.geo.S));
    PRE_CK(s.shifts_i.ensure(s.geo.S));
    PRE_CK(cudaMemcpy(s.shifts_f.p, s.geo.shifts_f.data(), s.geo.S * sizeof(float2), cudaMemcpyHostToDevice));
    PRE_CK(cudaMemcpy(s.shifts_i.p, s.geo.shifts_i.data(), s.geo.S * sizeof(int2), cudaMemcpyHostToDevice));
    return 0;
}

// copy n host images into the device stack dst
int upload(PreState& s, const float** imgs, unsigned n, float* dst)
{
    unsigned bad = 0;
    cudaError_t e = upload_host_images(imgs, n, (size_t)s.geo.D * s.geo.D, dst, 0, &bad);
    if (e == cudaErrorInvalidValue)
        return fail(E_ARG, "image pointer is NULL");
    PRE_CK(e);
    return 0;
}

} // namespace

namespace gpuisac {

// reset_shifts on the pre-alignment session, if one is open: rebuilds its
// shift grid (the reference requires the same grid length).  Returns -1 when
// no session is open, else 0 or an error code.
int prealign_reset_shifts(float shift_range, float shift_step)
{
    std::lock_guard<std::mutex> lk(g_pre.mu);
    PreState& s = g_pre;
    if (!s.active)
        return -1;
    std::vector<float2> sf = shift_grid_of(shift_range, shift_range, shift_step);
    if (sf.size() != s.geo.S)
        return fail(E_ARG, "reset_shifts: the new shift grid differs in length from the current one");
    s.geo.shifts_f = sf;
    for (size_t i = 0; i < sf.size(); i++)
        s.geo.shifts_i[i] = make_int2((int)sf[i].x, (int)sf[i].y);
    cudaSetDevice(s.device);
    return upload_shift_tables(s);
}

void prealign_clear()
{
    std::lock_guard<std::mutex> lk(g_pre.mu);
    if (g_pre.active)
        cudaSetDevice(g_pre.device);
    clear_pre(g_pre);
}

} // namespace gpuisac

extern "C" {

bool pre_align_size_check(unsigned int num_particles, const AlignConfig* cfg, unsigned int cuda_device_id,
                          float request, bool verbose)
{
    HostGeometry geo;
    if (host_geometry(cfg, geo))
        return false;
    if (cudaSetDevice((int)cuda_device_id) != cudaSuccess) {
        record_error(1, "pre_align_size_check: cudaSetDevice failed");
        return false;
    }
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
        record_error(1, "pre_align_size_check: cudaMemGetInfo failed");
        return false;
    }
    const size_t img = (size_t)geo.D * geo.D * sizeof(float);
    const size_t spectra_row = (size_t)geo.NR * kSlots * sizeof(float2);
    // the subject batch's images, one reference, the spectra of a chunk of
    // particles (the run works in chunks) and the per-particle outputs
    const size_t chunk = std::min<size_t>(geo.P, 4096);
    const size_t need = (size_t)geo.P * img + img + spectra_row + chunk * geo.S * spectra_row +
                        (size_t)geo.P * (sizeof(float) + sizeof(float4) + sizeof(float2)) + (64u << 20);
    if (verbose) {
        printf("GPU[%u] SIZE CHECK (pre-alignment)\n", cuda_device_id);
        printf("  sbj images:     %zuMB\n", (size_t)geo.P * img >> 20);
        printf("  spectra chunk:  %zuMB\n", chunk * geo.S * spectra_row >> 20);
        printf("TOTAL: %zuMB of %zuMB available\n", need >> 20, free_b >> 20);
        fflush(stdout);
    }
    (void)num_particles; // the AlignParam array lives in host memory
    return (double)need < (double)free_b * (double)request;
}

AlignParam* pre_align_init(unsigned int num_particles, const AlignConfig* aln_cfg, unsigned int cuda_device_id)
{
    std::lock_guard<std::mutex> lk(g_pre.mu);
    PreState& s = g_pre;
    HostGeometry geo;
    if (host_geometry(aln_cfg, geo))
        return nullptr;
    if (geo.P == 0 || num_particles == 0) {
        fail(E_ARG, "pre_align_init: empty stack");
        return nullptr;
    }
    if (cudaSetDevice((int)cuda_device_id) != cudaSuccess) {
        fail(1, "pre_align_init: cudaSetDevice failed");
        return nullptr;
    }
    if (s.active)
        clear_pre(s);
    s.geo = geo;
    s.cfg = aln_cfg;
    s.device = (int)cuda_device_id;
    s.capacity = geo.P;
    s.num_particles = num_particles;
    // every particle starts at zero shift, angle 0, reference 0
    s.params = static_cast<AlignParam*>(std::calloc(num_particles, sizeof(AlignParam)));
    if (!s.params) {
        fail(1, "pre_align_init: AlignParam allocation failed");
        return nullptr;
    }
    const size_t img = (size_t)geo.D * geo.D;
    const int2 zero = make_int2(0, 0);
    bool ok = s.sbj.ensure((size_t)s.capacity * img) == cudaSuccess && s.ref.ensure(img) == cudaSuccess &&
              s.tw.ensure(kRingLen) == cudaSuccess && s.tmpl.ensure(geo.tmpl.size()) == cudaSuccess &&
              s.zero.ensure(1) == cudaSuccess && s.err.ensure(2) == cudaSuccess &&
              s.ref_sp.ensure((size_t)geo.NR * kSlots) == cudaSuccess;
    // slots never fetched read as zero (the reference leaves them undefined)
    ok = ok && cudaMemset(s.sbj.p, 0, (size_t)s.capacity * img * sizeof(float)) == cudaSuccess &&
         cudaMemset(s.ref.p, 0, img * sizeof(float)) == cudaSuccess &&
         cudaMemcpy(s.tw.p, geo.tw.data(), kRingLen * sizeof(float2), cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(s.tmpl.p, geo.tmpl.data(), geo.tmpl.size() * sizeof(float2), cudaMemcpyHostToDevice) ==
             cudaSuccess &&
         cudaMemcpy(s.zero.p, &zero, sizeof(int2), cudaMemcpyHostToDevice) == cudaSuccess;
    if (!ok || upload_shift_tables(s)) {
        clear_pre(s);
        fail(1, "pre_align_init: device allocation failed");
        return nullptr;
    }
    s.active = true;
    return s.params;
}

void pre_align_fetch(const float** img_data, unsigned int img_num, const char* batch_type)
{
    std::lock_guard<std::mutex> lk(g_pre.mu);
    PreState& s = g_pre;
    if (!s.active) {
        fail(E_STATE, "pre_align_fetch called before pre_align_init");
        return;
    }
    if (!img_data || !batch_type) {
        fail(E_ARG, "pre_align_fetch: NULL argument");
        return;
    }
    cudaSetDevice(s.device);
    if (std::strcmp(batch_type, "sbj_batch") == 0) {
        if (img_num > s.capacity) {
            fail(E_ARG, "pre_align_fetch: more subject images than the batch holds (cfg->sbj_num at init)");
            return;
        }
        if (upload(s, img_data, img_num, s.sbj.p) == 0)
            s.fetched = img_num;
    } else if (std::strcmp(batch_type, "ref_batch") == 0) {
        if (img_num != 1) {
            fail(E_ARG, "pre_align_fetch: the pre-alignment takes exactly one reference");
            return;
        }
        if (upload(s, img_data, 1, s.ref.p) == 0)
            s.ref_fetched = true;
    } else {
        fail(E_ARG, "pre_align_fetch: batch type must be 'sbj_batch' or 'ref_batch'");
    }
}

void pre_align_run(int start_idx, int stop_idx)
{
    const gpuisac::NvtxRange nvtx_range("gpuisac:pre_align_run");
    std::lock_guard<std::mutex> lk(g_pre.mu);
    PreState& s = g_pre;
    auto run = [&]() -> int {
        if (!s.active)
            return fail(E_STATE, "pre_align_run called before pre_align_init");
        if (!s.ref_fetched)
            return fail(E_STATE, "pre_align_run: no reference fetched");
        if (start_idx < 0 || stop_idx < start_idx || (unsigned)stop_idx > s.num_particles)
            return fail(E_ARG, "pre_align_run: particle range outside 0..num_particles");
        const unsigned n = (unsigned)(stop_idx - start_idx);
        if (n > s.capacity)
            return fail(E_ARG, "pre_align_run: range longer than the subject batch");
        if (n == 0)
            return 0;
        PRE_CK(cudaSetDevice(s.device));
        const HostGeometry& g = s.geo;
        const unsigned tex = texture_images(s.device, g.D);
        const size_t row = (size_t)g.NR * kSlots;
        cudaStream_t st = 0;
        PRE_CK(cudaMemsetAsync(s.err.p, 0, sizeof(unsigned), st));
        // the reference at zero shift (reference basis, ring weights folded in)
        StackDesc refs{s.ref.p, 1, g.D, 1, tex};
        PRE_CK(launch_polar_spectra(refs, s.tmpl.p, s.tw.p, g.NR, s.zero.p, 1, nullptr, 0, 1, 1, s.ref_sp.p, st));
        // base shifts: the particles' accumulated shifts, by stack slot
        s.h_base.resize(n);
        for (unsigned i = 0; i < n; i++)
            s.h_base[i] = make_float2(s.params[start_idx + i].shift_x, s.params[start_idx + i].shift_y);
        PRE_CK(s.base.ensure(n));
        PRE_CK(s.d.ensure(n));
        PRE_CK(s.peak.ensure(n));
        PRE_CK(cudaMemcpyAsync(s.base.p, s.h_base.data(), n * sizeof(float2), cudaMemcpyHostToDevice, st));
        size_t free_b = 0, total_b = 0;
        PRE_CK(cudaMemGetInfo(&free_b, &total_b));
        const size_t per_part = row * g.S * sizeof(float2);
        const unsigned chunk = (unsigned)std::max<size_t>(
            1, std::min<size_t>({(size_t)n, (size_t)(0.4 * (double)free_b) / per_part, (size_t)16384}));
        PRE_CK(s.sbj_sp.ensure(row * g.S * chunk));
        StackDesc sbjs{s.sbj.p, s.capacity, g.D, s.capacity, tex};
        const unsigned long long* sbj_tx = nullptr;
        if (texture_unit_enabled())
            sbj_tx = s.sbj_tex.try_build(sbjs, st);
        for (unsigned c0 = 0; c0 < n; c0 += chunk) {
            const unsigned c = std::min(chunk, n - c0);
            PRE_CK(launch_polar_spectra(sbjs, s.tmpl.p, s.tw.p, g.NR, s.shifts_i.p, g.S, s.base.p, c0, c, 0,
                                        s.sbj_sp.p, st, nullptr, sbj_tx));
            PRE_CK(launch_ccf_peak(s.sbj_sp.p, s.ref_sp.p, s.tw.p, g.NR, g.S, 1, c, c0, n, s.shifts_f.p, s.base.p,
                                   s.d.p, s.peak.p, s.err.p, st, kPeakPreAlign, s.err.p + 1));
        }
        s.h_peak.resize(n);
        PRE_CK(cudaMemcpyAsync(s.h_peak.data(), s.peak.p, n * sizeof(float4), cudaMemcpyDeviceToHost, st));
        unsigned flag = 0;
        PRE_CK(cudaMemcpyAsync(&flag, s.err.p, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
        PRE_CK(cudaStreamSynchronize(st));
        if (flag)
            return fail(1, "a kernel timed out waiting for its own asynchronous copies");
        // the reference's update: accumulated shift clamped to
        // +-(img_dim - ring_num - 2), computed in unsigned arithmetic
        const float limit = (float)(s.cfg->img_dim - s.cfg->ring_num - 2u);
        for (unsigned i = 0; i < n; i++) {
            AlignParam& a = s.params[start_idx + i];
            const float4 pk = s.h_peak[i];
            a.ref_id = 0;
            a.mirror = pk.w != 0.f;
            a.shift_x = std::min(std::max(pk.y, -limit), limit);
            a.shift_y = std::min(std::max(pk.z, -limit), limit);
            a.angle = pk.x;
        }
        return 0;
    };
    run();
}

} // extern "C"
