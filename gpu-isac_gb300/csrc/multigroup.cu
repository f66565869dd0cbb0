// multigroup.cu -- the multigroup alignment of ISAC's stability test: every
// particle against the average of its own class, the particles' shifts
// accumulating over the iterations, then each class re-averaged from its
// particles transformed by their new parameters; between iterations the
// caller may low-pass the averages with the hyperbolic-tangent filter.
//
// Reference: ref_free_alignment_2D_init / _size_check / ref_free_alignment_2D
// / ref_free_alignment_2D_filter_references (cuda/gpu_aln_noref.cu:782-1005);
// the one-reference CCF cu_ccf_mult (:1356-1481); cu_transform_batch
// (:1539-1590); cu_average_batch (:1592-1622); cu_apply_tanl_filter_to_tex
// (:1007-1037) inside BatchHandler::apply_tangent_filter (:2203-2266); the
// parameter update CcfResultTable::compute_alignment_param with
// cu_max_idx_silly (:2463-2513, 1624-1665); the caller
// multigroup_refinement_gpu (bin/sp_isac_applications.py:4552-4650).
//
// * Alignment: the spectra and CCF kernels of the multi-reference search with
//   one reference per class -- a group table with one entry per (class, chunk
//   of particles) segment -- and the pre-alignment's peak rule (first strict
//   maximum from 0 at index 0, angle from the parabola in double precision);
//   the host applies the reference's update (mirror, accumulated shift clamped
//   to +-(img_dim - ring_num - 2) in unsigned arithmetic, angle).
// * Averages: the reference transforms every particle into a buffer, then sums
//   each class's buffers.  Here thread (class, pixel) samples that pixel of
//   every member's transformed image straight from the particle stack (the
//   texture unit's bilinear rule, clamped stacked-texture edges) and sums them
//   in member order, as the reference's averaging loop does: the same sums
//   without the intermediate images.
// * Filter: a 2D DFT per average (rows real-to-half-complex, columns, the
//   reference's filter factor, inverse columns, inverse rows) in FP32 with
//   twiddles computed in double, one CTA per average.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/gpu_aln_pack.h"
#include "gpuisac_kernels.h"
#include "host_geometry.h"

namespace gpuisac {
namespace {

enum { E_ARG = 2, E_STATE = 3 };

// Per-particle transform of the averaging step: cos and sin of the angle,
// accumulated shift, mirror flag.
struct MgXform {
    float c, s, sx, sy;
    int mirror;
};

// (class k, pixel q): sum over the class's members, in index order, of pixel q
// of the member's image transformed as cu_transform_batch does (mirror
// x -> D - x, rotation about (D/2, D/2), shift, +0.5 texel centre; each step
// rounded to float, the +0.5 added in double), then divided by the member
// count in float.
__global__ void __launch_bounds__(256)
mg_average_kernel(StackDesc st, const MgXform* __restrict__ xf, const unsigned* __restrict__ cid_idx,
                  float* __restrict__ avg, const unsigned long long* __restrict__ tex_objs)
{
    const unsigned k = blockIdx.y;
    const unsigned D = st.dim;
    const unsigned q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= D * D)
        return;
    const unsigned x = q % D, y = q / D;
    const float ctr = (float)(D / 2u);
    const unsigned i0 = cid_idx[k], i1 = cid_idx[k + 1];
    float sum = 0.0f;
    for (unsigned i = i0; i < i1; i++) {
        const MgXform t = xf[i];
        const float sxp = t.mirror ? (float)(D - x) : (float)x;
        const float x0 = __fsub_rn(sxp, ctr), y0 = __fsub_rn((float)y, ctr);
        float xr = __fsub_rn(__fmul_rn(x0, t.c), __fmul_rn(y0, t.s));
        float yr = __fadd_rn(__fmul_rn(x0, t.s), __fmul_rn(y0, t.c));
        xr = __fadd_rn(xr, ctr);
        yr = __fadd_rn(yr, ctr);
        float xs = half_up(__fadd_rn(xr, t.sx));
        float ys = half_up(__fadd_rn(yr, t.sy));
        // far-outside coordinates read the clamped edge either way; keep the
        // fixed-point conversion in range
        xs = fminf(fmaxf(xs, -1.0e6f), 1.0e6f);
        ys = fminf(fmaxf(ys, -1.0e6f), 1.0e6f);
        const TexPlacement pl = tex_place(st, i);
        const float yt = __fadd_rn((float)(pl.local * D), ys);
        // the texture unit when the stack has textures, else its emulation
        const float v = tex_objs ? tex2D<float>((cudaTextureObject_t)__ldg(tex_objs + pl.tex_id), xs, yt)
                                 : tex_sample(st, pl, xs, yt);
        sum = __fadd_rn(sum, v);
    }
    avg[(size_t)k * D * D + q] = __fdiv_rn(sum, (float)(i1 - i0));
}

// The hyperbolic-tangent low-pass of one average, as the reference applies it
// on the half spectrum: factor 0.5 (tanh(c (d + fc)) - tanh(c (d - fc))) with
// c = pi / (2 falloff fc), d = |(x, y)|, x = kx / (D/2 + 1) / 2 and
// y = min(ky, D - ky) / (D/2) / 2.  The reference's host rescaling reaches
// only the first image of the texture: average 0 comes out as filtered / N,
// the others as N x filtered (N = D^2).  Both scales vanish in the polar
// normalisation that follows; they are kept so that the averages match.
// scratch: two [D][D/2+1] complex buffers per average; tw[j] = exp(-2 pi i j / D).
__global__ void __launch_bounds__(256)
mg_filter_kernel(float* __restrict__ avg, unsigned D, float cutoff, float falloff, float2* __restrict__ scratch,
                 const float2* __restrict__ tw)
{
    const unsigned k = blockIdx.x, H = D / 2u + 1u;
    float* img = avg + (size_t)k * D * D;
    float2* F = scratch + (size_t)k * 2u * D * H;
    float2* G = F + (size_t)D * H;
    const unsigned tid = threadIdx.x, nt = blockDim.x;

    // rows: F[y][kx] = sum_x img[y][x] exp(-2 pi i kx x / D)
    for (unsigned e = tid; e < D * H; e += nt) {
        const unsigned yy = e / H, kx = e % H;
        const float* row = img + (size_t)yy * D;
        float re = 0.f, im = 0.f;
        unsigned j = 0;
        for (unsigned xx = 0; xx < D; xx++) {
            const float v = row[xx];
            const float2 w = tw[j];
            re = fmaf(v, w.x, re);
            im = fmaf(v, w.y, im);
            j += kx;
            if (j >= D)
                j -= D;
        }
        F[e] = make_float2(re, im);
    }
    __syncthreads();

    // columns and the filter: G[ky][kx] = h(kx, ky) sum_y F[y][kx] exp(-2 pi i ky y / D)
    const float c = 3.141592653589793f / (2.0f * falloff * cutoff);
    const float half = (float)D / 2.0f;
    for (unsigned e = tid; e < D * H; e += nt) {
        const unsigned ky = e / H, kx = e % H;
        float re = 0.f, im = 0.f;
        unsigned j = 0;
        for (unsigned yy = 0; yy < D; yy++) {
            const float2 v = F[yy * H + kx];
            const float2 w = tw[j];
            re = fmaf(v.x, w.x, fmaf(-v.y, w.y, re));
            im = fmaf(v.x, w.y, fmaf(v.y, w.x, im));
            j += ky;
            if (j >= D)
                j -= D;
        }
        const float fx = __fmul_rn(__fdiv_rn((float)kx, (float)H), 0.5f);
        float fy = ((float)ky < half) ? (float)ky : (float)(D - ky);
        fy = __fmul_rn(__fdiv_rn(fy, half), 0.5f);
        const float dd = __fsqrt_rn(__fadd_rn(__fmul_rn(fx, fx), __fmul_rn(fy, fy)));
        const float h = 0.5f * (tanhf(c * (dd + cutoff)) - tanhf(c * (dd - cutoff)));
        G[e] = make_float2(re * h, im * h);
    }
    __syncthreads();

    // inverse columns: F[y][kx] = sum_ky G[ky][kx] exp(+2 pi i ky y / D)
    for (unsigned e = tid; e < D * H; e += nt) {
        const unsigned yy = e / H, kx = e % H;
        float re = 0.f, im = 0.f;
        unsigned j = 0;
        for (unsigned ky = 0; ky < D; ky++) {
            const float2 v = G[ky * H + kx];
            const float2 w = tw[j]; // conj for the inverse
            re = fmaf(v.x, w.x, fmaf(v.y, w.y, re));
            im = fmaf(v.y, w.x, fmaf(-v.x, w.y, im));
            j += yy;
            if (j >= D)
                j -= D;
        }
        F[e] = make_float2(re, im);
    }
    __syncthreads();

    // inverse rows, half spectrum to real: the DC and (even D) Nyquist terms
    // once, the others twice (their conjugate partners)
    const unsigned top = (D % 2u == 0u) ? D / 2u : H; // first kx not doubled (Nyquist), or none
    const float n_pix = (float)(D * D);
    const float scale = (k == 0) ? 1.0f / n_pix : n_pix;
    for (unsigned e = tid; e < D * D; e += nt) {
        const unsigned yy = e / D, xx = e % D;
        const float2* row = F + (size_t)yy * H;
        float acc = row[0].x;
        unsigned j = 0;
        for (unsigned kx = 1; kx < H; kx++) {
            j += xx;
            if (j >= D)
                j -= D;
            const float2 w = tw[j];
            // Re(v exp(+i t)) = v.re cos t - v.im sin t, with w = (cos t, -sin t)
            const float t = fmaf(row[kx].x, w.x, row[kx].y * w.y);
            acc = fmaf(kx == top ? 1.0f : 2.0f, t, acc);
        }
        img[e] = (acc / n_pix) * scale;
    }
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

struct MgState {
    std::mutex mu;
    bool active = false;
    int device = -1;
    const AlignConfig* cfg = nullptr; // kept, as the reference keeps it
    HostGeometry geo;
    unsigned P = 0, R = 0, tex = 1, ftw_dim = 0;
    AlignParam* params = nullptr; // host memory the caller reads and writes
    std::vector<unsigned> cid_idx;
    DBuf<float> sbj, ref, d;
    DBuf<float2> tw, tmpl, shifts_f, ref_sp, sbj_sp, base, ftw, fscratch;
    DBuf<int2> shifts_i, zero;
    DBuf<float4> peak;
    TexStack sbj_tex, ref_tex; // the particles (built at init) and the averages (each iteration)
    DBuf<unsigned> err, cid;
    DBuf<MgXform> xf;
    DBuf<CcfGroup> table;
    std::vector<CcfGroup> h_table;
    std::vector<float4> h_peak;
    std::vector<float2> h_base;
    std::vector<MgXform> h_xf;
} g_mg;

void clear_mg(MgState& s)
{
    s.sbj.release();
    s.ref.release();
    s.d.release();
    s.tw.release();
    s.tmpl.release();
    s.shifts_f.release();
    s.ref_sp.release();
    s.sbj_sp.release();
    s.base.release();
    s.ftw.release();
    s.fscratch.release();
    s.shifts_i.release();
    s.zero.release();
    s.peak.release();
    s.err.release();
    s.cid.release();
    s.xf.release();
    s.table.release();
    s.sbj_tex.release();
    s.ref_tex.release();
    std::free(s.params);
    s.params = nullptr;
    s.cid_idx.clear();
    s.active = false;
    s.cfg = nullptr;
    s.P = s.R = s.ftw_dim = 0;
}

int fail(int code, const char* msg)
{
    record_error(code, msg);
    return code;
}

#define MG_CK(expr)                                                                                   \
    do {                                                                                              \
        cudaError_t e_ = (expr);                                                                      \
        if (e_ != cudaSuccess) {                                                                      \
            char m_[320];                                                                             \
            snprintf(m_, sizeof(m_), "%s (%s) in the multigroup alignment", cudaGetErrorString(e_), #expr); \
            return fail(1, m_);                                                                       \
        }                                                                                             \
    } while (0)

int upload_shift_tables(MgState& s)
{
    MG_CK(s.shifts_f.ensure(s.geo.S));
    MG_CK(s.shifts_i.ensure(s.geo.S));
    MG_CK(cudaMemcpy(s.shifts_f.p, s.geo.shifts_f.data(), s.geo.S * sizeof(float2), cudaMemcpyHostToDevice));
    MG_CK(cudaMemcpy(s.shifts_i.p, s.geo.shifts_i.data(), s.geo.S * sizeof(int2), cudaMemcpyHostToDevice));
    return 0;
}

// copy n host images (pointers) into the device stack dst
int upload_images(const float** imgs, unsigned n, unsigned D, float* dst)
{
    unsigned bad = 0;
    cudaError_t e = upload_host_images(imgs, n, (size_t)D * D, dst, 0, &bad);
    if (e == cudaErrorInvalidValue)
        return fail(E_ARG, "image pointer is NULL");
    MG_CK(e);
    return 0;
}

// one iteration: alignment of every particle to its class average, the
// parameter update, the new averages
int run_iteration(MgState& s)
{
    const HostGeometry& g = s.geo;
    const unsigned P = s.P, R = s.R, D = g.D, NR = g.NR, S = g.S;
    const size_t row = (size_t)NR * kSlots;
    cudaStream_t st = 0;
    MG_CK(cudaSetDevice(s.device));
    MG_CK(cudaMemsetAsync(s.err.p, 0, sizeof(unsigned), st));

    // the class averages at zero shift (reference basis, ring weights folded
    // in), read as one texture of R images
    StackDesc refs{s.ref.p, R, D, R, s.tex};
    StackDesc sbjs{s.sbj.p, P, D, P, s.tex};
    const bool hw = texture_unit_enabled();
    const unsigned long long* ref_tx = hw ? s.ref_tex.try_build(refs, st) : nullptr;
    const unsigned long long* sbj_tx = nullptr;
    if (hw)
        sbj_tx = s.sbj_tex.objects() ? s.sbj_tex.objects() : s.sbj_tex.try_build(sbjs, st);
    MG_CK(launch_polar_spectra(refs, s.tmpl.p, s.tw.p, NR, s.zero.p, 1, nullptr, 0, R, 1, s.ref_sp.p, st, nullptr,
                               ref_tx));

    // base shifts: the particles' accumulated shifts
    s.h_base.resize(P);
    for (unsigned i = 0; i < P; i++)
        s.h_base[i] = make_float2(s.params[i].shift_x, s.params[i].shift_y);
    MG_CK(cudaMemcpyAsync(s.base.p, s.h_base.data(), P * sizeof(float2), cudaMemcpyHostToDevice, st));

    size_t free_b = 0, total_b = 0;
    MG_CK(cudaMemGetInfo(&free_b, &total_b));
    const size_t per_part = row * S * sizeof(float2);
    const unsigned chunk = (unsigned)std::max<size_t>(
        1, std::min<size_t>({(size_t)P, (size_t)(0.4 * (double)(free_b + s.sbj_sp.n * sizeof(float2))) / per_part,
                             (size_t)16384}));
    MG_CK(s.sbj_sp.ensure(row * S * chunk));

    // group table: one entry per (class, chunk) segment, one reference each
    const CcfTile tile = ccf_tile(NR, S, true);
    const unsigned ppc = tile.ppc;
    struct ChunkWork {
        unsigned c0, c, first, n_groups, n_items;
    };
    std::vector<ChunkWork> work;
    s.h_table.clear();
    unsigned k = 0;
    for (unsigned c0 = 0; c0 < P; c0 += chunk) {
        const unsigned c1 = std::min(P, c0 + chunk);
        ChunkWork cw{c0, c1 - c0, (unsigned)s.h_table.size(), 0, 0};
        while (k < R && s.cid_idx[k + 1] <= c0)
            k++;
        for (unsigned kk = k; kk < R && s.cid_idx[kk] < c1; kk++) {
            const unsigned a = std::max(s.cid_idx[kk], c0), b = std::min(s.cid_idx[kk + 1], c1);
            if (a >= b)
                continue;
            const unsigned ck = s.cid_idx[kk];
            CcfGroup e{};
            e.sbj_sp = s.sbj_sp.p + (size_t)(a - c0) * row * S;
            e.ref_sp = s.ref_sp.p + (size_t)kk * row;
            e.base = s.base.p + ck;
            e.d_out = s.d.p + ck;
            e.peak_out = s.peak.p + ck;
            e.p_first = a - ck;
            e.n_part = b - a;
            e.n_ref = 1;
            e.p_total = s.cid_idx[kk + 1] - ck;
            e.item_begin = cw.n_items;
            e.ref_tiles = 1;
            e.ref_idx = nullptr;
            e.rule = kPeakPreAlign;
            cw.n_items += (e.n_part + ppc - 1) / ppc;
            s.h_table.push_back(e);
            cw.n_groups++;
        }
        work.push_back(cw);
    }
    MG_CK(s.table.ensure(s.h_table.size()));
    MG_CK(cudaMemcpyAsync(s.table.p, s.h_table.data(), s.h_table.size() * sizeof(CcfGroup),
                          cudaMemcpyHostToDevice, st));

    for (const ChunkWork& cw : work) {
        MG_CK(launch_polar_spectra(sbjs, s.tmpl.p, s.tw.p, NR, s.shifts_i.p, S, s.base.p, cw.c0, cw.c, 0, s.sbj_sp.p,
                                   st, nullptr, sbj_tx));
        CcfWork w{};
        w.groups = s.table.p + cw.first;
        w.n_groups = cw.n_groups;
        w.n_items = cw.n_items;
        w.ppc = ppc;
        w.max_ref = 1; // one reference (the class average) per group
        w.item_counter = s.err.p + 1; // (err holds the timeout flag and this counter)
        MG_CK(launch_ccf_peak_work(w, tile.variant, s.tw.p, NR, S, s.shifts_f.p, s.err.p, st));
    }
    s.h_peak.resize(P);
    MG_CK(cudaMemcpyAsync(s.h_peak.data(), s.peak.p, P * sizeof(float4), cudaMemcpyDeviceToHost, st));
    unsigned flag = 0;
    MG_CK(cudaMemcpyAsync(&flag, s.err.p, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    MG_CK(cudaStreamSynchronize(st));
    if (flag)
        return fail(1, "a kernel timed out waiting for its own asynchronous copies");

    // the reference's update, then the transform of the averaging step:
    // angle in radians as the reference's float DEG2RAD * angle, its cosine
    // and sine computed in double and rounded to float
    const float limit = (float)(s.cfg->img_dim - s.cfg->ring_num - 2u);
    const float deg2rad = 3.141592653589793f / 180.0f;
    s.h_xf.resize(P);
    for (unsigned i = 0; i < P; i++) {
        AlignParam& a = s.params[i];
        const float4 pk = s.h_peak[i];
        a.mirror = pk.w != 0.f;
        a.shift_x = std::min(std::max(pk.y, -limit), limit);
        a.shift_y = std::min(std::max(pk.z, -limit), limit);
        a.angle = pk.x;
        const float rad = deg2rad * a.angle;
        s.h_xf[i] = MgXform{(float)std::cos((double)rad), (float)std::sin((double)rad), a.shift_x, a.shift_y,
                            a.mirror ? 1 : 0};
    }
    MG_CK(cudaMemcpyAsync(s.xf.p, s.h_xf.data(), P * sizeof(MgXform), cudaMemcpyHostToDevice, st));
    dim3 grid((D * D + 255) / 256, R);
    mg_average_kernel<<<grid, 256, 0, st>>>(sbjs, s.xf.p, s.cid.p, s.ref.p, sbj_tx);
    g_kernel_launches.fetch_add(1, std::memory_order_relaxed);
    MG_CK(cudaGetLastError());
    MG_CK(cudaStreamSynchronize(st));
    return 0;
}

int filter_averages(MgState& s, float cutoff, float falloff)
{
    const unsigned D = s.geo.D, H = D / 2 + 1;
    MG_CK(cudaSetDevice(s.device));
    if (s.ftw_dim != D) {
        std::vector<float2> t(D);
        for (unsigned j = 0; j < D; j++) {
            const double a = 2.0 * 3.14159265358979323846 * (double)j / (double)D;
            t[j] = make_float2((float)std::cos(a), (float)-std::sin(a));
        }
        MG_CK(s.ftw.ensure(D));
        MG_CK(cudaMemcpy(s.ftw.p, t.data(), D * sizeof(float2), cudaMemcpyHostToDevice));
        s.ftw_dim = D;
    }
    MG_CK(s.fscratch.ensure((size_t)s.R * 2 * D * H));
    mg_filter_kernel<<<s.R, 256>>>(s.ref.p, D, cutoff, falloff, s.fscratch.p, s.ftw.p);
    g_kernel_launches.fetch_add(1, std::memory_order_relaxed);
    MG_CK(cudaGetLastError());
    MG_CK(cudaDeviceSynchronize());
    return 0;
}

} // namespace

int multigroup_reset_shifts(float shift_range, float shift_step)
{
    std::lock_guard<std::mutex> lk(g_mg.mu);
    MgState& s = g_mg;
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

void multigroup_clear()
{
    std::lock_guard<std::mutex> lk(g_mg.mu);
    if (g_mg.active)
        cudaSetDevice(g_mg.device);
    clear_mg(g_mg);
}

} // namespace gpuisac

using namespace gpuisac;

extern "C" {

bool ref_free_alignment_2D_size_check(const AlignConfig* cfg, unsigned int cuda_device_id, float request,
                                      bool verbose)
{
    HostGeometry geo;
    if (host_geometry(cfg, geo))
        return false;
    if (cudaSetDevice((int)cuda_device_id) != cudaSuccess) {
        record_error(1, "ref_free_alignment_2D_size_check: cudaSetDevice failed");
        return false;
    }
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
        record_error(1, "ref_free_alignment_2D_size_check: cudaMemGetInfo failed");
        return false;
    }
    const size_t img = (size_t)geo.D * geo.D * sizeof(float);
    const size_t row = (size_t)geo.NR * kSlots * sizeof(float2);
    const size_t chunk = std::min<size_t>(std::max(geo.P, 1u), 16384);
    const size_t half = (size_t)geo.D * (geo.D / 2 + 1) * sizeof(float2);
    const size_t need = (size_t)geo.P * img + (size_t)geo.R * img + (size_t)geo.R * row + chunk * geo.S * row +
                        (size_t)geo.R * 2 * half +
                        (size_t)geo.P * (sizeof(float) + sizeof(float4) + sizeof(float2) + sizeof(MgXform)) +
                        (64u << 20);
    if (verbose) {
        printf("GPU[%u] SIZE CHECK (multigroup alignment)\n", cuda_device_id);
        printf("  sbj images:     %zuMB\n", (size_t)geo.P * img >> 20);
        printf("  averages:       %zuMB\n", (size_t)geo.R * img >> 20);
        printf("  spectra chunk:  %zuMB\n", chunk * geo.S * row >> 20);
        printf("TOTAL: %zuMB of %zuMB available\n", need >> 20, free_b >> 20);
        fflush(stdout);
    }
    return (double)need < (double)free_b * (double)request;
}

AlignParam* ref_free_alignment_2D_init(const AlignConfig* aln_cfg, const float** sbj_data_list,
                                       const float** ref_data_list, const int* sbj_cid_list,
                                       unsigned int cuda_device_id)
{
    std::lock_guard<std::mutex> lk(g_mg.mu);
    MgState& s = g_mg;
    HostGeometry geo;
    if (host_geometry(aln_cfg, geo))
        return nullptr;
    if (geo.P == 0 || geo.R == 0 || !sbj_data_list || !ref_data_list || !sbj_cid_list) {
        fail(E_ARG, "ref_free_alignment_2D_init: empty stack or NULL list");
        return nullptr;
    }
    if (geo.R > 65535u || geo.R > geo.P) {
        fail(E_ARG, "ref_free_alignment_2D_init: needs 1 <= ref_num <= min(sbj_num, 65535)");
        return nullptr;
    }
    // classes are contiguous runs 0, 1, .., ref_num - 1 of the particle list
    // (the reference builds its class index from the runs, noref.cu:825-835)
    std::vector<unsigned> cid_idx(geo.R + 1, 0);
    if (sbj_cid_list[0] != 0) {
        fail(E_ARG, "ref_free_alignment_2D_init: the class list must start with class 0");
        return nullptr;
    }
    for (unsigned i = 1; i < geo.P; i++) {
        const int a = sbj_cid_list[i - 1], b = sbj_cid_list[i];
        if (b != a && b != a + 1) {
            fail(E_ARG, "ref_free_alignment_2D_init: classes must be sorted runs 0, 1, .. with none empty");
            return nullptr;
        }
        if (b == a + 1)
            cid_idx[b] = i;
    }
    if ((unsigned)sbj_cid_list[geo.P - 1] != geo.R - 1) {
        fail(E_ARG, "ref_free_alignment_2D_init: the last class must be ref_num - 1");
        return nullptr;
    }
    cid_idx[geo.R] = geo.P;
    if (cudaSetDevice((int)cuda_device_id) != cudaSuccess) {
        fail(1, "ref_free_alignment_2D_init: cudaSetDevice failed");
        return nullptr;
    }
    if (s.active)
        clear_mg(s);
    s.geo = geo;
    s.cfg = aln_cfg;
    s.device = (int)cuda_device_id;
    s.P = geo.P;
    s.R = geo.R;
    s.tex = texture_images(s.device, geo.D);
    s.cid_idx = cid_idx;
    s.params = static_cast<AlignParam*>(std::calloc(geo.P, sizeof(AlignParam)));
    if (!s.params) {
        fail(1, "ref_free_alignment_2D_init: AlignParam allocation failed");
        return nullptr;
    }
    for (unsigned i = 0; i < geo.P; i++)
        s.params[i].ref_id = sbj_cid_list[i];
    const size_t img = (size_t)geo.D * geo.D;
    const size_t row = (size_t)geo.NR * kSlots;
    const int2 zero = make_int2(0, 0);
    bool ok = s.sbj.ensure((size_t)s.P * img) == cudaSuccess && s.ref.ensure((size_t)s.R * img) == cudaSuccess &&
              s.d.ensure(s.P) == cudaSuccess && s.tw.ensure(kRingLen) == cudaSuccess &&
              s.tmpl.ensure(geo.tmpl.size()) == cudaSuccess && s.ref_sp.ensure((size_t)s.R * row) == cudaSuccess &&
              s.base.ensure(s.P) == cudaSuccess && s.zero.ensure(1) == cudaSuccess &&
              s.peak.ensure(s.P) == cudaSuccess && s.err.ensure(2) == cudaSuccess &&
              s.cid.ensure(s.R + 1) == cudaSuccess && s.xf.ensure(s.P) == cudaSuccess;
    ok = ok && cudaMemcpy(s.tw.p, geo.tw.data(), kRingLen * sizeof(float2), cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(s.tmpl.p, geo.tmpl.data(), geo.tmpl.size() * sizeof(float2), cudaMemcpyHostToDevice) ==
             cudaSuccess &&
         cudaMemcpy(s.zero.p, &zero, sizeof(int2), cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(s.cid.p, cid_idx.data(), (s.R + 1) * sizeof(unsigned), cudaMemcpyHostToDevice) == cudaSuccess;
    if (!ok || upload_shift_tables(s) || upload_images(sbj_data_list, s.P, geo.D, s.sbj.p) ||
        upload_images(ref_data_list, s.R, geo.D, s.ref.p)) {
        clear_mg(s);
        fail(1, "ref_free_alignment_2D_init: device allocation or upload failed");
        return nullptr;
    }
    s.active = true;
    return s.params;
}

void ref_free_alignment_2D(void)
{
    const gpuisac::NvtxRange nvtx_range("gpuisac:ref_free_alignment_2D");
    std::lock_guard<std::mutex> lk(g_mg.mu);
    if (!g_mg.active) {
        fail(E_STATE, "ref_free_alignment_2D called before ref_free_alignment_2D_init");
        return;
    }
    run_iteration(g_mg);
}

void ref_free_alignment_2D_filter_references(float cutoff_freq, float falloff)
{
    std::lock_guard<std::mutex> lk(g_mg.mu);
    if (!g_mg.active) {
        fail(E_STATE, "ref_free_alignment_2D_filter_references called before ref_free_alignment_2D_init");
        return;
    }
    filter_averages(g_mg, cutoff_freq, falloff);
}

int gpuisac_ref_free_averages(float* out)
{
    std::lock_guard<std::mutex> lk(g_mg.mu);
    MgState& s = g_mg;
    if (!s.active)
        return fail(E_STATE, "gpuisac_ref_free_averages called before ref_free_alignment_2D_init");
    if (!out)
        return fail(E_ARG, "gpuisac_ref_free_averages: NULL output");
    MG_CK(cudaSetDevice(s.device));
    MG_CK(cudaMemcpy(out, s.ref.p, (size_t)s.R * s.geo.D * s.geo.D * sizeof(float), cudaMemcpyDeviceToHost));
    return 0;
}

} // extern "C"
