// ring512.cu -- the multi-reference alignment with 512 samples per ring.
//
// The reference's GPU driver fixes the ring length at 256
// (bin/sp_isac2_gpu.py:113); its library takes the length from
// cfg->ring_len, and Numrinit (bin/sp_isac_alignment.py:713-747) gives a
// maximum ring length of 512 for a last ring of 41..81 (61 rings at 128^2).
// These kernels run the same semantics -- the reference's sample positions,
// texture filtering, normalisation (cuda/gpu_aln_noref.cu:1221-1354), ring
// weights (r+1) and CCF of both mirrors (:1483-1537), first-maximum scan and
// 7-point parabola (:1667-1794) -- at L = 512, in FP32 on the CUDA cores.
//
// Layouts: a spectra row (image x shift) is [ring][256 slots] float2 in the
// basis of the 256-sample kernels (slot k = 1..255 holds F[k], slot 0 holds
// (F[0], F[256]); subjects (Re+Im, Re-Im), references (r+1)(Re+Im, Re-Im)).
// A 512-point FFT is two 256-point FFTs of 16-thread groups (even and odd
// samples) and one radix-2 step.
//
// Work: spectra, one CTA per row; CCF, one CTA per (particle, reference)
// with the reference row in shared memory, the particle's shift rows read
// from L2/HBM eight shifts at a time, sixteen 256-point inverse FFTs side by
// side (two per shift), a warp per shift for the peak search.
#include <cuda_runtime.h>

#include "ccf_device.cuh"
#include "gpuisac_kernels.h"

namespace gpuisac {
namespace {

constexpr int kL = kRingLen512;  // samples per ring
constexpr int kS = kSlots512;    // spectrum slots per ring
constexpr int kPair = 544;       // float2 per ring-pair region: two rings' samples (512), or two FFT workspaces (2 x 272)
constexpr int kShiftBlock = 8;   // shifts per CCF block

// float offset of ring r's samples
__device__ __forceinline__ unsigned ring_off(unsigned r) { return (r >> 1) * 2 * kPair + (r & 1) * kL; }

__global__ void __launch_bounds__(256)
polar_spectra512_kernel(StackDesc st, const float2* __restrict__ tmpl, const float2* __restrict__ tw512,
                        unsigned ring_num, const int2* __restrict__ shift_int, unsigned n_shift,
                        const float2* __restrict__ base, unsigned img0, unsigned n_img, int is_ref,
                        float2* __restrict__ out, const unsigned long long* __restrict__ tex_objs)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float* polar = reinterpret_cast<float*>(smem_raw);
    const unsigned n_pairs = (ring_num + 1) / 2;
    float2* tw = reinterpret_cast<float2*>(polar + (size_t)n_pairs * 2 * kPair); // [512] e^(-2 pi i e / 512)
    float2* tw256 = tw + kL;                                                    // [256] e^(-2 pi i e / 256)
    double* red = reinterpret_cast<double*>(tw256 + 256);                       // 2 x 8 warps + 2

    const unsigned row = blockIdx.x;
    const unsigned img_local = row / n_shift;
    const unsigned s = row - img_local * n_shift;
    if (img_local >= n_img)
        return;
    const unsigned img = img0 + img_local;
    const int tid = threadIdx.x;
    tw[tid] = tw512[tid];
    tw[tid + 256] = tw512[tid + 256];
    tw256[tid] = tw512[2 * tid];

    // sampling positions as the 256-sample kernel computes them
    const int2 sh = shift_int[s];
    const float* bx = base ? &base[img].x : nullptr;
    const float* by = base ? &base[img].y : nullptr;
    const float cnt_x = centre_coord(st.dim, sh.x, bx);
    const float cnt_y = centre_coord(st.dim, sh.y, by);
    const TexPlacement place = tex_place(st, img);
    const float yoff = (float)(place.local * st.dim);
    const cudaTextureObject_t tobj = tex_objs ? (cudaTextureObject_t)__ldg(tex_objs + place.tex_id) : 0;

    float s1 = 0.f, s2 = 0.f;
    for (unsigned r = 0; r < ring_num; r++) {
        const float w = (float)(r + 1);
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const unsigned j = tid + 256 * h;
            const float2 o = __ldg(&tmpl[r * kL + j]);
            const float x = cnt_x + o.x;
            const float y = (yoff + cnt_y) + o.y;
            const float v = tex_objs ? tex2D<float>(tobj, x, y) : tex_sample(st, place, x, y);
            polar[ring_off(r) + j] = v;
            s1 += w * v;
            s2 += w * v * v;
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        s1 += __shfl_xor_sync(0xffffffffu, s1, off);
        s2 += __shfl_xor_sync(0xffffffffu, s2, off);
    }
    const int warp = tid >> 5, lane = tid & 31;
    if (lane == 0) {
        red[warp] = s1;
        red[8 + warp] = s2;
    }
    __syncthreads();
    if (tid == 0) {
        double a = 0.0, q = 0.0;
        for (int w = 0; w < 8; w++) {
            a += red[w];
            q += red[8 + w];
        }
        // avg = sum (r+1) A_r / (L sum (r+1)); the same for the squares
        const double nn = 0.5 * (double)ring_num * (double)(ring_num + 1) * (double)kL;
        const double avg = a / nn, msq = q / nn;
        const double sd = sqrt(fabs(msq - avg * avg));
        float* redf = reinterpret_cast<float*>(red + 16);
        redf[0] = (float)avg;
        redf[1] = (float)(1.0 / (sd + 0.0000001));
    }
    __syncthreads();
    const float avg_f = reinterpret_cast<const float*>(red + 16)[0];
    const float inv_f = reinterpret_cast<const float*>(red + 16)[1];

    // two rings per complex 512-point FFT: z = ring a + i ring b
    const int g = tid >> 4;
    const int l = tid & 15;
    const unsigned gmask = 0xffffu << (tid & 16);
    float2* out_row = out + (size_t)row * ring_num * kS;
    for (unsigned pr = g; pr < n_pairs; pr += 16) {
        const unsigned ra = 2 * pr, rb = 2 * pr + 1;
        const bool has_b = rb < ring_num;
        const float* pa = polar + pr * 2 * kPair;
        float2* ws = reinterpret_cast<float2*>(polar) + pr * kPair;
        float2 xe[16], xo[16];
#pragma unroll
        for (int m = 0; m < 16; m++) {
            const unsigned n = 2 * (l + 16 * m);
            xe[m] = make_float2((pa[n] - avg_f) * inv_f, has_b ? (pa[kL + n] - avg_f) * inv_f : 0.f);
            xo[m] = make_float2((pa[n + 1] - avg_f) * inv_f, has_b ? (pa[kL + n + 1] - avg_f) * inv_f : 0.f);
        }
        __syncwarp(gmask); // the pair's samples are read before its region turns workspace
        fft256_group<-1, false>(xe, ws, tw256, l, gmask);
        fft256_group<-1, false>(xo, ws, tw256, l, gmask);
        // Z[k] = E[k] + w^k O[k], Z[k + 256] = E[k] - w^k O[k]
#pragma unroll
        for (int k2 = 0; k2 < 16; k2++) {
            const int k = l + 16 * k2;
            const float2 e = xe[perm16(k2)], o = cmul(xo[perm16(k2)], tw[k]);
            ws[k] = cadd(e, o);
            ws[k + 256] = csub(e, o);
        }
        __syncwarp(gmask);
        const float wa = is_ref ? (float)(ra + 1) : 1.f;
        const float wb = is_ref ? (float)(rb + 1) : 1.f;
#pragma unroll 4
        for (int i = 0; i < 16; i++) {
            const int k = l + 16 * i;
            const float2 z = ws[k];
            const float2 zc = ws[(kL - k) & (kL - 1)];
            float2 fa = make_float2(0.5f * (z.x + zc.x), 0.5f * (z.y - zc.y));
            float2 fb = make_float2(0.5f * (z.y + zc.y), -0.5f * (z.x - zc.x));
            if (k == 0) { // slot 0 carries (F[0], F[256]); both are real
                const float2 zn = ws[kS];
                fa = make_float2(z.x, zn.x);
                fb = make_float2(z.y, zn.y);
            }
            const size_t n_out = (size_t)n_img * n_shift * ring_num * kS;
            const size_t at = (size_t)row * ring_num * kS + ra * kS + k;
            if (GPUISAC_IN_BOUNDS(kChkR512Out, at, n_out))
                out_row[ra * kS + k] = make_float2(wa * (fa.x + fa.y), wa * (fa.x - fa.y));
            if (has_b && GPUISAC_IN_BOUNDS(kChkR512Out, at + kS, n_out))
                out_row[rb * kS + k] = make_float2(wb * (fb.x + fb.y), wb * (fb.x - fb.y));
        }
        __syncwarp(gmask);
    }
}

// Z[k] and Z[512-k] of one pair from the four ring sums at slot k
__device__ __forceinline__ void write_z512(float2* zp, int k, float a1, float a2, float a3, float a4)
{
    if (k == 0) {
        const float p1 = 0.25f * (a1 + a2 + a3 + a4);
        const float p2 = 0.25f * (a1 - a2 + a3 - a4);
        zp[0] = make_float2(p1, p1);
        zp[kS] = make_float2(p2, p2);
    } else {
        zp[k] = make_float2(a1, a2);
        zp[kL - k] = make_float2(a3, a4);
    }
}

__global__ void __launch_bounds__(256)
ccf_peak512_kernel(const float2* __restrict__ sbj_sp, const float2* __restrict__ ref_sp,
                   const float2* __restrict__ tw512, unsigned ring_num, unsigned n_shift, unsigned n_ref,
                   unsigned n_part, unsigned p_first, unsigned p_total, const float2* __restrict__ shifts_f,
                   const float2* __restrict__ base, float* __restrict__ d_out, float4* __restrict__ peak_out)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2* refs = reinterpret_cast<float2*>(smem_raw);           // [ring_num][256]
    float2* zb = refs + (size_t)ring_num * kS;                    // [8][kPair]: Z, then FFT workspaces, then c
    float2* tw256 = zb + kShiftBlock * kPair;                     // [256] e^(-2 pi i e / 256)
    float2* twc = tw256 + 256;                                    // [256] e^(+2 pi i k / 512)
    PeakSlot* slots = reinterpret_cast<PeakSlot*>(twc + 256);     // [8]

    const unsigned item = blockIdx.x;
    const unsigned p = item / n_ref, q = item - p * n_ref;
    if (p >= n_part)
        return;
    const int tid = threadIdx.x;
    const float2* rrow = ref_sp + (size_t)q * ring_num * kS;
    for (unsigned i = tid; i < ring_num * kS; i += 256)
        refs[i] = rrow[i];
    tw256[tid] = tw512[2 * tid];
    const float2 t = tw512[tid];
    twc[tid] = make_float2(t.x, -t.y);
    __syncthreads();

    const int warp = tid >> 5, lane = tid & 31;
    const int gi = tid >> 4, l = tid & 15;
    const unsigned gmask = 0xffffu << (tid & 16);
    const int gsh = gi >> 1, half = gi & 1;
    // running best of the shifts this warp searches (lanes 0..6 keep the 7
    // samples around it)
    float bv = -3.40282e+038f, nb = 0.f;
    unsigned bh = 0, bt = 0;
    const float2* sp = sbj_sp + (size_t)p * n_shift * ring_num * kS;
    for (unsigned s0 = 0; s0 < n_shift; s0 += kShiftBlock) {
        const unsigned ns = min((unsigned)kShiftBlock, n_shift - s0);
        // contraction: thread tid is slot k of every shift of the block
        for (unsigned g = 0; g < ns; g++) {
            const float2* row = sp + (size_t)(s0 + g) * ring_num * kS + tid;
            float a1 = 0.f, a2 = 0.f, a3 = 0.f, a4 = 0.f;
#pragma unroll 4
            const size_t row_at = ((size_t)p * n_shift + s0 + g) * ring_num * kS + tid;
            for (unsigned r = 0; r < ring_num; r++) {
                const float2 sv = GPUISAC_IN_BOUNDS(kChkR512Row, row_at + (size_t)r * kS,
                                                    (size_t)n_part * n_shift * ring_num * kS)
                                      ? __ldg(row + (size_t)r * kS)
                                      : make_float2(0.f, 0.f);
                const float2 rv = refs[r * kS + tid];
                a1 = fmaf(rv.x, sv.x, a1);
                a2 = fmaf(rv.x, sv.y, a2);
                a3 = fmaf(rv.y, sv.y, a3);
                a4 = fmaf(rv.y, sv.x, a4);
            }
            write_z512(zb + g * kPair, tid, a1, a2, a3, a4);
        }
        __syncthreads();
        // inverse FFT, two groups per shift: even outputs from Z[k] + Z[k+256],
        // odd outputs from (Z[k] - Z[k+256]) e^(2 pi i k / 512)
        float2 x[16];
        if ((unsigned)gsh < ns) {
            const float2* Z = zb + gsh * kPair;
#pragma unroll
            for (int m = 0; m < 16; m++) {
                const int k = l + 16 * m;
                const float2 z0 = Z[k], z1 = Z[k + 256];
                x[m] = half ? cmul(csub(z0, z1), twc[k]) : cadd(z0, z1);
            }
        }
        __syncthreads(); // every group holds its inputs: the Z regions turn workspace
        if ((unsigned)gsh < ns)
            fft256_group<+1, false>(x, zb + gsh * kPair + half * 272, tw256, l, gmask);
        __syncthreads(); // workspace reads done: the regions take the outputs
        if ((unsigned)gsh < ns) {
            float2* c = zb + gsh * kPair; // c[tau] = (normal, mirrored) correlation
#pragma unroll
            for (int k2 = 0; k2 < 16; k2++)
                c[2 * (l + 16 * k2) + half] = x[perm16(k2)];
        }
        __syncthreads();
        // peak search: warp w takes shift s0 + w, first maximum in the
        // reference's order (normal before mirrored, shift, then angle)
        if ((unsigned)warp < ns) {
            const float2* c = zb + warp * kPair;
            const unsigned s = s0 + warp;
#pragma unroll
            for (int mir = 0; mir < 2; mir++) {
                float v = mir ? c[lane].y : c[lane].x;
                unsigned ti = lane;
#pragma unroll
                for (int j = 1; j < 16; j++) {
                    const unsigned tau = lane + 32 * j;
                    const float cv = mir ? c[tau].y : c[tau].x;
                    if (cv > v) {
                        v = cv;
                        ti = tau;
                    }
                }
#pragma unroll
                for (int off = 16; off > 0; off >>= 1) {
                    const float ov = __shfl_xor_sync(0xffffffffu, v, off);
                    const unsigned ot = __shfl_xor_sync(0xffffffffu, ti, off);
                    if (ov > v || (ov == v && ot < ti)) {
                        v = ov;
                        ti = ot;
                    }
                }
                const unsigned hc = mir ? n_shift + s : s;
                if (better(v, hc, ti, bv, bh, bt)) {
                    bv = v;
                    bh = hc;
                    bt = ti;
                    if (lane < 7) {
                        const float2 cn = c[(ti + (unsigned)lane - 3u) & (kL - 1)];
                        nb = mir ? cn.y : cn.x;
                    }
                }
            }
        }
        __syncthreads(); // the block's regions are free again
    }
    // merge the warps' bests and write the outputs
    const unsigned n_warps = min((unsigned)kShiftBlock, n_shift);
    if ((unsigned)warp < n_warps) {
        if (lane == 0) {
            slots[warp].v = bv;
            slots[warp].h = bh;
            slots[warp].t = bt;
        }
        if (lane < 7)
            slots[warp].nb[lane] = nb;
    }
    __syncthreads();
    if (tid == 0) {
        unsigned best = 0;
        for (unsigned w = 1; w < n_warps; w++)
            if (better(slots[w].v, slots[w].h, slots[w].t, slots[best].v, slots[best].h, slots[best].t))
                best = w;
        const PeakSlot& ps = slots[best];
        const bool mirror = ps.h >= n_shift;
        const unsigned sidx = mirror ? ps.h - n_shift : ps.h;
        const unsigned pg = p_first + p;
        const float angle = peak_angle(ps.nb, ps.t, mirror, kL);
        const float bxv = base ? base[pg].x : 0.f;
        const float byv = base ? base[pg].y : 0.f;
        const float2 sf = shifts_f[sidx];
        const size_t o = (size_t)q * p_total + pg;
        if (GPUISAC_IN_BOUNDS(kChkR512Res, o, (size_t)n_ref * p_total)) {
            d_out[o] = ps.v;
            peak_out[o] = make_float4(angle, bxv + sf.x, byv + sf.y, mirror ? 1.f : 0.f);
        }
    }
}

size_t spectra512_smem(unsigned ring_num)
{
    return (size_t)((ring_num + 1) / 2) * kPair * sizeof(float2) + (kL + 256) * sizeof(float2) + 24 * sizeof(double);
}

size_t ccf512_smem(unsigned ring_num)
{
    return ((size_t)ring_num * kS + kShiftBlock * kPair + 512) * sizeof(float2) + kShiftBlock * sizeof(PeakSlot);
}

} // namespace

GPUISAC_CHECKED_READER(checked_read_ring512)

cudaError_t launch_polar_spectra512(const StackDesc& st, const float2* tmpl, const float2* tw512, unsigned ring_num,
                                    const int2* shift_int, unsigned n_shift, const float2* base, unsigned img0,
                                    unsigned n_img, int is_ref, float2* out, cudaStream_t stream,
                                    const unsigned long long* tex_objs)
{
    if (n_img == 0 || n_shift == 0)
        return cudaSuccess;
    if (ring_num == 0 || ring_num > kMaxRingNum)
        return cudaErrorInvalidValue;
    cudaError_t e = opt_in_smem_k(polar_spectra512_kernel, spectra512_smem(kMaxRingNum));
    if (e != cudaSuccess)
        return e;
    const size_t rows = (size_t)n_img * n_shift;
    if (rows > 0x7FFFFFFFull)
        return cudaErrorInvalidValue;
    polar_spectra512_kernel<<<(unsigned)rows, 256, spectra512_smem(ring_num), stream>>>(
        st, tmpl, tw512, ring_num, shift_int, n_shift, base, img0, n_img, is_ref, out, tex_objs);
    g_kernel_launches.fetch_add(1, std::memory_order_relaxed);
    return cudaGetLastError();
}

cudaError_t launch_ccf_peak512(const float2* sbj_sp, const float2* ref_sp, const float2* tw512, unsigned ring_num,
                               unsigned n_shift, unsigned n_ref, unsigned n_part, unsigned p_first, unsigned p_total,
                               const float2* shifts_f, const float2* base, float* d_out, float4* peak_out,
                               cudaStream_t stream)
{
    if (n_part == 0 || n_ref == 0)
        return cudaSuccess;
    if (ring_num == 0 || ring_num > kMaxRingNum || n_shift == 0)
        return cudaErrorInvalidValue;
    const size_t items = (size_t)n_part * n_ref;
    if (items > 0x7FFFFFFFull)
        return cudaErrorInvalidValue;
    cudaError_t e = opt_in_smem_k(ccf_peak512_kernel, ccf512_smem(kMaxRingNum));
    if (e != cudaSuccess)
        return e;
    ccf_peak512_kernel<<<(unsigned)items, 256, ccf512_smem(ring_num), stream>>>(
        sbj_sp, ref_sp, tw512, ring_num, n_shift, n_ref, n_part, p_first, p_total, shifts_f, base, d_out, peak_out);
    g_kernel_launches.fetch_add(1, std::memory_order_relaxed);
    return cudaGetLastError();
}

} // namespace gpuisac
