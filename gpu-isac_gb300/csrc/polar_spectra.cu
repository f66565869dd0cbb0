// polar_spectra.cu -- polar resampling, per-image normalisation and per-ring
// real FFT of images (one CTA per image x shift), written straight in the
// basis the CCF contraction consumes.
//
// Reference semantics: cu_resample_to_polar (cuda/gpu_aln_noref.cu:1221-1354)
// followed by the in-place R2C cuFFT of every ring (:2121-2125).
//
// Output, per (image, shift) row, [ring][slot] float2:
//   slot k = 1..127 holds F[k]; slot 0 holds (F[0], F[128]) (both real);
//   subjects store (Re+Im, Re-Im)            of that pair of numbers,
//   references store (r+1) * (Re+Im, Re-Im)  (the ring weight folded in).
// With refs (u, v) and subjects (a, b) the four sums sum_r u a, u b, v b, v a
// are exactly Re/Im of Z[k] = O[k] + i M[k] and of Z[256-k], the spectrum
// whose inverse FFT gives the normal (real part) and mirrored (imaginary
// part) correlation at once.
#include <cuda_bf16.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <utility>

#include "gpuisac_device.cuh"
#include "gpuisac_kernels.h"

namespace gpuisac {

std::atomic<unsigned long long> g_kernel_launches{0};

namespace {
std::mutex g_optin_mu;
std::map<std::pair<int, const void*>, int> g_optin; // (device, kernel) -> bytes opted in
} // namespace

cudaError_t opt_in_smem(const void* kernel, int bytes)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return e;
    std::lock_guard<std::mutex> lk(g_optin_mu);
    auto it = g_optin.find({dev, kernel});
    if (it != g_optin.end() && it->second >= bytes)
        return cudaSuccess;
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess)
        g_optin[{dev, kernel}] = bytes;
    return e;
}

int smem_optin_max()
{
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    return v;
}

// smem offset (floats) of ring r's samples
__device__ __forceinline__ unsigned polar_index(unsigned r) { return (r >> 1) * 2 * kPairStride + (r & 1) * kRingLen; }

// split x into BF16 hi = rn(x) and lo = rn(x - hi) (x - hi is exact in FP32)
__device__ __forceinline__ void bf16_split(float x, uint32_t& hi, uint32_t& lo)
{
    const __nv_bfloat16 h = __float2bfloat16_rn(x);
    const __nv_bfloat16 l = __float2bfloat16_rn(x - __bfloat162float(h));
    hi = (uint32_t)__bfloat16_as_ushort(h);
    lo = (uint32_t)__bfloat16_as_ushort(l);
}

// kOperand: the spectra go to shared memory and leave as BF16 hi/lo
// tensor-core operands (OperandLayout) instead of FP32 rows
template <bool kOperand>
__device__ __forceinline__ void
polar_spectra_body(const StackDesc& st, const float2* __restrict__ tmpl, const float2* __restrict__ twiddle,
                   unsigned ring_num, const int2* __restrict__ shift_int, unsigned n_shift,
                   const float2* __restrict__ base, unsigned img0, unsigned n_img, int is_ref,
                   float2* __restrict__ out, const unsigned* __restrict__ img_list,
                   const unsigned long long* __restrict__ tex_objs, const OperandLayout& opnd, unsigned row)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    // ring pair p's samples at polar[p * 2 * kPairStride + (r & 1) * 256 + angle];
    // once a pair is in registers its region is the FFT workspace
    float* polar = reinterpret_cast<float*>(smem_raw);
    const unsigned n_pairs = (ring_num + 1) / 2;
    float2* tw = reinterpret_cast<float2*>(polar + n_pairs * 2 * kPairStride);  // 256
    double* red = reinterpret_cast<double*>(tw + kRingLen);                   // 2 x 8 warps + 2

    const unsigned img_local = row / n_shift;
    const unsigned s = row - img_local * n_shift;
    if (img_local >= n_img)
        return;
    // output row i holds image img0 + i, or img_list[i] when a list is given
    const unsigned img = img_list ? img_list[img_local] : img0 + img_local;
    const int tid = threadIdx.x;

    tw[tid] = twiddle[tid];

    // ---- sampling positions exactly as the reference computes them ----
    const int2 sh = shift_int[s];
    const float* bx = base ? &base[img].x : nullptr;
    const float* by = base ? &base[img].y : nullptr;
    const float cnt_x = centre_coord(st.dim, sh.x, bx);
    const float cnt_y = centre_coord(st.dim, sh.y, by);
    const TexPlacement place = tex_place(st, img);
    const float yoff = (float)(place.local * st.dim);
    // the texture unit itself when the stack has textures, else its emulation
    const cudaTextureObject_t tobj = tex_objs ? (cudaTextureObject_t)__ldg(tex_objs + place.tex_id) : 0;

    // thread tid samples angle tid of every ring; FP32 ring-weighted partial
    // sums, reduced in FP32 across each warp, feed the image mean / deviation
    // (the eight warp sums are added in FP64)
    float s1 = 0.f, s2 = 0.f;
#pragma unroll 8
    for (unsigned r = 0; r < ring_num; r++) {
        const float2 o = GPUISAC_IN_BOUNDS(kChkSpectraTmpl, r * kRingLen + tid, ring_num * kRingLen)
                             ? __ldg(&tmpl[r * kRingLen + tid])
                             : make_float2(0.f, 0.f);
        float x = cnt_x + o.x;
        float y = (yoff + cnt_y) + o.y;
        float v = tex_objs ? tex2D<float>(tobj, x, y) : tex_sample(st, place, x, y);
        polar[polar_index(r) + tid] = v;
        float w = (float)(r + 1);
        s1 += w * v;
        s2 += w * v * v;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        s1 += __shfl_xor_sync(0xffffffffu, s1, off);
        s2 += __shfl_xor_sync(0xffffffffu, s2, off);
    }
    const double d1 = s1, d2 = s2;
    const int warp = tid >> 5, lane = tid & 31;
    if (lane == 0) {
        red[warp] = d1;
        red[8 + warp] = d2;
    }
    __syncthreads();
    if (tid == 0) {
        double a = 0.0, q = 0.0;
        for (int w = 0; w < 8; w++) {
            a += red[w];
            q += red[8 + w];
        }
        // avg = sum (r+1) A_r / (L sum (r+1)); same for the squares (noref.cu:1314-1337)
        double nn = 0.5 * (double)ring_num * (double)(ring_num + 1) * (double)kRingLen;
        double avg = a / nn, msq = q / nn;
        double sd = sqrt(fabs(msq - avg * avg));
        // stored as the floats every thread uses (one conversion, not 256)
        float* redf = reinterpret_cast<float*>(red + 16);
        redf[0] = (float)avg;
        redf[1] = (float)(1.0 / (sd + 0.0000001));
    }
    __syncthreads();
    const float avg_f = reinterpret_cast<const float*>(red + 16)[0];
    const float inv_f = reinterpret_cast<const float*>(red + 16)[1];

    // ---- per-ring FFT, two rings per complex 256-point FFT ----
    const int g = tid >> 4;          // FFT group 0..15
    const int l = tid & 15;
    const unsigned gmask = 0xffffu << (tid & 16);
    float2* out_row = out + (size_t)row * ring_num * kSlots;
    for (unsigned pr = g; pr < n_pairs; pr += 16) {
        const unsigned ra = 2 * pr, rb = 2 * pr + 1;
        const bool has_b = rb < ring_num;
        const float* pa = polar + pr * 2 * kPairStride;
        float2* gws = reinterpret_cast<float2*>(polar) + pr * kPairStride;
        float2 x[16];
        float2 oa[kOperand ? 8 : 1], ob[kOperand ? 8 : 1];
#pragma unroll
        for (int m = 0; m < 16; m++) {
            float va = (pa[l + 16 * m] - avg_f) * inv_f;
            float vb = has_b ? (pa[kRingLen + l + 16 * m] - avg_f) * inv_f : 0.f;
            x[m] = make_float2(va, vb);
        }
        __syncwarp(gmask); // the pair's samples are read before its region turns workspace
        fft256_group<-1, false>(x, gws, tw, l, gmask);
        // natural-order spectrum Z[l + 16 k2] to the workspace
#pragma unroll
        for (int k2 = 0; k2 < 16; k2++)
            gws[l + 16 * k2] = x[perm16(k2)];
        __syncwarp(gmask);
        // unpack the two real spectra and write slots k = l + 16 i (i = 0..7)
#pragma unroll
        for (int i = 0; i < 8; i++) {
            const int k = l + 16 * i;
            float2 z = gws[k];
            float2 zc = gws[(kRingLen - k) & (kRingLen - 1)];
            // F_a = (Z[k] + conj Z[256-k]) / 2 ; F_b = (Z[k] - conj Z[256-k]) / (2i)
            float2 fa = make_float2(0.5f * (z.x + zc.x), 0.5f * (z.y - zc.y));
            float2 fb = make_float2(0.5f * (z.y + zc.y), -0.5f * (z.x - zc.x));
            if (k == 0) {
                // slot 0 carries (F[0], F[128]); both are real
                float2 zn = gws[kSlots];
                fa = make_float2(z.x, zn.x);
                fb = make_float2(z.y, zn.y);
            }
            float wa = is_ref ? (float)(ra + 1) : 1.f;
            float wb = is_ref ? (float)(rb + 1) : 1.f;
            if (kOperand) {
                oa[i] = make_float2(wa * (fa.x + fa.y), wa * (fa.x - fa.y));
                ob[i] = make_float2(wb * (fb.x + fb.y), wb * (fb.x - fb.y));
            } else {
                const size_t n_out = (size_t)n_img * n_shift * ring_num * kSlots;
                const size_t at = (size_t)row * ring_num * kSlots + ra * kSlots + k;
                if (GPUISAC_IN_BOUNDS(kChkSpectraOut, at, n_out))
                    out_row[ra * kSlots + k] = make_float2(wa * (fa.x + fa.y), wa * (fa.x - fa.y));
                if (has_b && GPUISAC_IN_BOUNDS(kChkSpectraOut, at + kSlots, n_out))
                    out_row[rb * kSlots + k] = make_float2(wb * (fb.x + fb.y), wb * (fb.x - fb.y));
            }
        }
        __syncwarp(gmask);
        if (kOperand) {
            // the pair's region now holds its two rings' spectra: ring ra at
            // [0, 128), ring rb at [128, 256) (zero for a missing ring)
#pragma unroll
            for (int i = 0; i < 8; i++) {
                gws[l + 16 * i] = oa[i];
                gws[kSlots + l + 16 * i] = has_b ? ob[i] : make_float2(0.f, 0.f);
            }
            __syncwarp(gmask);
        }
    }
    if (!kOperand)
        return;
    __syncthreads();
    // ---- write-out as BF16 hi/lo operand rows ----
    const unsigned tile = is_ref ? img_local / opnd.block : img_local * opnd.n_blocks + s / opnd.block;
    const unsigned orow = 2 * (is_ref ? img_local % opnd.block : s % opnd.block); // a / u; +1: b / v
    unsigned char* tb = opnd.base + (size_t)tile * opnd.tile_bytes() + (orow >> 3) * 128 + (orow & 7) * 16;
    const size_t sb = opnd.slot_bytes(), hb = (size_t)opnd.kg * opnd.rg * 128, kb = (size_t)opnd.rg * 128;
    const float2* spec = reinterpret_cast<const float2*>(polar);
    for (unsigned it = tid; it < kSlots * opnd.kg; it += 256) {
        const unsigned k = it & (kSlots - 1), kgi = it >> 7;
        uint32_t ah[4], al[4], bh[4], bl[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
            float2 v[2];
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const unsigned r = 8 * kgi + 2 * j + h;
                v[h] = r < ring_num ? spec[(r >> 1) * kPairStride + (r & 1) * kSlots + k] : make_float2(0.f, 0.f);
            }
            uint32_t h0, l0, h1, l1;
            bf16_split(v[0].x, h0, l0);
            bf16_split(v[1].x, h1, l1);
            ah[j] = h0 | (h1 << 16);
            al[j] = l0 | (l1 << 16);
            bf16_split(v[0].y, h0, l0);
            bf16_split(v[1].y, h1, l1);
            bh[j] = h0 | (h1 << 16);
            bl[j] = l0 | (l1 << 16);
        }
        unsigned char* p = tb + k * sb + kgi * kb;
        const size_t n_tiles = is_ref ? (n_img + opnd.block - 1) / opnd.block : (size_t)n_img * opnd.n_blocks;
        if (!GPUISAC_IN_BOUNDS(kChkOperandOut, (size_t)(p - opnd.base) + hb + 31, n_tiles * opnd.tile_bytes()))
            continue;
        *reinterpret_cast<uint4*>(p) = make_uint4(ah[0], ah[1], ah[2], ah[3]);
        *reinterpret_cast<uint4*>(p + 16) = make_uint4(bh[0], bh[1], bh[2], bh[3]);
        *reinterpret_cast<uint4*>(p + hb) = make_uint4(al[0], al[1], al[2], al[3]);
        *reinterpret_cast<uint4*>(p + hb + 16) = make_uint4(bl[0], bl[1], bl[2], bl[3]);
    }
}

__global__ void __launch_bounds__(256, 5)
polar_spectra_kernel(StackDesc st, const float2* __restrict__ tmpl, const float2* __restrict__ twiddle,
                     unsigned ring_num, const int2* __restrict__ shift_int, unsigned n_shift,
                     const float2* __restrict__ base, unsigned img0, unsigned n_img, int is_ref,
                     float2* __restrict__ out, const unsigned* __restrict__ img_list,
                     const unsigned long long* __restrict__ tex_objs)
{
    polar_spectra_body<false>(st, tmpl, twiddle, ring_num, shift_int, n_shift, base, img0, n_img, is_ref, out,
                              img_list, tex_objs, OperandLayout(), blockIdx.x);
}

// The same rows for a table of jobs (SpectraJobs), one CTA per row, the row
// count read from device memory so that a recorded launch (grid = the
// capacity) serves any table the buffers hold.  A row's job: the lookup entry
// of its block of kJobLutRows rows (the job holding the block's first row),
// then forward over the jobs that start inside the block.
__global__ void __launch_bounds__(256, 5)
polar_spectra_jobs_kernel(const SpectraJob* __restrict__ jobs, const unsigned* __restrict__ hdr,
                          const unsigned* __restrict__ lut, const float2* __restrict__ tmpl,
                          const float2* __restrict__ twiddle, unsigned ring_num)
{
    const unsigned row = blockIdx.x;
    if (row >= hdr[2])
        return;
    const unsigned last = hdr[0] + hdr[1] - 1;
    unsigned j = lut[hdr[3] + row / kJobLutRows];
    while (j < last && jobs[j + 1].row_begin <= row)
        j++;
    const SpectraJob& jb = jobs[j];
    polar_spectra_body<false>(jb.st, tmpl, twiddle, ring_num, jb.shift_int, jb.n_shift, jb.base, jb.img0, jb.n_img,
                              jb.is_ref, jb.out, nullptr, jb.tex_objs, OperandLayout(), row - jb.row_begin);
}

__global__ void __launch_bounds__(256, 4)
polar_operands_kernel(StackDesc st, const float2* __restrict__ tmpl, const float2* __restrict__ twiddle,
                      unsigned ring_num, const int2* __restrict__ shift_int, unsigned n_shift,
                      const float2* __restrict__ base, unsigned img0, unsigned n_img, int is_ref,
                      OperandLayout opnd, const unsigned long long* __restrict__ tex_objs)
{
    polar_spectra_body<true>(st, tmpl, twiddle, ring_num, shift_int, n_shift, base, img0, n_img, is_ref, nullptr,
                             nullptr, tex_objs, opnd, blockIdx.x);
}

GPUISAC_CHECKED_READER(checked_read_spectra)

cudaError_t launch_polar_spectra(const StackDesc& st, const float2* tmpl, const float2* twiddle,
                                 unsigned ring_num, const int2* shift_int, unsigned n_shift,
                                 const float2* base, unsigned img0, unsigned n_img, int is_ref,
                                 float2* out, cudaStream_t stream, const unsigned* img_list,
                                 const unsigned long long* tex_objs)
{
    if (n_img == 0 || n_shift == 0)
        return cudaSuccess;
    size_t smem = polar_spectra_smem_bytes(ring_num);
    cudaError_t e = opt_in_smem_k(polar_spectra_kernel, polar_spectra_smem_bytes(kMaxRingNum));
    if (e != cudaSuccess)
        return e;
    unsigned rows = n_img * n_shift;
    polar_spectra_kernel<<<rows, 256, smem, stream>>>(st, tmpl, twiddle, ring_num, shift_int, n_shift, base,
                                                       img0, n_img, is_ref, out, img_list, tex_objs);
    g_kernel_launches.fetch_add(1, std::memory_order_relaxed);
    return cudaGetLastError();
}

cudaError_t launch_polar_spectra_jobs(const SpectraJob* jobs, const unsigned* hdr, const unsigned* lut,
                                      const float2* tmpl, const float2* twiddle, unsigned ring_num, unsigned grid,
                                      cudaStream_t stream)
{
    if (grid == 0)
        return cudaSuccess;
    cudaError_t e = opt_in_smem_k(polar_spectra_jobs_kernel, polar_spectra_smem_bytes(kMaxRingNum));
    if (e != cudaSuccess)
        return e;
    polar_spectra_jobs_kernel<<<grid, 256, polar_spectra_smem_bytes(ring_num), stream>>>(jobs, hdr, lut, tmpl,
                                                                                         twiddle, ring_num);
    g_kernel_launches.fetch_add(1, std::memory_order_relaxed);
    return cudaGetLastError();
}

cudaError_t launch_polar_operands(const StackDesc& st, const float2* tmpl, const float2* twiddle,
                                  unsigned ring_num, const int2* shift_int, unsigned n_shift,
                                  const float2* base, unsigned img0, unsigned n_img, int is_ref,
                                  const OperandLayout& opnd, cudaStream_t stream,
                                  const unsigned long long* tex_objs)
{
    if (n_img == 0 || n_shift == 0)
        return cudaSuccess;
    if (!opnd.base || opnd.block == 0 || opnd.kg * 8 < ring_num || (is_ref && n_shift != 1) ||
        opnd.rg * 8 < 2 * opnd.block || (!is_ref && opnd.block * opnd.n_blocks < n_shift))
        return cudaErrorInvalidValue;
    size_t smem = polar_spectra_smem_bytes(ring_num);
    cudaError_t e = opt_in_smem_k(polar_operands_kernel, polar_spectra_smem_bytes(kMaxRingNum));
    if (e != cudaSuccess)
        return e;
    unsigned rows = n_img * n_shift;
    polar_operands_kernel<<<rows, 256, smem, stream>>>(st, tmpl, twiddle, ring_num, shift_int, n_shift, base, img0,
                                                        n_img, is_ref, opnd, tex_objs);
    g_kernel_launches.fetch_add(1, std::memory_order_relaxed);
    return cudaGetLastError();
}

} // namespace gpuisac
