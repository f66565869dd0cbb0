// gpuisac_device.cuh -- device building blocks shared by the alignment kernels:
// complex helpers, the 16-point DFT, the 256-point FFT split over 16 threads,
// and the texture-unit-faithful bilinear sampler of the stacked image arrays.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace gpuisac {

// ---------------------------------------------------------------------------
// Checked build (-DGPUISAC_CHECKED): a guarded global access first tests its
// element (or byte) index against the extent the kernel was given; a failing
// access is skipped and recorded -- a count and the first (site, index) -- in
// this translation unit's device words, never trapped.  The host reads and
// clears them with the translation unit's reader (GPUISAC_CHECKED_READER,
// collected by gpuisac_checked_failures).  In the normal build the guard is
// the constant true.
#ifdef GPUISAC_CHECKED
static __device__ unsigned g_chk_count;
static __device__ unsigned long long g_chk_first;
__device__ __forceinline__ bool chk_in_bounds(unsigned site, unsigned long long i, unsigned long long n)
{
    if (i < n)
        return true;
    if (atomicAdd(&g_chk_count, 1u) == 0u)
        g_chk_first = ((unsigned long long)site << 48) | (i & 0xFFFFFFFFFFFFull);
    return false;
}
#define GPUISAC_IN_BOUNDS(site, i, n) \
    (::gpuisac::chk_in_bounds((site), (unsigned long long)(i), (unsigned long long)(n)))
#define GPUISAC_CHECKED_READER(fn)                                                        \
    void fn(unsigned& count, unsigned long long& first)                                    \
    {                                                                                      \
        cudaMemcpyFromSymbol(&count, g_chk_count, sizeof(count));                          \
        cudaMemcpyFromSymbol(&first, g_chk_first, sizeof(first));                          \
        const unsigned zero = 0;                                                           \
        cudaMemcpyToSymbol(g_chk_count, &zero, sizeof(zero));                              \
    }
#else
#define GPUISAC_IN_BOUNDS(site, i, n) true
#define GPUISAC_CHECKED_READER(fn)                                                        \
    void fn(unsigned& count, unsigned long long& first)                                    \
    {                                                                                      \
        count = 0;                                                                         \
        first = 0;                                                                         \
    }
#endif
// guarded sites (the high 16 bits of a recorded failure)
enum {
    kChkSpectraOut = 1, kChkSpectraTmpl, kChkOperandOut, kChkMmaZ, kChkMmaA, kChkMmaB, kChkZfftZ, kChkZfftOut,
    kChkMergeOut, kChkCcfRow, kChkR512Out, kChkR512Row, kChkR512Res, kChkAvgImg, kChkAvgPartial, kChkAvgOut
};

constexpr int kRingLen = 256;        // polar samples per ring (angles)
constexpr int kSlots = kRingLen / 2; // spectrum slots per ring: k = 1..127, slot 0 = (F[0], F[128])
constexpr int kFftGroup = 16;        // threads per 256-point FFT
constexpr int kPairStride = 272;     // float2 per FFT workspace (16 x 17, padded transpose)

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// multiply by +i (SIGN>0) or -i (SIGN<0)
template <int SIGN>
__device__ __forceinline__ float2 cmul_i(float2 a)
{
    return SIGN > 0 ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

// 4-point DFT in place, X[k] = sum_n x[n] w4^(SIGN n k), w4 = e^(2 pi i / 4).
// The component-wise sums and differences run as packed two-lane FP32
// instructions (x - y as fma(y, -1, x): the product is exact, so each lane
// rounds exactly as a scalar subtraction); the two outputs that need the
// multiplication by +-i swap components and stay scalar.
template <int SIGN, bool kPacked = true>
__device__ __forceinline__ void dft4(float2& x0, float2& x1, float2& x2, float2& x3)
{
    if (!kPacked) { // the same sums in scalar instructions (fewer live registers)
        const float2 a = cadd(x0, x2), b = csub(x0, x2);
        const float2 c = cadd(x1, x3), d = cmul_i<SIGN>(csub(x1, x3));
        x0 = cadd(a, c);
        x2 = csub(a, c);
        x1 = cadd(b, d);
        x3 = csub(b, d);
        return;
    }
    const float2 m1 = make_float2(-1.f, -1.f);
    const float2 a = __fadd2_rn(x0, x2), b = __ffma2_rn(x2, m1, x0);
    const float2 c = __fadd2_rn(x1, x3), d = cmul_i<SIGN>(__ffma2_rn(x3, m1, x1));
    x0 = __fadd2_rn(a, c);
    x2 = __ffma2_rn(c, m1, a);
    x1 = cadd(b, d);
    x3 = csub(b, d);
}

// e^(SIGN 2 pi i m / 16) for m = 0..9 (cos/sin of multiples of 22.5 degrees)
template <int SIGN>
__device__ __forceinline__ float2 w16(int m)
{
    const float c1 = 0.923879532511286756f, s1 = 0.382683432365089772f, c2 = 0.707106781186547524f;
    float2 r;
    switch (m) {
    case 0: r = make_float2(1.f, 0.f); break;
    case 1: r = make_float2(c1, s1); break;
    case 2: r = make_float2(c2, c2); break;
    case 3: r = make_float2(s1, c1); break;
    case 4: r = make_float2(0.f, 1.f); break;
    case 6: r = make_float2(-c2, c2); break;
    case 9: r = make_float2(-c1, -s1); break;
    default: r = make_float2(1.f, 0.f); break;
    }
    r.y *= (float)SIGN;
    return r;
}

// 16-point DFT in registers, in place:
// X[k] = sum_n x[n] e^(SIGN 2 pi i n k / 16) for natural-order input x[n];
// the output is left 4x4-transposed: X[k] is found at x[perm16(k)].
// 16 = 4 x 4 with twiddles w16^(n1 k1).
__host__ __device__ constexpr int perm16(int k) { return 4 * (k & 3) + (k >> 2); }

template <int SIGN, bool kPacked = true>
__device__ __forceinline__ void dft16(float2 (&x)[16])
{
    // stage 1: for each n1, 4-point DFT over n2 of x[n1 + 4 n2] -> T[n1][k1] at x[n1 + 4 k1]
#pragma unroll
    for (int n1 = 0; n1 < 4; n1++)
        dft4<SIGN, kPacked>(x[n1], x[n1 + 4], x[n1 + 8], x[n1 + 12]);
    // twiddle by w16^(n1 k1)
#pragma unroll
    for (int n1 = 1; n1 < 4; n1++)
#pragma unroll
        for (int k1 = 1; k1 < 4; k1++)
            x[n1 + 4 * k1] = cmul(x[n1 + 4 * k1], w16<SIGN>(n1 * k1));
    // stage 2: for each k1, 4-point DFT over n1 of x[4 k1 + n1] -> X[k1 + 4 k2] at x[4 k1 + k2]
#pragma unroll
    for (int k1 = 0; k1 < 4; k1++)
        dft4<SIGN, kPacked>(x[4 * k1 + 0], x[4 * k1 + 1], x[4 * k1 + 2], x[4 * k1 + 3]);
}

// 256-point complex FFT over a group of 16 threads (thread l = 0..15).
// In:  x[m] = z[l + 16 m].
// Out: x[perm16(k2)] = Z[l + 16 k2],  Z[k] = sum_n z[n] e^(SIGN 2 pi i n k / 256).
// ws: this group's workspace of kPairStride float2; tw: e^(-2 pi i e / 256),
// e = 0..255 (forward twiddles; the inverse conjugates them).
// Every thread of the group must call; mask = the group's lanes.
template <int SIGN, bool kPacked = true>
__device__ __forceinline__ void fft256_group(float2 (&x)[16], float2* ws, const float2* tw, int l,
                                             unsigned mask)
{
    dft16<SIGN, kPacked>(x);
    // twiddle w256^(SIGN l j) of output j
#pragma unroll
    for (int j = 1; j < 16; j++) {
        float2 w = tw[(l * j) & 255];
        w.y *= (float)(-SIGN); // table holds e^(-...), flip for SIGN=+1
        x[perm16(j)] = cmul(x[perm16(j)], w);
    }
    // transpose through shared memory (row stride 17 avoids bank conflicts)
    __syncwarp(mask);
#pragma unroll
    for (int j = 0; j < 16; j++)
        ws[l * 17 + j] = x[perm16(j)];
    __syncwarp(mask);
#pragma unroll
    for (int n = 0; n < 16; n++)
        x[n] = ws[n * 17 + l];
    __syncwarp(mask);
    dft16<SIGN, kPacked>(x);
}

// The same FFT with this thread's twiddles precomputed: twl[j] = the factor
// fft256_group applies to output j of thread l (the table's e^(-2 pi i l j / 256)
// with the sign of SIGN), read at fixed offsets instead of through (l j) & 255.
// Rows of 17 float2 keep the 16 threads of a group on distinct banks.
constexpr int kTwRow = 17;
template <int SIGN>
__device__ __forceinline__ void fft256_group_twl(float2 (&x)[16], float2* ws, const float2* twl, unsigned mask)
{
    const int l = threadIdx.x & 15;
    dft16<SIGN>(x);
#pragma unroll
    for (int j = 1; j < 16; j++)
        x[perm16(j)] = cmul(x[perm16(j)], twl[j]);
    __syncwarp(mask);
#pragma unroll
    for (int j = 0; j < 16; j++)
        ws[l * 17 + j] = x[perm16(j)];
    __syncwarp(mask);
#pragma unroll
    for (int n = 0; n < 16; n++)
        x[n] = ws[n * 17 + l];
    __syncwarp(mask);
    dft16<SIGN>(x);
}

// ---------------------------------------------------------------------------
// Stacked image arrays read the way the reference's 2D textures are read
// (bilinear, clamp, unnormalised coordinates; cuda/gpu_aln_noref.cu:1258-1286,
// 2314-2339): images are grouped in batches of `batch`, each batch in textures
// of `tex` images; a bilinear tap below/above an image reads the neighbouring
// image of the same texture, the ends of a texture clamp, and texture slots a
// short final batch leaves untouched still hold the previous batch's images.
struct StackDesc {
    const float* img; // [n][dim][dim]
    unsigned n, dim, batch, tex;
};

struct TexPlacement {
    unsigned local;      // image index inside its texture (the reference's block index)
    unsigned tex_id;     // texture (batch-major, textures of a batch in order) holding the image
    unsigned tex_first;  // global index of the texture's slot 0
    unsigned batch_end;  // one past the last image of the current batch
    long rows;           // texture height in rows
};

__device__ __forceinline__ TexPlacement tex_place(const StackDesc& s, unsigned img)
{
    TexPlacement t;
    unsigned bstart = (img / s.batch) * s.batch;
    unsigned blen = min(s.batch, s.n - bstart);
    unsigned loc = img - bstart;
    unsigned tex_idx = loc / s.tex;
    unsigned n_tex_alloc = (s.batch + s.tex - 1) / s.tex;
    unsigned alloc = (tex_idx != n_tex_alloc - 1) ? s.tex : s.batch - tex_idx * s.tex;
    t.local = loc - tex_idx * s.tex;
    t.tex_id = (bstart / s.batch) * n_tex_alloc + tex_idx;
    t.tex_first = bstart + tex_idx * s.tex;
    t.batch_end = bstart + blen;
    t.rows = (long)alloc * s.dim;
    return t;
}

__device__ __forceinline__ const float* tex_row(const StackDesc& s, const TexPlacement& t, long row)
{
    row = row < 0 ? 0 : (row > t.rows - 1 ? t.rows - 1 : row);
    // a sample's rows lie in its own image or a neighbour: resolve the slot
    // without a 64-bit division (the general case keeps it)
    const int dim = (int)s.dim;
    const long rel = row - (long)t.local * dim;
    unsigned slot, yy;
    if (rel >= 0 && rel < dim) {
        slot = t.local;
        yy = (unsigned)rel;
    } else if (rel < 0 && rel >= -dim) {
        slot = t.local - 1;
        yy = (unsigned)(rel + dim);
    } else if (rel >= dim && rel < 2 * dim) {
        slot = t.local + 1;
        yy = (unsigned)(rel - dim);
    } else {
        slot = (unsigned)(row / s.dim);
        yy = (unsigned)(row - (long)slot * s.dim);
    }
    unsigned g = t.tex_first + slot;
    if (g >= t.batch_end)
        g -= s.batch; // slot not refilled by a short final batch
    return s.img + ((size_t)g * s.dim + yy) * s.dim;
}

// Texel-space coordinates in fixed point with 8 fractional bits, rounded to
// nearest with ties upward, as the texture unit does (the oracle's
// orc_tex_split; (t - 0.5) * 256 is exact in float).  The texture unit's tap
// weights, in units of 1/256: w11 = round(A*B/256) (ties upward) for the 8-bit
// fractions A, B; the other taps take what is left of each fraction, so the
// weights sum to 256 (the oracle's orc_tex_weights, pinned against the
// hardware).
__device__ __forceinline__ float tex_sample(const StackDesc& s, const TexPlacement& t, float x, float y)
{
    // fixed-point coordinates q = round((t - 0.5) * 256), ties upward; the
    // integer part selects the texel, the low 8 bits are the fraction
    const float xs = (x - 0.5f) * 256.0f, ys = (y - 0.5f) * 256.0f;
    const float flx = floorf(xs), fly = floorf(ys);
    const int qx = (int)flx + ((xs - flx) >= 0.5f ? 1 : 0);
    const int qy = (int)fly + ((ys - fly) >= 0.5f ? 1 : 0);
    const int ix = qx >> 8, iy = qy >> 8;
    const int A = qx & 255, B = qy & 255;
    const int w11 = (A * B + 128) >> 8;
    const float f00 = (float)(256 - A - B + w11), f10 = (float)(A - w11), f01 = (float)(B - w11), f11 = (float)w11;
    const int dim = (int)s.dim;
    const float *r0, *r1;
    const int rel = iy - (int)t.local * dim;
    if (rel >= 0 && rel < dim - 1) {
        // both rows inside the sample's own image (the common case)
        r0 = s.img + ((size_t)(t.tex_first + t.local) * dim + rel) * dim;
        r1 = r0 + dim;
    } else {
        r0 = tex_row(s, t, iy);
        r1 = tex_row(s, t, (long)iy + 1);
    }
    float t00, t10, t01, t11;
    if (ix >= 0 && ix < dim - 1) {
        t00 = __ldg(r0 + ix);
        t10 = __ldg(r0 + ix + 1);
        t01 = __ldg(r1 + ix);
        t11 = __ldg(r1 + ix + 1);
    } else {
        const int x0 = min(max(ix, 0), dim - 1), x1 = min(max(ix + 1, 0), dim - 1);
        t00 = __ldg(r0 + x0);
        t10 = __ldg(r0 + x1);
        t01 = __ldg(r1 + x0);
        t11 = __ldg(r1 + x1);
    }
    return (f00 * t00 + f10 * t10 + f01 * t01 + f11 * t11) * (1.0f / 256.0f);
}

// Reference: polar grid centre, cuda/gpu_aln_noref.cu:1262-1269 (D/2 + shift in
// unsigned arithmetic, base shift added in float, +0.5 in double, stored
// float).  A float plus 0.5 is exact in double, so rounding that sum to float
// is the float addition itself: half_up(f) == (float)((double)f + 0.5).
__device__ __forceinline__ float half_up(float f) { return __fadd_rn(f, 0.5f); }

__device__ __forceinline__ float centre_coord(unsigned dim, int shift, const float* base)
{
    unsigned u = dim / 2u + (unsigned)shift;
    if (base)
        return half_up(__fadd_rn((float)u, *base));
    return half_up((float)u); // u < 2^24: exact as float
}

} // namespace gpuisac
