// averages.cu -- the averaging step of ISAC's main iteration, after the
// equal-size group assignment (bin/sp_isac2_gpu.py:1153-1234): every particle
// rot_shift2D'd by the alignment parameters of its pair with its group's
// reference and added to the group's sum; the groups' mean shifts; every
// particle's parameters re-centred by them; each sum times 1/members,
// low-passed (filt_tanl) and moved by minus its mean shift (fshift).  The
// reference runs these steps on the host through EMAN2 (not part of the
// reference tree): rot_shift2D with its default quadratic interpolation in
// "background" mode and the x-mirror after it, add_img, mul_scalar,
// filt_tanl, fshift; the caller's conversion of the peak parameters
// (:1015-1022) comes first.
//
// Kernels, in stream order:
//  1. avg_count_kernel       members per (chunk of 1024 particles, group)
//  2. avg_chunk_scan_kernel  per group: exclusive offsets over the chunks
//  3. avg_group_scan_kernel  per group: first member, first piece, totals
//  4. avg_convert_kernel     thread per particle: its converted parameters
//  5. avg_scatter_kernel     stable counting sort: each group's members in
//                            particle order
//  6. avg_shift_kernel       one warp per group: mean shifts, parameters
//  7. avg_sum_kernel         one CTA per piece (a run of one group's members):
//                            each member image staged in shared memory by a
//                            bulk copy (two buffers, the member's record
//                            written beside it), every thread one column
//                            and every G-th row of the output, the quadratic
//                            interpolation from shared memory, FP32 sums in
//                            registers, one partial image per piece
//  8. avg_finish_kernel      one CTA per group: its pieces summed in order,
//                            times float(1/members); real 2D DFT, filter and
//                            phase shift, inverse DFT
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <mutex>
#include <vector>

#include "../../include/gpu_aln_pack.h"
#include "ccf_device.cuh"
#include "gpuisac_kernels.h"
#include "host_geometry.h"

namespace gpuisac {
namespace {

constexpr unsigned kAvgChunk = 1024;      // particles per counting-sort chunk
constexpr unsigned kSmemGroups = 16384;   // scatter: a chunk's group offsets in shared memory up to this
constexpr unsigned kMaxDim = 256;         // image side limit
constexpr unsigned kStagedMaxDim = 160;   // member images staged in shared memory (two buffers) up to this
constexpr unsigned kFinishSmemDim = 160;  // finish kernel's spectra in shared memory up to this
constexpr unsigned kFinishThreads = 512;
constexpr double kPi = 3.141592653589793;

// error words: [0] belongsto entries outside [0, n_class), [1] the first such
// particle, [2] empty groups, [3] the first empty group, [4] bulk-copy waits
// that ran out
enum { kErrBad = 0, kErrBadFirst, kErrEmpty, kErrEmptyFirst, kErrWait, kErrWords };

// one member of a group, in the group's particle order (32 bytes)
struct AvgMember {
    float c, s;   // cos, sin of the angle (FP64 values rounded to float)
    float sx, sy; // the caller's converted shift, float as its peak_list
    float ang;
    unsigned img;
    unsigned mirror;
    unsigned pad;
};

__global__ void __launch_bounds__(256)
avg_count_kernel(const int* __restrict__ bel, unsigned P, unsigned R, unsigned* __restrict__ cnt,
                 unsigned* __restrict__ err)
{
    const unsigned c = blockIdx.x;
    const unsigned i1 = min(P, (c + 1) * kAvgChunk);
    for (unsigned i = c * kAvgChunk + threadIdx.x; i < i1; i += blockDim.x) {
        const int r = bel[i];
        if (r < 0 || (unsigned)r >= R) {
            atomicAdd(err + kErrBad, 1u);
            atomicMin(err + kErrBadFirst, i);
        } else {
            atomicAdd(cnt + (size_t)c * R + r, 1u);
        }
    }
}

// thread per group: cnt[c][r] <- members of r in chunks before c; total[r]
__global__ void __launch_bounds__(256)
avg_chunk_scan_kernel(unsigned* __restrict__ cnt, unsigned n_chunks, unsigned R, unsigned* __restrict__ total)
{
    const unsigned r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= R)
        return;
    unsigned run = 0;
    for (unsigned c0 = 0; c0 < n_chunks; c0 += 8) {
        unsigned v[8];
#pragma unroll
        for (unsigned k = 0; k < 8; k++)
            v[k] = c0 + k < n_chunks ? cnt[(size_t)(c0 + k) * R + r] : 0u;
#pragma unroll
        for (unsigned k = 0; k < 8; k++)
            if (c0 + k < n_chunks) {
                cnt[(size_t)(c0 + k) * R + r] = run;
                run += v[k];
            }
    }
    total[r] = run;
}

// one CTA of 1024 threads: start[r] = members of the groups before r,
// pstart[r] = pieces of the groups before r (pstart[R] = all pieces),
// members[r] (optional output), empty groups flagged
__global__ void __launch_bounds__(1024)
avg_group_scan_kernel(const unsigned* __restrict__ total, unsigned R, unsigned piece, unsigned* __restrict__ start,
                      unsigned* __restrict__ pstart, int* __restrict__ members, unsigned* __restrict__ err)
{
    __shared__ unsigned wa[32], wb[32], carry[2];
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0)
        carry[0] = carry[1] = 0;
    __syncthreads();
    for (unsigned r0 = 0; r0 < R; r0 += 1024) {
        const unsigned r = r0 + threadIdx.x;
        const unsigned m = r < R ? total[r] : 0u;
        const unsigned np = (m + piece - 1) / piece;
        unsigned a = m, b = np;
#pragma unroll
        for (unsigned o = 1; o < 32; o <<= 1) {
            const unsigned ta = __shfl_up_sync(0xffffffffu, a, o), tb = __shfl_up_sync(0xffffffffu, b, o);
            if (lane >= o) {
                a += ta;
                b += tb;
            }
        }
        if (lane == 31)
            wa[warp] = a, wb[warp] = b;
        __syncthreads();
        if (warp == 0) {
            unsigned x = wa[lane], y = wb[lane];
#pragma unroll
            for (unsigned o = 1; o < 32; o <<= 1) {
                const unsigned tx = __shfl_up_sync(0xffffffffu, x, o), ty = __shfl_up_sync(0xffffffffu, y, o);
                if (lane >= o) {
                    x += tx;
                    y += ty;
                }
            }
            wa[lane] = x;
            wb[lane] = y;
        }
        __syncthreads();
        const unsigned ca = carry[0], cb = carry[1];
        if (r < R) {
            start[r] = ca + (warp ? wa[warp - 1] : 0u) + a - m;
            pstart[r] = cb + (warp ? wb[warp - 1] : 0u) + b - np;
            if (members)
                members[r] = (int)m;
            if (m == 0) {
                atomicAdd(err + kErrEmpty, 1u);
                atomicMin(err + kErrEmptyFirst, r);
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            carry[0] = ca + wa[31];
            carry[1] = cb + wb[31];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0)
        pstart[R] = carry[1];
}

// thread per particle: its member record from the peak of its group's pair,
// with the caller's conversion (bin/sp_isac2_gpu.py:1015-1022):
// sx = -sx_peak cos(a) - sy_peak sin(a), sy = sx_peak sin(a) - sy_peak cos(a),
// in FP64 (one rounding per operation), rounded to float
__global__ void __launch_bounds__(256)
avg_convert_kernel(const int* __restrict__ bel, unsigned P, unsigned R, const float4* __restrict__ peaks,
                   unsigned long long pitch, AvgMember* __restrict__ rec)
{
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P)
        return;
    const int r = bel[i];
    if (r < 0 || (unsigned)r >= R)
        return;
    const float4 pk = peaks[(size_t)r * pitch + i];
    const double t = __dmul_rn((double)pk.x, kPi / 180.0);
    double sn, cs;
    sincos(t, &sn, &cs);
    const double sxn = -(double)pk.y, syn = -(double)pk.z, ss = -sn;
    AvgMember m;
    m.sx = (float)__dsub_rn(__dmul_rn(sxn, cs), __dmul_rn(syn, ss));
    m.sy = (float)__dadd_rn(__dmul_rn(sxn, ss), __dmul_rn(syn, cs));
    m.c = (float)cs;
    m.s = (float)sn;
    m.ang = pk.x;
    m.img = i;
    m.mirror = pk.w != 0.0f;
    m.pad = 0;
    rec[i] = m;
}

// one warp per chunk, particles in order: order[slot] = particle, the slot
// its group's first member + the members of its group in earlier chunks +
// those earlier in this chunk (match_any within each 32 particles, then the
// group's running count in shared memory).  The chunk's groups are loaded
// first, 32 per lane, so the 32 steps wait on no global load.
__global__ void __launch_bounds__(32)
avg_scatter_kernel(const int* __restrict__ bel, unsigned P, unsigned R, unsigned* __restrict__ cnt,
                   const unsigned* __restrict__ start, unsigned* __restrict__ order)
{
    extern __shared__ unsigned row_s[];
    const unsigned c = blockIdx.x, lane = threadIdx.x;
    const bool in_smem = R <= kSmemGroups;
    unsigned* row = in_smem ? row_s : cnt + (size_t)c * R;
    if (in_smem)
        for (unsigned r = lane; r < R; r += 32)
            row_s[r] = cnt[(size_t)c * R + r] + start[r];
    const unsigned i0 = c * kAvgChunk, i1 = min(P, i0 + kAvgChunk);
    int g[kAvgChunk / 32];
#pragma unroll
    for (unsigned s = 0; s < kAvgChunk / 32; s++) {
        const unsigned i = i0 + s * 32 + lane;
        g[s] = i < i1 ? bel[i] : -1;
    }
    __syncwarp();
#pragma unroll
    for (unsigned s = 0; s < kAvgChunk / 32; s++) {
        const unsigned i = i0 + s * 32 + lane;
        const bool ok = g[s] >= 0 && (unsigned)g[s] < R;
        const unsigned r = ok ? (unsigned)g[s] : 0xffffffffu;
        const unsigned peers = __match_any_sync(0xffffffffu, r);
        const unsigned leader = __ffs(peers) - 1;
        const unsigned rank = __popc(peers & ((1u << lane) - 1u));
        unsigned base = (ok && lane == leader) ? row[r] : 0u;
        base = __shfl_sync(0xffffffffu, base, leader);
        __syncwarp();
        if (ok && lane == leader)
            row[r] = base + __popc(peers);
        if (ok)
            order[base + rank + (in_smem ? 0u : start[r])] = i;
        __syncwarp();
    }
}

// one warp per group: the shift sums in FP64 (a mirrored particle's sx
// subtracted), rounded to float and divided by the member count; every
// member's parameters (ang, sx -/+ mean, sy - mean, mirror) as float
__global__ void __launch_bounds__(256)
avg_shift_kernel(const AvgMember* __restrict__ rec, const unsigned* __restrict__ order, const unsigned* __restrict__ start,
                 const unsigned* __restrict__ total, unsigned R, double2* __restrict__ mean, float2* __restrict__ shifts,
                 float4* __restrict__ params)
{
    const unsigned r = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5), lane = threadIdx.x & 31u;
    if (r >= R)
        return;
    const unsigned k0 = start[r], m = total[r];
    double ax = 0.0, ay = 0.0;
    for (unsigned k = lane; k < m; k += 32) {
        const AvgMember b = rec[order[k0 + k]];
        ax += b.mirror ? -(double)b.sx : (double)b.sx;
        ay += (double)b.sy;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        ax += __shfl_xor_sync(0xffffffffu, ax, o);
        ay += __shfl_xor_sync(0xffffffffu, ay, o);
    }
    const double mx = m ? (double)(float)ax / (double)m : 0.0;
    const double my = m ? (double)(float)ay / (double)m : 0.0;
    if (lane == 0) {
        mean[r] = make_double2(mx, my);
        if (shifts)
            shifts[r] = make_float2((float)mx, (float)my);
    }
    if (params)
        for (unsigned k = lane; k < m; k += 32) {
            const AvgMember b = rec[order[k0 + k]];
            const double sx = b.mirror ? (double)b.sx + mx : (double)b.sx - mx;
            params[b.img] = make_float4(b.ang, (float)sx, (float)((double)b.sy - my), b.mirror ? 1.0f : 0.0f);
        }
}

struct AvgSumArgs {
    const float* imgs;
    const AvgMember* rec;
    const unsigned* order;
    const unsigned* start;
    const unsigned* total;
    const unsigned* pstart;
    float* partial;
    unsigned* err;
    unsigned P, R, D, G, piece;
    unsigned test_stall, wait_iters; // failure-path tests only (gpuisac_test_stall_ccf)
};

// The interpolated value of output pixel (ixs, iy) of one member: the source
// point from the rotation (float operations in the order of the restatement),
// the pixel itself outside [0, D)^2, then the six-point quadratic rule with
// periodic neighbours.  Indices stay in [0, D) for every input (a NaN or
// infinite source point fails the range test).
__device__ __forceinline__ float quadri_at(const float* __restrict__ src, int D, float xo, float yo)
{
    const float fx = floorf(xo), fy = floorf(yo);
    const int i = (int)fx, j = (int)fy;
    const float dx = xo - fx, dy = yo - fy;
    const int ip = i + 1 == D ? 0 : i + 1, im = i == 0 ? D - 1 : i - 1;
    const int jp = j + 1 == D ? 0 : j + 1, jm = j == 0 ? D - 1 : j - 1;
    const float f00 = src[j * D + i];
    const float c1 = src[j * D + ip] - f00;
    const float c2 = (c1 - f00 + src[j * D + im]) * 0.5f;
    const float c3 = src[jp * D + i] - f00;
    const float c4 = (c3 - f00 + src[jm * D + i]) * 0.5f;
    const float c5 = src[jp * D + ip] - f00 - c1 - c3;
    return f00 + dx * (c1 + (dx - 1.0f) * c2 + dy * c5) + dy * (c3 + (dy - 1.0f) * c4);
}

constexpr int kRowsPerThread = 16; // output rows per thread and pass

__device__ __forceinline__ void accumulate(float (&acc)[kRowsPerThread], const float* __restrict__ src,
                                           const AvgMember& b, unsigned ix, unsigned row0, unsigned G, unsigned D)
{
    const float h = (float)(D >> 1), Df = (float)D;
    const unsigned ixs = b.mirror ? (ix == 0 ? 0u : D - ix) : ix;
    const float x = __fsub_rn((float)ixs, __fadd_rn(h, b.sx));
    const float hy = __fadd_rn(h, b.sy);
    const float xc = __fmul_rn(x, b.c), xs = __fmul_rn(x, b.s);
#pragma unroll
    for (int p = 0; p < kRowsPerThread; p++) {
        const unsigned iy = row0 + (unsigned)p * G;
        if (iy < D) {
            const float y = __fsub_rn((float)iy, hy);
            float xo = __fadd_rn(__fsub_rn(xc, __fmul_rn(y, b.s)), h);
            float yo = __fadd_rn(__fadd_rn(xs, __fmul_rn(y, b.c)), h);
            if (!(xo >= 0.0f && xo < Df && yo >= 0.0f && yo < Df)) {
                xo = (float)ixs;
                yo = (float)iy;
            }
            acc[p] += quadri_at(src, (int)D, xo, yo);
        }
    }
}

// grid: an upper bound on the pieces; CTA t >= pieces returns.  Threads
// D x G: thread (ix, g) sums output rows row0 + g + p G, p < 16, of column ix,
// in passes of 16 G rows over the piece's members (one pass up to D = 128).
template <bool STAGED>
__global__ void __launch_bounds__(1024)
avg_sum_kernel(AvgSumArgs a)
{
    extern __shared__ __align__(16) float sbuf[];
    __shared__ uint64_t bars[2];
    __shared__ AvgMember mrec[2]; // the member whose image a buffer holds (written with the copy's issue)
    const unsigned t = blockIdx.x, R = a.R, D = a.D, G = a.G;
    const unsigned n_pieces = a.pstart[R];
    if (t >= n_pieces)
        return;
    // the group whose pieces hold t: the last r with pstart[r] <= t
    unsigned lo = 0, hi = R; // pstart[lo] <= t < pstart[hi]
    while (hi - lo > 1) {
        const unsigned mid = (lo + hi) >> 1;
        if (a.pstart[mid] <= t)
            lo = mid;
        else
            hi = mid;
    }
    const unsigned r = lo;
    const unsigned k0 = a.start[r] + (t - a.pstart[r]) * a.piece;
    const unsigned k1 = min(a.start[r] + a.total[r], k0 + a.piece);
    const unsigned tid = threadIdx.x, ix = tid % D, g = tid / D;
    const size_t npix = (size_t)D * D;
    const uint32_t bytes = (uint32_t)(npix * sizeof(float));
    const uint32_t wlim = wait_tries(a.wait_iters);
    auto issue = [&](unsigned k, unsigned buf) {
        if (a.test_stall)
            return; // failure-path test: no copy, a wait that runs out
        const AvgMember b = a.rec[a.order[k]];
        mrec[buf] = b; // published to the other threads by the arrive below (release) and their wait (acquire)
        if (GPUISAC_IN_BOUNDS(kChkAvgImg, b.img, a.P)) {
            mbar_expect_tx(&bars[buf], bytes);
            bulk_g2s(sbuf + buf * npix, a.imgs + (size_t)b.img * npix, bytes, &bars[buf]);
        } else {
            mbar_expect_tx(&bars[buf], 0);
        }
    };
    if (STAGED) {
        if (tid == 0) {
            mbar_init(&bars[0], 1);
            mbar_init(&bars[1], 1);
            mbar_fence_init();
        }
        __syncthreads();
    }
    unsigned u = 0; // members consumed: use u of buffer u & 1 completes phase (u >> 1) & 1
    for (unsigned row0 = 0; row0 < D; row0 += kRowsPerThread * G) {
        float acc[kRowsPerThread];
#pragma unroll
        for (int p = 0; p < kRowsPerThread; p++)
            acc[p] = 0.0f;
        if (STAGED) {
            if (tid == 0) {
                fence_proxy_async(); // the previous pass read both buffers
                issue(k0, u & 1u);
                if (k0 + 1 < k1)
                    issue(k0 + 1, (u + 1) & 1u);
            }
            for (unsigned k = k0; k < k1; k++, u++) {
                const unsigned buf = u & 1u;
                const bool ok = mbar_wait(&bars[buf], (u >> 1) & 1u, wlim);
                if (ok)
                    accumulate(acc, sbuf + buf * npix, mrec[buf], ix, row0 + g, G, D);
                if (__syncthreads_or(!ok)) {
                    if (tid == 0) {
                        atomicAdd(a.err + kErrWait, 1u);
                        // the copies still in flight land before the CTA leaves
                        if (!ok && !a.test_stall)
                            mbar_wait(&bars[buf], (u >> 1) & 1u, wlim);
                        if (k + 1 < k1 && !a.test_stall)
                            mbar_wait(&bars[buf ^ 1u], ((u + 1) >> 1) & 1u, wlim);
                    }
                    return;
                }
                if (tid == 0 && k + 2 < k1) {
                    fence_proxy_async();
                    issue(k + 2, buf);
                }
            }
        } else {
            for (unsigned k = k0; k < k1; k++) {
                const AvgMember b = a.rec[a.order[k]];
                if (GPUISAC_IN_BOUNDS(kChkAvgImg, b.img, a.P))
                    accumulate(acc, a.imgs + (size_t)b.img * npix, b, ix, row0 + g, G, D);
            }
        }
        float* out = a.partial + (size_t)t * npix;
#pragma unroll
        for (int p = 0; p < kRowsPerThread; p++) {
            const unsigned iy = row0 + g + (unsigned)p * G;
            if (iy < D && GPUISAC_IN_BOUNDS(kChkAvgPartial, (size_t)t * npix + (size_t)iy * D + ix,
                                            (size_t)n_pieces * npix))
                out[(size_t)iy * D + ix] = acc[p];
        }
    }
}

struct AvgFinishArgs {
    const float* partial;
    const unsigned* pstart;
    const unsigned* total;
    const double2* mean;
    const float2* tw; // e^(2 pi i j / D), j = 0..D-1
    float2* scratch;  // [R][2][D][H] when the spectra do not fit in shared memory
    float* avg;
    unsigned R, D;
    float fl, ff;
    int center;
};

// Per group: the sum of its pieces times float(1/members); then, when
// filtering or centring, the real DFT over rows (x) then columns (y), the
// spectrum times the filter 0.5 (tanh(k (r + fl)) - tanh(k (r - fl))),
// k = pi / (2 ff fl), r = |(kx, ky)| / D (ky > D/2 taken as ky - D; a step at fl
// when ff = 0), and the phase exp(-2 pi i (kx dx + ky dy) / D) with (dx, dy) =
// -mean shift, then the inverse DFT over columns and the real inverse over rows
// (the imaginary parts of the kx = 0 and D/2 terms dropped), divided by D^2.
// Memory (shared, or global scratch above side 160): the twiddles tw[D], then
// two spectra F, G of D rows of Hs = H | 1 entries (an odd row length keeps a
// warp's accesses down a column free of bank conflicts); the image and the
// result sit in G's space with row stride D + 1.  In every pass a warp's lanes
// run along the dimension its data is contiguous or oddly strided in, and all
// lanes of a warp read the same twiddle (at most two distinct); each thread
// computes two outputs that share their data loads.
__global__ void __launch_bounds__(kFinishThreads)
avg_finish_kernel(AvgFinishArgs a)
{
    extern __shared__ __align__(16) float2 fsm[];
    const unsigned r = blockIdx.x, D = a.D, H = D / 2 + 1, Hs = H | 1u, S = D + 1, tid = threadIdx.x;
    const size_t npix = (size_t)D * D, nspec = (size_t)D * Hs;
    float* out = a.avg + (size_t)r * npix;
    const unsigned m = a.total[r];
    if (m == 0) {
        for (size_t q = tid; q < npix; q += kFinishThreads)
            out[q] = 0.0f;
        return;
    }
    const float inv = __double2float_rn(1.0 / (double)m);
    const unsigned p0 = a.pstart[r], p1 = a.pstart[r + 1];
    auto piece_sum = [&](size_t q) {
        float s = 0.0f;
        for (unsigned p = p0; p < p1; p++)
            s += a.partial[(size_t)p * npix + q];
        return s * inv;
    };
    if (!(a.fl > 0.0f || a.center)) {
        for (size_t q = tid; q < npix; q += kFinishThreads)
            out[q] = piece_sum(q);
        return;
    }
    float2* tw = fsm;
    float2* F = a.scratch ? a.scratch + (size_t)r * 2 * nspec : fsm + D;
    float2* G = F + nspec;
    float* img = reinterpret_cast<float*>(G); // [D][S]
    for (size_t q = tid; q < npix; q += kFinishThreads)
        img[(q / D) * S + q % D] = piece_sum(q);
    for (unsigned j = tid; j < D; j += kFinishThreads)
        tw[j] = a.tw[j];
    __syncthreads();

    // rows: F[y][kx] = sum_x img[y][x] e^(-2 pi i kx x / D); lanes along y
    const unsigned Hh = (H + 1) / 2;
    for (unsigned e = tid; e < D * Hh; e += kFinishThreads) {
        const unsigned k1 = e / D, y = e % D, k2 = k1 + Hh;
        const bool two = k2 < H;
        const unsigned k2s = two ? k2 : 0u;
        const float* rowp = img + (size_t)y * S;
        float r1 = 0.0f, i1 = 0.0f, r2 = 0.0f, i2 = 0.0f;
        unsigned j1 = 0, j2 = 0;
        for (unsigned x = 0; x < D; x++) {
            const float v = rowp[x];
            const float2 w1 = tw[j1], w2 = tw[j2];
            r1 = fmaf(v, w1.x, r1);
            i1 = fmaf(-v, w1.y, i1);
            r2 = fmaf(v, w2.x, r2);
            i2 = fmaf(-v, w2.y, i2);
            j1 += k1;
            j1 = j1 >= D ? j1 - D : j1;
            j2 += k2s;
            j2 = j2 >= D ? j2 - D : j2;
        }
        F[(size_t)y * Hs + k1] = make_float2(r1, i1);
        if (two)
            F[(size_t)y * Hs + k2] = make_float2(r2, i2);
    }
    __syncthreads();

    // columns, filter and phase: G[ky][kx] = h ph sum_y F[y][kx] e^(-2 pi i ky y / D);
    // lanes along kx.  The phase exp(-2 pi i (kx dx + ky dy) / D) is
    // sincospi(kx px + ky py), px = -2 dx / D rounded to float once per group.
    const double2 mn = a.mean[r];
    const float px = a.center ? (float)(2.0 * mn.x / (double)D) : 0.0f;
    const float py = a.center ? (float)(2.0 * mn.y / (double)D) : 0.0f;
    const float kf = a.ff > 0.0f ? (float)(kPi / (2.0 * (double)a.ff * (double)a.fl)) : 0.0f;
    auto finish_term = [&](unsigned ky, unsigned kx, float re, float im) {
        const int kys = 2 * ky > D ? (int)ky - (int)D : (int)ky;
        float hf = 1.0f;
        if (a.fl > 0.0f) {
            const float fx = (float)kx / (float)D, fy = (float)kys / (float)D;
            const float rr = sqrtf(fx * fx + fy * fy);
            hf = a.ff > 0.0f ? 0.5f * (tanhf(kf * (rr + a.fl)) - tanhf(kf * (rr - a.fl)))
                             : (rr < a.fl ? 1.0f : (rr == a.fl ? 0.5f : 0.0f));
        }
        float ps = 0.0f, pc = 1.0f;
        if (a.center)
            sincospif(fmaf((float)kx, px, (float)kys * py), &ps, &pc);
        G[(size_t)ky * Hs + kx] = make_float2((re * pc - im * ps) * hf, (re * ps + im * pc) * hf);
    };
    const unsigned Dh = (D + 1) / 2;
    for (unsigned e = tid; e < Dh * H; e += kFinishThreads) {
        const unsigned k1 = e / H, kx = e % H, k2 = k1 + Dh;
        const bool two = k2 < D;
        const unsigned k2s = two ? k2 : 0u;
        float r1 = 0.0f, i1 = 0.0f, r2 = 0.0f, i2 = 0.0f;
        unsigned j1 = 0, j2 = 0;
        for (unsigned y = 0; y < D; y++) {
            const float2 v = F[(size_t)y * Hs + kx];
            const float2 w1 = tw[j1], w2 = tw[j2]; // (v.x + i v.y)(w.x - i w.y)
            r1 = fmaf(v.x, w1.x, fmaf(v.y, w1.y, r1));
            i1 = fmaf(v.y, w1.x, fmaf(-v.x, w1.y, i1));
            r2 = fmaf(v.x, w2.x, fmaf(v.y, w2.y, r2));
            i2 = fmaf(v.y, w2.x, fmaf(-v.x, w2.y, i2));
            j1 += k1;
            j1 = j1 >= D ? j1 - D : j1;
            j2 += k2s;
            j2 = j2 >= D ? j2 - D : j2;
        }
        finish_term(k1, kx, r1, i1);
        if (two)
            finish_term(k2, kx, r2, i2);
    }
    __syncthreads();

    // inverse columns: F[y][kx] = sum_ky G[ky][kx] e^(+2 pi i ky y / D); lanes along kx
    for (unsigned e = tid; e < Dh * H; e += kFinishThreads) {
        const unsigned y1 = e / H, kx = e % H, y2 = y1 + Dh;
        const bool two = y2 < D;
        const unsigned y2s = two ? y2 : 0u;
        float r1 = 0.0f, i1 = 0.0f, r2 = 0.0f, i2 = 0.0f;
        unsigned j1 = 0, j2 = 0;
        for (unsigned ky = 0; ky < D; ky++) {
            const float2 v = G[(size_t)ky * Hs + kx];
            const float2 w1 = tw[j1], w2 = tw[j2];
            r1 = fmaf(v.x, w1.x, fmaf(-v.y, w1.y, r1));
            i1 = fmaf(v.y, w1.x, fmaf(v.x, w1.y, i1));
            r2 = fmaf(v.x, w2.x, fmaf(-v.y, w2.y, r2));
            i2 = fmaf(v.y, w2.x, fmaf(v.x, w2.y, i2));
            j1 += y1;
            j1 = j1 >= D ? j1 - D : j1;
            j2 += y2s;
            j2 = j2 >= D ? j2 - D : j2;
        }
        F[(size_t)y1 * Hs + kx] = make_float2(r1, i1);
        if (two)
            F[(size_t)y2 * Hs + kx] = make_float2(r2, i2);
    }
    __syncthreads();

    // inverse rows, half spectrum to real, into G's space; lanes along y
    float* res = img;
    const float scale = 1.0f / (float)npix;
    const unsigned K = (D - 1) / 2;
    for (unsigned e = tid; e < D * Dh; e += kFinishThreads) {
        const unsigned x1 = e / D, y = e % D, x2 = x1 + Dh;
        const bool two = x2 < D;
        const unsigned x2s = two ? x2 : 0u;
        const float2* fr = F + (size_t)y * Hs;
        float s1 = 0.0f, s2 = 0.0f;
        unsigned j1 = x1, j2 = x2s;
        for (unsigned kx = 1; kx <= K; kx++) {
            const float2 v = fr[kx];
            const float2 w1 = tw[j1], w2 = tw[j2];
            s1 = fmaf(v.x, w1.x, fmaf(-v.y, w1.y, s1));
            s2 = fmaf(v.x, w2.x, fmaf(-v.y, w2.y, s2));
            j1 += x1;
            j1 = j1 >= D ? j1 - D : j1;
            j2 += x2s;
            j2 = j2 >= D ? j2 - D : j2;
        }
        const float nyq = (D & 1u) == 0 ? fr[D / 2].x : 0.0f;
        res[(size_t)y * S + x1] = (fr[0].x + 2.0f * s1 + ((x1 & 1u) ? -nyq : nyq)) * scale;
        if (two)
            res[(size_t)y * S + x2] = (fr[0].x + 2.0f * s2 + ((x2 & 1u) ? -nyq : nyq)) * scale;
    }
    __syncthreads();
    for (size_t q = tid; q < npix; q += kFinishThreads)
        if (GPUISAC_IN_BOUNDS(kChkAvgOut, (size_t)r * npix + q, (size_t)a.R * npix))
            out[q] = res[(q / D) * S + q % D];
}

template <typename T>
struct Buf {
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
};

struct AvgState {
    std::mutex mu;
    int dev = -1;
    Buf<unsigned> cnt, total, start, pstart, err;
    Buf<AvgMember> rec;
    Buf<unsigned> order;
    Buf<double2> mean;
    Buf<float> partial;
    Buf<float2> scratch, tw;
    unsigned tw_dim = 0;
    unsigned* h_err = nullptr; // pinned
} g_avg;

int fail(int code, const char* msg)
{
    record_error(code, msg);
    return code;
}

#define AV_CK(expr)                                                                                    \
    do {                                                                                               \
        cudaError_t e_ = (expr);                                                                       \
        if (e_ != cudaSuccess) {                                                                       \
            char m_[384];                                                                              \
            snprintf(m_, sizeof(m_), "%s (%s) in the class averages", cudaGetErrorString(e_), #expr); \
            return fail(1, m_);                                                                        \
        }                                                                                              \
    } while (0)

// threads D x G: G = ceil(D / 16) (one pass) up to D = 128, else as many
// rows per pass as 1024 threads give
unsigned sum_groups(unsigned D) { return D <= 128 ? (D + kRowsPerThread - 1) / kRowsPerThread : 1024 / D; }

void release(AvgState& w)
{
    if (w.dev < 0)
        return;
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(w.dev);
    cudaFree(w.cnt.p), cudaFree(w.total.p), cudaFree(w.start.p), cudaFree(w.pstart.p), cudaFree(w.err.p);
    cudaFree(w.rec.p), cudaFree(w.order.p), cudaFree(w.mean.p), cudaFree(w.partial.p), cudaFree(w.scratch.p), cudaFree(w.tw.p);
    cudaSetDevice(cur);
    w.cnt = {}, w.total = {}, w.start = {}, w.pstart = {}, w.err = {}, w.rec = {}, w.order = {}, w.mean = {}, w.partial = {};
    w.scratch = {}, w.tw = {};
    w.tw_dim = 0;
}

} // namespace

GPUISAC_CHECKED_READER(checked_read_averages)

void averages_clear()
{
    std::lock_guard<std::mutex> lk(g_avg.mu);
    release(g_avg);
    g_avg.dev = -1;
    if (g_avg.h_err)
        cudaFreeHost(g_avg.h_err);
    g_avg.h_err = nullptr;
}

} // namespace gpuisac

using namespace gpuisac;

extern "C" int gpuisac_class_averages(const float* imgs, unsigned int n_img, unsigned int img_dim, const float* peaks,
                                      unsigned long long peak_pitch, const int* belongsto, unsigned int n_class,
                                      float fl, float ff, int center, float* averages, float* params, int* members,
                                      float* shifts, void* stream_)
{
    const gpuisac::NvtxRange nvtx_range("gpuisac:class_averages");
    if (!imgs || !peaks || !belongsto || !averages)
        return fail(2, "class_averages: NULL imgs, peaks, belongsto or averages");
    if (n_img == 0 || n_class == 0)
        return fail(2, "class_averages: needs n_img >= 1 and n_class >= 1");
    if (img_dim < 2 || img_dim > kMaxDim)
        return fail(2, "class_averages: img_dim outside 2..256");
    if (peak_pitch == 0)
        peak_pitch = n_img;
    if (peak_pitch < n_img)
        return fail(2, "class_averages: peak_pitch smaller than n_img");
    if ((uintptr_t)peaks % 16 != 0)
        return fail(2, "class_averages: peaks not 16-byte aligned");
    if (!(fl <= 0.5f) || !(ff >= 0.0f && ff <= 0.5f))
        return fail(2, "class_averages: needs fl <= 0.5 and 0 <= ff <= 0.5");
    if ((params && (uintptr_t)params % 16 != 0) || (shifts && (uintptr_t)shifts % 8 != 0))
        return fail(2, "class_averages: params not 16-byte or shifts not 8-byte aligned");
    cudaStream_t st = static_cast<cudaStream_t>(stream_);
    std::lock_guard<std::mutex> lk(g_avg.mu);
    AvgState& w = g_avg;
    int dev = 0;
    AV_CK(cudaGetDevice(&dev));
    if (w.dev != dev) { // buffers of another device are not reused
        release(w);
        w.dev = dev;
    }
    const unsigned D = img_dim, R = n_class, P = n_img;
    const size_t npix = (size_t)D * D;
    const unsigned n_chunks = (P + kAvgChunk - 1) / kAvgChunk;
    // member images staged by bulk copies: whole rows of 16-byte multiples
    const bool staged = D % 2 == 0 && D <= kStagedMaxDim && (uintptr_t)imgs % 16 == 0;
    void (*sum_kernel)(AvgSumArgs) = staged ? avg_sum_kernel<true> : avg_sum_kernel<false>;
    const unsigned G = sum_groups(D), sum_threads = D * G;
    const size_t sum_smem = staged ? 2 * sizeof(float) * npix : 0;
    int sms = 0, per_sm = 0;
    AV_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    if (sum_smem > 48 * 1024)
        AV_CK(cudaFuncSetAttribute(sum_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sum_smem));
    AV_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sum_kernel, (int)sum_threads, sum_smem));
    // pieces of about P / (4 waves of resident CTAs) members, 8..256
    const unsigned resident = (unsigned)std::max(1, sms * std::max(per_sm, 1));
    const unsigned piece = std::min(256u, std::max(8u, (P + 4 * resident - 1) / (4 * resident)));
    const size_t pieces_cap = (size_t)P / piece + R + 1;
    const bool fin_smem = D <= kFinishSmemDim;
    const size_t nspec = (size_t)D * ((D / 2 + 1) | 1u);
    const size_t fin_smem_bytes = sizeof(float2) * (D + (fin_smem ? 2 * nspec : 0));

    AV_CK(w.cnt.ensure((size_t)n_chunks * R));
    AV_CK(w.total.ensure(R));
    AV_CK(w.start.ensure(R));
    AV_CK(w.pstart.ensure((size_t)R + 1));
    AV_CK(w.err.ensure(kErrWords));
    AV_CK(w.rec.ensure(P));
    AV_CK(w.order.ensure(P));
    AV_CK(w.mean.ensure(R));
    AV_CK(w.partial.ensure(pieces_cap * npix));
    if (!fin_smem)
        AV_CK(w.scratch.ensure((size_t)R * 2 * nspec));
    if (!w.h_err)
        AV_CK(cudaMallocHost(&w.h_err, kErrWords * sizeof(unsigned)));
    if (w.tw_dim != D) {
        std::vector<float2> tw(D);
        for (unsigned j = 0; j < D; j++)
            tw[j] = make_float2((float)cos(2.0 * kPi * j / D), (float)sin(2.0 * kPi * j / D));
        AV_CK(w.tw.ensure(D));
        AV_CK(cudaMemcpy(w.tw.p, tw.data(), D * sizeof(float2), cudaMemcpyHostToDevice));
        w.tw_dim = D;
    }

    AV_CK(cudaMemsetAsync(w.cnt.p, 0, (size_t)n_chunks * R * sizeof(unsigned), st));
    AV_CK(cudaMemsetAsync(w.err.p, 0, kErrWords * sizeof(unsigned), st));
    AV_CK(cudaMemsetAsync(w.err.p + kErrBadFirst, 0xff, sizeof(unsigned), st));
    AV_CK(cudaMemsetAsync(w.err.p + kErrEmptyFirst, 0xff, sizeof(unsigned), st));
    avg_count_kernel<<<n_chunks, 256, 0, st>>>(belongsto, P, R, w.cnt.p, w.err.p);
    avg_chunk_scan_kernel<<<(R + 255) / 256, 256, 0, st>>>(w.cnt.p, n_chunks, R, w.total.p);
    avg_group_scan_kernel<<<1, 1024, 0, st>>>(w.total.p, R, piece, w.start.p, w.pstart.p, members, w.err.p);
    const size_t scat_smem = R <= kSmemGroups ? (size_t)R * sizeof(unsigned) : 0;
    if (scat_smem > 48 * 1024)
        AV_CK(cudaFuncSetAttribute(avg_scatter_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)scat_smem));
    avg_convert_kernel<<<(P + 255) / 256, 256, 0, st>>>(belongsto, P, R, reinterpret_cast<const float4*>(peaks),
                                                        peak_pitch, w.rec.p);
    avg_scatter_kernel<<<n_chunks, 32, scat_smem, st>>>(belongsto, P, R, w.cnt.p, w.start.p, w.order.p);
    avg_shift_kernel<<<(R + 7) / 8, 256, 0, st>>>(w.rec.p, w.order.p, w.start.p, w.total.p, R, w.mean.p,
                                                  reinterpret_cast<float2*>(shifts), reinterpret_cast<float4*>(params));
    AvgSumArgs sa{imgs, w.rec.p, w.order.p, w.start.p, w.total.p, w.pstart.p, w.partial.p, w.err.p, P, R, D, G, piece,
                  0, 0};
    ccf_test_settings(sa.test_stall, sa.wait_iters);
    sum_kernel<<<(unsigned)pieces_cap, sum_threads, sum_smem, st>>>(sa);
    AvgFinishArgs fa{w.partial.p, w.pstart.p, w.total.p, w.mean.p, w.tw.p, fin_smem ? nullptr : w.scratch.p,
                     averages, R, D, fl, ff, center};
    if (fin_smem_bytes > 48 * 1024)
        AV_CK(cudaFuncSetAttribute(avg_finish_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)fin_smem_bytes));
    avg_finish_kernel<<<R, kFinishThreads, fin_smem_bytes, st>>>(fa);
    g_kernel_launches.fetch_add(8, std::memory_order_relaxed);
    AV_CK(cudaGetLastError());
    AV_CK(cudaMemcpyAsync(w.h_err, w.err.p, kErrWords * sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    AV_CK(cudaStreamSynchronize(st));
    char msg[256];
    if (w.h_err[kErrBad]) {
        snprintf(msg, sizeof(msg), "class_averages: %u belongsto entries outside [0, %u), the first at particle %u",
                 w.h_err[kErrBad], R, w.h_err[kErrBadFirst]);
        return fail(2, msg);
    }
    if (w.h_err[kErrWait])
        return fail(1, "class_averages: an image copy timed out (bounded wait ran out)");
    if (w.h_err[kErrEmpty]) {
        snprintf(msg, sizeof(msg), "class_averages: %u groups have no members, the first is group %u",
                 w.h_err[kErrEmpty], w.h_err[kErrEmptyFirst]);
        return fail(2, msg);
    }
    return 0;
}
