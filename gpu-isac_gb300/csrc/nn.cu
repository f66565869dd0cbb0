// nn.cu -- kernels of the learned reference proposal: rotation-invariant
// features from ring spectra, and the forward / backward / update steps of a
// small embedding network (dense layers, ReLU, row L2 normalisation, softmax
// cross-entropy over reference scores, Adam) plus per-row top-k.
//
// The network has no counterpart in the reference; it only decides which
// references the exhaustive search visits first.  All buffers are row-major
// FP32 device arrays owned by the caller; every entry point is asynchronous on
// the given stream.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "../../include/gpu_aln_pack.h"
#include "gpuisac_kernels.h"

namespace gpuisac {
namespace {

// ---------------------------------------------------------------- features
// feat[i][r*nk + k] = log(1 + |F_r[k]|) for k < nk (k = 0 from slot 0's F[0]),
// then the whole row scaled to unit L2 norm, then (when given) standardised
// per column, (v - mu[f]) * inv_sd[f].  Magnitudes of ring spectra do not
// change when the image turns (a circular shift of every ring) or is mirrored
// (conjugate spectra).
__global__ void features_kernel(const float2* __restrict__ sp, unsigned n, unsigned ring_num, unsigned nk,
                                const float* __restrict__ mu, const float* __restrict__ inv_sd,
                                float* __restrict__ feat)
{
    const unsigned i = blockIdx.x;
    if (i >= n)
        return;
    const unsigned nf = ring_num * nk;
    const float2* row = sp + (size_t)i * ring_num * kSlots;
    float* out = feat + (size_t)i * nf;
    float ss = 0.f;
    for (unsigned f = threadIdx.x; f < nf; f += blockDim.x) {
        const unsigned r = f / nk, k = f - r * nk;
        const float2 ab = row[r * kSlots + k];
        // stored basis (Re+Im, Re-Im); slot 0 holds (F[0], F[128])
        float re = 0.5f * (ab.x + ab.y), im = 0.5f * (ab.x - ab.y);
        if (k == 0)
            im = 0.f;
        const float v = log1pf(sqrtf(re * re + im * im));
        out[f] = v;
        ss += v * v;
    }
    __shared__ float red[32];
    for (int o = 16; o > 0; o >>= 1)
        ss += __shfl_xor_sync(0xffffffffu, ss, o);
    if ((threadIdx.x & 31) == 0)
        red[threadIdx.x >> 5] = ss;
    __syncthreads();
    if (threadIdx.x < 32) {
        float t = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.f;
        for (int o = 16; o > 0; o >>= 1)
            t += __shfl_xor_sync(0xffffffffu, t, o);
        if (threadIdx.x == 0)
            red[0] = t;
    }
    __syncthreads();
    const float inv = rsqrtf(fmaxf(red[0], 1e-30f));
    if (mu) {
        for (unsigned f = threadIdx.x; f < nf; f += blockDim.x)
            out[f] = (out[f] * inv - mu[f]) * inv_sd[f];
    } else {
        for (unsigned f = threadIdx.x; f < nf; f += blockDim.x)
            out[f] *= inv;
    }
}

// ---------------------------------------------------------------- column statistics
// acc[2j], acc[2j+1] += sum, sum of squares of column j over a chunk of rows
__global__ void col_stats_kernel(const float* __restrict__ X, long rows, int cols, long rows_per_chunk,
                                 double* __restrict__ acc)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= cols)
        return;
    const long r0 = (long)blockIdx.y * rows_per_chunk;
    const long r1 = min(rows, r0 + rows_per_chunk);
    double s = 0.0, ss = 0.0;
    for (long i = r0; i < r1; i++) {
        const double v = X[i * cols + j];
        s += v;
        ss += v * v;
    }
    atomicAdd(&acc[2 * j], s);
    atomicAdd(&acc[2 * j + 1], ss);
}

__global__ void col_stats_final_kernel(const double* __restrict__ acc, long rows, int cols, float eps,
                                       float* __restrict__ mean, float* __restrict__ inv_sd)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= cols)
        return;
    const double m = acc[2 * j] / (double)rows;
    const double var = fmax(acc[2 * j + 1] / (double)rows - m * m, 0.0);
    mean[j] = (float)m;
    inv_sd[j] = (float)(1.0 / sqrt(var + (double)eps));
}

// X[i][j] = (X[i][j] - mu[j]) * inv_sd[j]
__global__ void affine_cols_kernel(float* __restrict__ X, long rows, int cols, const float* __restrict__ mu,
                                   const float* __restrict__ inv_sd)
{
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= rows * cols)
        return;
    const int j = (int)(idx % cols);
    X[idx] = (X[idx] - mu[j]) * inv_sd[j];
}

// out[i][j] = max over s < group of G[i*group + s][j]
__global__ void group_max_kernel(const float* __restrict__ G, long n, int group, int cols, float* __restrict__ out)
{
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= n * cols)
        return;
    const long i = idx / cols;
    const int j = (int)(idx - i * cols);
    const float* g = G + (i * group) * cols + j;
    float m = g[0];
    for (int s = 1; s < group; s++)
        m = fmaxf(m, g[(long)s * cols]);
    out[idx] = m;
}

// ---------------------------------------------------------------- GEMM
// C[m][n] = alpha * sum_k A(m,k) B(k,n) + beta * C[m][n], with A(m,k) at
// A[m*sam + k*sak] and B(k,n) at B[k*sbk + n*sbn] (strides give transposes).
// 64x64 tile per CTA of 256 threads, 4x4 outputs per thread, K in steps of 16.
constexpr int TM = 64, TN = 64, TK = 16;

__global__ void __launch_bounds__(256) gemm_kernel(int M, int N, int K, float alpha, const float* __restrict__ A,
                                                   long sam, long sak, const float* __restrict__ B, long sbk,
                                                   long sbn, float beta, float* __restrict__ C, long ldc)
{
    __shared__ float As[TK][TM + 4];
    __shared__ float Bs[TK][TN + 4];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int m0 = blockIdx.y * TM, n0 = blockIdx.x * TN;
    float acc[4][4] = {};
    for (int k0 = 0; k0 < K; k0 += TK) {
        for (int e = threadIdx.x; e < TK * TM; e += 256) {
            const int kk = e / TM, mm = e - kk * TM;
            const int gm = m0 + mm, gk = k0 + kk;
            As[kk][mm] = (gm < M && gk < K) ? A[(long)gm * sam + (long)gk * sak] : 0.f;
        }
        for (int e = threadIdx.x; e < TK * TN; e += 256) {
            const int kk = e / TN, nn = e - kk * TN;
            const int gn = n0 + nn, gk = k0 + kk;
            Bs[kk][nn] = (gn < N && gk < K) ? B[(long)gk * sbk + (long)gn * sbn] : 0.f;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < TK; kk++) {
            float a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; i++) {
                a[i] = As[kk][ty * 4 + i];
                b[i] = Bs[kk][tx * 4 + i];
            }
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++)
                    acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const int gm = m0 + ty * 4 + i;
        if (gm >= M)
            continue;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int gn = n0 + tx * 4 + j;
            if (gn >= N)
                continue;
            float* c = C + (long)gm * ldc + gn;
            *c = alpha * acc[i][j] + (beta != 0.f ? beta * *c : 0.f);
        }
    }
}

// ---------------------------------------------------------------- elementwise
// Y[i][j] += b[j]; optionally ReLU
__global__ void bias_act_kernel(float* __restrict__ Y, const float* __restrict__ b, long rows, int cols, int relu)
{
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= rows * cols)
        return;
    float v = Y[idx] + b[idx % cols];
    Y[idx] = relu ? fmaxf(v, 0.f) : v;
}

// dY *= (Y > 0)
__global__ void relu_bwd_kernel(float* __restrict__ dY, const float* __restrict__ Y, long n)
{
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx < n && !(Y[idx] > 0.f))
        dY[idx] = 0.f;
}

// db[j] = sum_i dY[i][j] (added to db when accumulate)
__global__ void colsum_kernel(const float* __restrict__ dY, long rows, int cols, float* __restrict__ db,
                              int accumulate)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= cols)
        return;
    float s = 0.f;
    for (long i = 0; i < rows; i++)
        s += dY[i * cols + j];
    db[j] = accumulate ? db[j] + s : s;
}

// one warp per row: E = X / |X| (norm stored)
__global__ void l2norm_kernel(const float* __restrict__ X, long rows, int cols, float* __restrict__ E,
                              float* __restrict__ norm)
{
    const long r = (long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (r >= rows)
        return;
    float ss = 0.f;
    for (int j = lane; j < cols; j += 32) {
        const float v = X[r * cols + j];
        ss += v * v;
    }
    for (int o = 16; o > 0; o >>= 1)
        ss += __shfl_xor_sync(0xffffffffu, ss, o);
    const float nr = sqrtf(fmaxf(ss, 1e-24f));
    for (int j = lane; j < cols; j += 32)
        E[r * cols + j] = X[r * cols + j] / nr;
    if (lane == 0)
        norm[r] = nr;
}

// dX = (dE - E (E . dE)) / norm
__global__ void l2norm_bwd_kernel(const float* __restrict__ E, const float* __restrict__ dE,
                                  const float* __restrict__ norm, long rows, int cols, float* __restrict__ dX)
{
    const long r = (long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (r >= rows)
        return;
    float dot = 0.f;
    for (int j = lane; j < cols; j += 32)
        dot += E[r * cols + j] * dE[r * cols + j];
    for (int o = 16; o > 0; o >>= 1)
        dot += __shfl_xor_sync(0xffffffffu, dot, o);
    const float inv = 1.f / norm[r];
    for (int j = lane; j < cols; j += 32)
        dX[r * cols + j] = (dE[r * cols + j] - E[r * cols + j] * dot) * inv;
}

// one warp per row: softmax over the row's scores, cross-entropy against the
// label; dS = (softmax - onehot) / rows when dS is given
__global__ void softmax_xent_kernel(const float* __restrict__ S, const int* __restrict__ labels, long rows, int cols,
                                    float* __restrict__ loss, float* __restrict__ dS)
{
    const long r = (long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (r >= rows)
        return;
    const float* s = S + r * cols;
    float mx = -INFINITY;
    for (int j = lane; j < cols; j += 32)
        mx = fmaxf(mx, s[j]);
    for (int o = 16; o > 0; o >>= 1)
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    float se = 0.f;
    for (int j = lane; j < cols; j += 32)
        se += expf(s[j] - mx);
    for (int o = 16; o > 0; o >>= 1)
        se += __shfl_xor_sync(0xffffffffu, se, o);
    const int lab = labels[r];
    if (lane == 0)
        loss[r] = logf(se) + mx - s[lab];
    if (dS) {
        const float inv = 1.f / (se * (float)rows);
        for (int j = lane; j < cols; j += 32)
            dS[r * cols + j] = expf(s[j] - mx) * inv - (j == lab ? 1.f / (float)rows : 0.f);
    }
}

// AdamW step on n parameters (step counts from 1)
__global__ void adam_kernel(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, long n, float lr, float b1, float b2, float eps, float wd, float c1,
                            float c2)
{
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * ((mi / c1) / (sqrtf(vi / c2) + eps) + wd * p[i]);
}

// one warp per row: indices of the k largest scores, best first (ties: the
// smaller index); cols <= 1024, k <= 64
__global__ void topk_kernel(const float* __restrict__ S, long rows, int cols, int k, unsigned* __restrict__ idx)
{
    const long r = (long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (r >= rows)
        return;
    const float* s = S + r * cols;
    unsigned taken = 0; // bit t: column lane + 32 t already chosen
    for (int pick = 0; pick < k; pick++) {
        float bv = -INFINITY;
        int bj = 0x7fffffff;
        for (int t = 0; t < 32; t++) {
            const int j = lane + 32 * t;
            if (j >= cols)
                break;
            if (taken & (1u << t))
                continue;
            const float v = s[j];
            if (v > bv || (v == bv && j < bj) || bj == 0x7fffffff) {
                bv = v;
                bj = j;
            }
        }
        for (int o = 16; o > 0; o >>= 1) {
            const float ov = __shfl_xor_sync(0xffffffffu, bv, o);
            const int oj = __shfl_xor_sync(0xffffffffu, bj, o);
            if (oj != 0x7fffffff && (bj == 0x7fffffff || ov > bv || (ov == bv && oj < bj))) {
                bv = ov;
                bj = oj;
            }
        }
        if (bj == 0x7fffffff)
            bj = 0;
        if ((bj & 31) == lane)
            taken |= 1u << (bj >> 5);
        if (lane == 0)
            idx[r * k + pick] = (unsigned)bj;
    }
}

inline unsigned blocks(long n, int per) { return (unsigned)((n + per - 1) / per); }

} // namespace
} // namespace gpuisac

using namespace gpuisac;

// ============================================================ C-ABI
extern "C" {

int gpuisac_nn_features(const float* spectra, unsigned int n, unsigned int ring_num, unsigned int nk,
                        const float* mu, const float* inv_sd, float* feat, void* stream)
{
    if (!spectra || !feat || nk == 0 || nk > kSlots || ring_num == 0 || (!mu) != (!inv_sd))
        return 2;
    if (n == 0)
        return 0;
    features_kernel<<<n, 256, 0, (cudaStream_t)stream>>>(reinterpret_cast<const float2*>(spectra), n, ring_num, nk,
                                                          mu, inv_sd, feat);
    g_kernel_launches.fetch_add(1, std::memory_order_relaxed);
    return cudaGetLastError() == cudaSuccess ? 0 : 1;
}

int gpuisac_nn_gemm(int M, int N, int K, float alpha, const float* A, long sam, long sak, const float* B, long sbk,
                    long sbn, float beta, float* C, long ldc, void* stream)
{
    if (M < 0 || N < 0 || K < 0 || !A || !B || !C)
        return 2;
    if (M == 0 || N == 0)
        return 0;
    // grid.y is limited to 65535 tiles: long M runs in slabs
    const int slab = 65535 * TM;
    for (int m0 = 0; m0 < M; m0 += slab) {
        const int mm = M - m0 < slab ? M - m0 : slab;
        dim3 grid((N + TN - 1) / TN, (mm + TM - 1) / TM);
        gemm_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(mm, N, K, alpha, A + (long)m0 * sam, sam, sak, B, sbk,
                                                            sbn, beta, C + (long)m0 * ldc, ldc);
        g_kernel_launches.fetch_add(1, std::memory_order_relaxed);
    }
    return cudaGetLastError() == cudaSuccess ? 0 : 1;
}

int gpuisac_nn_bias_act(float* Y, const float* b, long rows, int cols, int relu, void* stream)
{
    if (!Y || !b || rows < 0 || cols <= 0)
        return 2;
    if (rows == 0)
        return 0;
    bias_act_kernel<<<blocks(rows * cols, 256), 256, 0, (cudaStream_t)stream>>>(Y, b, rows, cols, relu);
    g_kernel_launches.fetch_add(1, std::memory_order_relaxed);
    return cudaGetLastError() == cudaSuccess ? 0 : 1;
}

int gpuisac_nn_relu_backward(float* dY, const float* Y, long n, void* stream)
{
    if (!dY || !Y || n < 0)
        return 2;
    if (n == 0)
        return 0;
    relu_bwd_kernel<<<blocks(n, 256), 256, 0, (cudaStream_t)stream>>>(dY, Y, n);
    g_kernel_launches.fetch_add(1, std::memory_order_relaxed);
    return cudaGetLastError() == cudaSuccess ? 0 : 1;
}

int gpuisac_nn_colsum(const float* dY, long rows, int cols, float* db, int accumulate, void* stream)
{
    if (!dY || !db || rows < 0 || cols <= 0)
        return 2;
    colsum_kernel<<<blocks(cols, 128), 128, 0, (cudaStream_t)stream>>>(dY, rows, cols, db, accumulate);
    g_kernel_launches.fetch_add(1, std::memory_order_relaxed);
    return cudaGetLastError() == cudaSuccess ? 0 : 1;
}

int gpuisac_nn_l2norm(const float* X, long rows, int cols, float* E, float* norm, void* stream)
{
    if (!X || !E || !norm || rows < 0 || cols <= 0)
        return 2;
    if (rows == 0)
        return 0;
    l2norm_kernel<<<blocks(rows, 8), 256, 0, (cudaStream_t)stream>>>(X, rows, cols, E, norm);
    g_kernel_launches.fetch_add(1, std::memory_order_relaxed);
    return cudaGetLastError() == cudaSuccess ? 0 : 1;
}

int gpuisac_nn_l2norm_backward(const float* E, const float* dE, const float* norm, long rows, int cols, float* dX,
                               void* stream)
{
    if (!E || !dE || !norm || !dX || rows < 0 || cols <= 0)
        return 2;
    if (rows == 0)
        return 0;
    l2norm_bwd_kernel<<<blocks(rows, 8), 256, 0, (cudaStream_t)stream>>>(E, dE, norm, rows, cols, dX);
    g_kernel_launches.fetch_add(1, std::memory_order_relaxed);
    return cudaGetLastError() == cudaSuccess ? 0 : 1;
}

int gpuisac_nn_softmax_xent(const float* S, const int* labels, long rows, int cols, float* loss, float* dS,
                            void* stream)
{
    if (!S || !labels || !loss || rows < 0 || cols <= 0)
        return 2;
    if (rows == 0)
        return 0;
    softmax_xent_kernel<<<blocks(rows, 8), 256, 0, (cudaStream_t)stream>>>(S, labels, rows, cols, loss, dS);
    g_kernel_launches.fetch_add(1, std::memory_order_relaxed);
    return cudaGetLastError() == cudaSuccess ? 0 : 1;
}

int gpuisac_nn_adam(float* p, const float* g, float* m, float* v, long n, float lr, float b1, float b2, float eps,
                    float wd, int step, void* stream)
{
    if (!p || !g || !m || !v || n < 0 || step < 1)
        return 2;
    if (n == 0)
        return 0;
    const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
    adam_kernel<<<blocks(n, 256), 256, 0, (cudaStream_t)stream>>>(p, g, m, v, n, lr, b1, b2, eps, wd, c1, c2);
    g_kernel_launches.fetch_add(1, std::memory_order_relaxed);
    return cudaGetLastError() == cudaSuccess ? 0 : 1;
}

int gpuisac_nn_topk(const float* S, long rows, int cols, int k, unsigned int* idx, void* stream)
{
    if (!S || !idx || rows < 0 || cols <= 0 || cols > 1024 || k <= 0 || k > 64 || k > cols)
        return 2;
    if (rows == 0)
        return 0;
    topk_kernel<<<blocks(rows, 8), 256, 0, (cudaStream_t)stream>>>(S, rows, cols, k, idx);
    g_kernel_launches.fetch_add(1, std::memory_order_relaxed);
    return cudaGetLastError() == cudaSuccess ? 0 : 1;
}

int gpuisac_nn_col_stats(const float* X, long rows, int cols, float eps, float* mean, float* inv_sd, void* stream)
{
    if (!X || !mean || !inv_sd || rows <= 0 || cols <= 0)
        return 2;
    cudaStream_t st = (cudaStream_t)stream;
    double* acc = nullptr;
    if (cudaMallocAsync(&acc, 2 * (size_t)cols * sizeof(double), st) != cudaSuccess)
        return 1;
    cudaMemsetAsync(acc, 0, 2 * (size_t)cols * sizeof(double), st);
    const long chunk = 512;
    dim3 grid(blocks(cols, 128), (unsigned)((rows + chunk - 1) / chunk));
    col_stats_kernel<<<grid, 128, 0, st>>>(X, rows, cols, chunk, acc);
    col_stats_final_kernel<<<blocks(cols, 128), 128, 0, st>>>(acc, rows, cols, eps, mean, inv_sd);
    g_kernel_launches.fetch_add(2, std::memory_order_relaxed);
    cudaFreeAsync(acc, st);
    return cudaGetLastError() == cudaSuccess ? 0 : 1;
}

int gpuisac_nn_affine_cols(float* X, long rows, int cols, const float* mu, const float* inv_sd, void* stream)
{
    if (!X || !mu || !inv_sd || rows < 0 || cols <= 0)
        return 2;
    if (rows == 0)
        return 0;
    affine_cols_kernel<<<blocks(rows * cols, 256), 256, 0, (cudaStream_t)stream>>>(X, rows, cols, mu, inv_sd);
    g_kernel_launches.fetch_add(1, std::memory_order_relaxed);
    return cudaGetLastError() == cudaSuccess ? 0 : 1;
}

int gpuisac_nn_group_max(const float* G, long n, int group, int cols, float* out, void* stream)
{
    if (!G || !out || n < 0 || group <= 0 || cols <= 0)
        return 2;
    if (n == 0)
        return 0;
    group_max_kernel<<<blocks(n * cols, 256), 256, 0, (cudaStream_t)stream>>>(G, n, group, cols, out);
    g_kernel_launches.fetch_add(1, std::memory_order_relaxed);
    return cudaGetLastError() == cudaSuccess ? 0 : 1;
}

} // extern "C"
