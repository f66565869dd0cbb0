// gemm_tc.cu -- BF16 tensor-core GEMM of the proposal network's inference:
// C = alpha * A B^T (+ bias[n], ReLU), A [M][K] and B [N][K] FP32 row-major
// (both K-major), converted to BF16 while they are staged, FP32 accumulate in
// tensor memory, FP32 out.
//
// One CTA of 128 threads per 128 x 128 tile of C: for every 64-wide K slice
// the threads stage A's and B's slices in shared memory in the canonical
// no-swizzle K-major layout (8-row x 16-byte core matrices), one elected
// thread issues four tcgen05.mma (K = 16 each) and commits them to an
// mbarrier; the accumulator (128 lanes x 128 FP32 columns) is read back with
// tcgen05.ld for the epilogue.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/gpu_aln_pack.h"
#include "gpuisac_kernels.h"

namespace gpuisac {
namespace {

constexpr int kTM = 128, kTN = 128, kTK = 64;
constexpr uint32_t kTcCols = 128; // tensor-memory columns of the accumulator

__device__ __forceinline__ uint32_t saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// byte offset of element (row, k) of a [128][64] BF16 slice in the canonical
// no-swizzle K-major layout: core matrix (row/8, k/8) of 8 rows x 16 bytes,
// core matrices K-adjacent 128 bytes apart, row groups 1024 bytes apart
__device__ __forceinline__ uint32_t slice_offset(int row, int k)
{
    return (uint32_t)(((row >> 3) * 8 + (k >> 3)) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

// shared-memory matrix descriptor: start, leading (K) and stride (row-group)
// byte offsets in 16-byte units, the fixed version bits, no swizzle
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}

// instruction descriptor of kind::f16: F32 accumulator, BF16 A and B, both
// K-major, N = 128, M = 128
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kTN >> 3) << 17) |
                            ((uint32_t)(kTM >> 4) << 24);

__device__ __forceinline__ bool bar_try(uint64_t* bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(saddr(bar)), "r"(parity)
                 : "memory");
    return ok != 0;
}

__device__ __forceinline__ bool bar_wait(uint64_t* bar, uint32_t parity)
{
    for (uint32_t it = 0; it < (1u << 22); it++) {
        if (bar_try(bar, parity))
            return true;
        __nanosleep(it < 64 ? 0 : 256);
    }
    return false;
}

// stage rows [r0, r0+128) x k [k0, k0+64) of X [rows][K] (pitch ld) as BF16;
// rows / k beyond the matrix read zero
__device__ __forceinline__ void stage_slice(unsigned char* dst, const float* __restrict__ X, long rows, int K,
                                           long ld, long r0, int k0)
{
    for (int e = threadIdx.x; e < kTM * (kTK / 4); e += blockDim.x) {
        const int row = e / (kTK / 4), kq = e % (kTK / 4);
        const long gr = r0 + row;
        const int gk = k0 + 4 * kq;
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (gr < rows && gk < K)
            v = __ldg(reinterpret_cast<const float4*>(X + gr * ld + gk));
        __nv_bfloat162 lo = __floats2bfloat162_rn(v.x, v.y), hi = __floats2bfloat162_rn(v.z, v.w);
        uint2 packed;
        packed.x = *reinterpret_cast<uint32_t*>(&lo);
        packed.y = *reinterpret_cast<uint32_t*>(&hi);
        *reinterpret_cast<uint2*>(dst + slice_offset(row, 4 * kq)) = packed;
    }
}

__global__ void __launch_bounds__(128)
gemm_tc_kernel(int M, int N, int K, float alpha, const float* __restrict__ A, long lda, const float* __restrict__ B,
               long ldb, const float* __restrict__ bias, int relu, float* __restrict__ C, long ldc,
               unsigned* __restrict__ err)
{
    __shared__ __align__(1024) unsigned char sa[kTM * kTK * 2];
    __shared__ __align__(1024) unsigned char sb[kTN * kTK * 2];
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tmem_base;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const long m0 = (long)blockIdx.y * kTM, n0 = (long)blockIdx.x * kTN;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(&tmem_base)),
                     "r"(kTcCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(saddr(&bar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_base;

    uint32_t phase = 0;
    bool ok = true;
    for (int k0 = 0; k0 < K; k0 += kTK) {
        stage_slice(sa, A, M, K, lda, m0, k0);
        stage_slice(sb, B, N, K, ldb, n0, k0);
        // the generic-proxy writes above become visible to the tensor cores
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
            for (int j = 0; j < kTK / 16; j++) {
                const uint64_t da = smem_desc(saddr(sa) + j * 256, 128, 1024);
                const uint64_t db = smem_desc(saddr(sb) + j * 256, 128, 1024);
                const uint32_t acc = (k0 > 0 || j > 0) ? 1u : 0u;
                asm volatile("{\n\t.reg .pred p;\n\t"
                             "setp.ne.u32 p, %4, 0;\n\t"
                             "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
                             "l"(da), "l"(db), "r"(kIdesc), "r"(acc)
                             : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             saddr(&bar))
                         : "memory");
        }
        // the slices are read by the tensor cores until the commit lands
        ok = bar_wait(&bar, phase) && ok;
        phase ^= 1u;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        __syncthreads();
    }
    if (!ok && tid == 0)
        atomicExch(err, 1u);

    // epilogue: warp w holds rows 32w..32w+31 (lane = row), 16 columns per load
    const long row = m0 + warp * 32 + lane;
    const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll 1
    for (int c0 = 0; c0 < kTN; c0 += 16) {
        uint32_t r[16];
        asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, "
                     "%12, %13, %14, %15}, [%16];"
                     : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                       "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
                       "=r"(r[14]), "=r"(r[15])
                     : "r"(taddr + (uint32_t)c0)
                     : "memory");
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        if (row < M && K > 0) {
#pragma unroll
            for (int i = 0; i < 16; i++) {
                const long n = n0 + c0 + i;
                if (n < N) {
                    float v = alpha * __uint_as_float(r[i]);
                    if (bias)
                        v += bias[n];
                    if (relu)
                        v = fmaxf(v, 0.f);
                    C[row * ldc + n] = v;
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTcCols) : "memory");
}

} // namespace
} // namespace gpuisac

using namespace gpuisac;

extern "C" int gpuisac_nn_gemm_bf16(int M, int N, int K, float alpha, const float* A, long lda, const float* B,
                                    long ldb, const float* bias, int relu, float* C, long ldc, unsigned int* err,
                                    void* stream)
{
    if (M < 0 || N < 0 || K <= 0 || !A || !B || !C || !err)
        return 2;
    // staged with 16-byte loads: K, the pitches and the bases in whole float4s
    if ((K % 4) || (lda % 4) || (ldb % 4) || ((uintptr_t)A & 15) || ((uintptr_t)B & 15))
        return 2;
    if (M == 0 || N == 0)
        return 0;
    if ((M + kTM - 1) / kTM > 65535)
        return 2;
    dim3 grid((N + kTN - 1) / kTN, (M + kTM - 1) / kTM);
    gemm_tc_kernel<<<grid, 128, 0, (cudaStream_t)stream>>>(M, N, K, alpha, A, lda, B, ldb, bias, relu, C, ldc, err);
    g_kernel_launches.fetch_add(1, std::memory_order_relaxed);
    return cudaGetLastError() == cudaSuccess ? 0 : 1;
}
