// normalize.cu -- the masked normalisation ISAC applies to every image before
// each alignment call (bin/sp_isac2_gpu.py:925-931, the "normalize.mask"
// processor of the un-vendored EMAN2 library: references with no_sigma = 1,
// particles with no_sigma = 0), batched over a device stack, in place.
//
// Per image: mean and standard deviation of the pixels where mask > 0.5
// (population deviation, sums in FP64), then every pixel of the image
// x <- (x - mean) / sigma, or x <- x - mean when no_sigma is set or the
// masked pixels have no spread.  One CTA per image: the image and the mask
// are read once for the sums and the image once more for the update (an
// image is 23 KB at 76^2, so the second read is an L2 hit).
#include <cuda_runtime.h>

#include "../../include/gpu_aln_pack.h"
#include "gpuisac_kernels.h"
#include "host_geometry.h"

using namespace gpuisac;

namespace {

constexpr int kNormThreads = 256;

__global__ void __launch_bounds__(kNormThreads)
normalize_mask_kernel(float* __restrict__ imgs, size_t pixels, const float* __restrict__ mask, int no_sigma)
{
    __shared__ double red[3][kNormThreads / 32];
    float* img = imgs + (size_t)blockIdx.x * pixels;
    double s1 = 0.0, s2 = 0.0, cnt = 0.0;
    const float4* i4 = reinterpret_cast<const float4*>(img);
    const float4* m4 = reinterpret_cast<const float4*>(mask);
    const bool vec = (pixels % 4) == 0 && ((uintptr_t)img % 16) == 0 && ((uintptr_t)mask % 16) == 0;
    auto add = [&](float x, float m) {
        if (m > 0.5f) {
            s1 += x;
            s2 += (double)x * x;
            cnt += 1.0;
        }
    };
    if (vec) {
        for (size_t i = threadIdx.x; i < pixels / 4; i += kNormThreads) {
            const float4 x = i4[i], m = __ldg(m4 + i);
            add(x.x, m.x);
            add(x.y, m.y);
            add(x.z, m.z);
            add(x.w, m.w);
        }
    } else {
        for (size_t i = threadIdx.x; i < pixels; i += kNormThreads)
            add(img[i], __ldg(mask + i));
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        s1 += __shfl_xor_sync(0xffffffffu, s1, off);
        s2 += __shfl_xor_sync(0xffffffffu, s2, off);
        cnt += __shfl_xor_sync(0xffffffffu, cnt, off);
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
        red[0][warp] = s1;
        red[1][warp] = s2;
        red[2][warp] = cnt;
    }
    __syncthreads();
    double a = 0.0, b = 0.0, n = 0.0;
    for (int w = 0; w < kNormThreads / 32; w++) {
        a += red[0][w];
        b += red[1][w];
        n += red[2][w];
    }
    const double mean = n > 0.0 ? a / n : 0.0;
    const double var = n > 0.0 ? b / n - mean * mean : 0.0;
    const double sd = var > 0.0 ? sqrt(var) : 0.0;
    const float meanf = (float)mean;
    const float inv = (!no_sigma && sd > 0.0) ? (float)(1.0 / sd) : 1.0f;
    if (vec) {
        float4* o4 = reinterpret_cast<float4*>(img);
        for (size_t i = threadIdx.x; i < pixels / 4; i += kNormThreads) {
            float4 x = o4[i];
            x.x = (x.x - meanf) * inv;
            x.y = (x.y - meanf) * inv;
            x.z = (x.z - meanf) * inv;
            x.w = (x.w - meanf) * inv;
            o4[i] = x;
        }
    } else {
        for (size_t i = threadIdx.x; i < pixels; i += kNormThreads)
            img[i] = (img[i] - meanf) * inv;
    }
}

} // namespace

extern "C" int gpuisac_normalize_mask(float* imgs, unsigned int n_img, unsigned int img_dim, const float* mask,
                                      int no_sigma, void* stream)
{
    const gpuisac::NvtxRange nvtx_range("gpuisac:normalize_mask");
    if (n_img == 0)
        return 0;
    if (!imgs || !mask || img_dim == 0 || img_dim > 4096) {
        record_error(2, "gpuisac_normalize_mask: NULL pointer or img_dim outside 1..4096");
        return 2;
    }
    normalize_mask_kernel<<<n_img, kNormThreads, 0, static_cast<cudaStream_t>(stream)>>>(
        imgs, (size_t)img_dim * img_dim, mask, no_sigma);
    g_kernel_launches.fetch_add(1, std::memory_order_relaxed);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        record_error(1, cudaGetErrorString(e));
        return 1;
    }
    return 0;
}
