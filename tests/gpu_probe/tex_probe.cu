// tex_probe.cu -- test helper: samples a float image through a 2D texture set
// up the way the reference sets up its image stacks (pitched linear memory,
// linear filter, clamp addressing, unnormalised coordinates;
// cuda/gpu_aln_noref.cu:2314-2339), so the oracle's emulation of the texture
// unit's filter weights can be compared with the hardware.  Test only.
#include <cuda_runtime.h>
#include <string.h>

__global__ void probe_kernel(cudaTextureObject_t tex, const float2* xy, int n, float* out)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        out[i] = tex2D<float>(tex, xy[i].x, xy[i].y);
}

extern "C" int tex_probe(const float* h_img, int w, int h, const float* h_xy, int n, float* h_out)
{
    float* d_img = nullptr;
    size_t pitch = 0;
    float2* d_xy = nullptr;
    float* d_out = nullptr;
    cudaTextureObject_t tex = 0;
    int rc = 0;
    if (cudaMallocPitch(&d_img, &pitch, w * sizeof(float), h) != cudaSuccess) return 1;
    if (cudaMemcpy2D(d_img, pitch, h_img, w * sizeof(float), w * sizeof(float), h, cudaMemcpyHostToDevice) != cudaSuccess) rc = 2;
    cudaResourceDesc res;
    memset(&res, 0, sizeof(res));
    res.resType = cudaResourceTypePitch2D;
    res.res.pitch2D.desc = cudaCreateChannelDesc<float>();
    res.res.pitch2D.devPtr = d_img;
    res.res.pitch2D.width = w;
    res.res.pitch2D.height = h;
    res.res.pitch2D.pitchInBytes = pitch;
    cudaTextureDesc td;
    memset(&td, 0, sizeof(td));
    td.addressMode[0] = cudaAddressModeClamp;
    td.addressMode[1] = cudaAddressModeClamp;
    td.filterMode = cudaFilterModeLinear;
    td.readMode = cudaReadModeElementType;
    td.normalizedCoords = 0;
    if (!rc && cudaCreateTextureObject(&tex, &res, &td, nullptr) != cudaSuccess) rc = 3;
    if (!rc && cudaMalloc(&d_xy, n * sizeof(float2)) != cudaSuccess) rc = 4;
    if (!rc && cudaMalloc(&d_out, n * sizeof(float)) != cudaSuccess) rc = 5;
    if (!rc && cudaMemcpy(d_xy, h_xy, n * sizeof(float2), cudaMemcpyHostToDevice) != cudaSuccess) rc = 6;
    if (!rc) {
        probe_kernel<<<(n + 255) / 256, 256>>>(tex, d_xy, n, d_out);
        if (cudaGetLastError() != cudaSuccess) rc = 7;
    }
    if (!rc && cudaMemcpy(h_out, d_out, n * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess) rc = 8;
    if (tex) cudaDestroyTextureObject(tex);
    cudaFree(d_xy);
    cudaFree(d_out);
    cudaFree(d_img);
    return rc;
}
