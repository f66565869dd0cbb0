// tex_stack.cu -- image stacks laid out as the reference's textures hold
// them, for the hardware texture unit.
//
// The reference fetches images batch by batch into 2D pitched textures of
// `tex` images each (BatchHandler::fetch_data / create_texture_objects,
// cuda/gpu_aln_noref.cu:2001-2052, 2314-2339: linear filtering, clamped
// addressing, unnormalised coordinates); the textures are sized for a full
// batch, so the free slots of a short final batch still hold the previous
// batch's images.  TexStack builds one texture per (batch, texture) segment
// of a device stack, fills every slot -- stale slots included -- from the
// stack in one copy kernel, and hands the kernels a device array of texture
// objects indexed by TexPlacement::tex_id.  Sampling through it is the
// filtering the reference's own samples get; the emulation in tex_sample
// (gpuisac_device.cuh) remains for callers without a texture set.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>

#include "gpuisac_kernels.h"

namespace gpuisac {
namespace {

// One warp per destination row (8 per block): row r of the whole layout is
// batch b = r / (batch*dim), texture t, slot j, image row y; the slot's image
// is b*batch + t*tex + j, or the previous batch's image in that slot past n.
__global__ void __launch_bounds__(256)
tex_fill_kernel(const float* __restrict__ src, unsigned n, unsigned dim, unsigned batch, unsigned tex,
                size_t full_bytes, size_t batch_bytes, size_t pitch, size_t rows, unsigned char* __restrict__ mem)
{
    const size_t r = (size_t)blockIdx.x * 8 + (threadIdx.x >> 5);
    if (r >= rows)
        return;
    const size_t per_batch = (size_t)batch * dim;
    const unsigned b = (unsigned)(r / per_batch);
    const unsigned rb = (unsigned)(r - (size_t)b * per_batch);
    const unsigned t = rb / (tex * dim);
    const unsigned in_seg = rb - t * tex * dim;
    const unsigned j = in_seg / dim, y = in_seg - j * dim;
    unsigned g = b * batch + t * tex + j;
    if (g >= n)
        g -= batch;
    float* dst = reinterpret_cast<float*>(mem + (size_t)b * batch_bytes + (size_t)t * full_bytes + (size_t)in_seg * pitch);
    const float* s = src + ((size_t)g * dim + y) * dim;
    for (unsigned x = threadIdx.x & 31; x < dim; x += 32)
        dst[x] = s[x];
}

size_t round_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

} // namespace

bool texture_unit_enabled()
{
    const char* e = std::getenv("GPUISAC_TEXTURE");
    return !(e && e[0] == '0');
}

void TexStack::destroy_objects()
{
    for (unsigned long long o : objs)
        cudaDestroyTextureObject((cudaTextureObject_t)o);
    objs.clear();
}

void TexStack::release()
{
    destroy_objects();
    if (mem)
        cudaFree(mem);
    if (d_objs)
        cudaFree(d_objs);
    mem = nullptr;
    d_objs = nullptr;
    mem_bytes = 0;
    d_objs_n = 0;
    n = dim = batch = tex = 0;
}

const unsigned long long* TexStack::try_build(const StackDesc& st, cudaStream_t stream)
{
    if (build(st, stream) == cudaSuccess)
        return d_objs;
    (void)cudaGetLastError(); // allocation and launch-configuration errors are not sticky
    release();
    return nullptr;
}

cudaError_t TexStack::build(const StackDesc& st, cudaStream_t stream)
{
    cudaError_t e = prepare(st);
    return e != cudaSuccess ? e : fill(st, stream);
}

cudaError_t TexStack::prepare(const StackDesc& st)
{
    if (st.n == 0 || st.dim == 0 || st.batch == 0 || st.tex == 0 || st.batch > st.n)
        return cudaErrorInvalidValue;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return e;
    int tex_align = 512, pitch_align = 32;
    cudaDeviceGetAttribute(&tex_align, cudaDevAttrTextureAlignment, dev);
    cudaDeviceGetAttribute(&pitch_align, cudaDevAttrTexturePitchAlignment, dev);
    const unsigned D = st.dim;
    const size_t pitch = round_up((size_t)D * sizeof(float), (size_t)std::max(pitch_align, 4));
    const unsigned ntpb = (st.batch + st.tex - 1) / st.tex;     // textures per batch
    const unsigned nb = (st.n + st.batch - 1) / st.batch;        // batches
    const unsigned last_alloc = st.batch - (ntpb - 1) * st.tex;  // images of a batch's last texture
    const size_t full_bytes = round_up((size_t)st.tex * D * pitch, (size_t)tex_align);
    const size_t last_bytes = round_up((size_t)last_alloc * D * pitch, (size_t)tex_align);
    const size_t batch_bytes = (size_t)(ntpb - 1) * full_bytes + last_bytes;
    const size_t need = (size_t)nb * batch_bytes;

    const bool same_layout = mem && need <= mem_bytes && dim == D && batch == st.batch && tex == st.tex &&
                             n == st.n && pitch_ == pitch && device == dev;
    if (!same_layout) {
        destroy_objects();
        if (need > mem_bytes) {
            if (mem)
                cudaFree(mem);
            mem = nullptr;
            mem_bytes = 0;
            e = cudaMalloc(&mem, need);
            if (e != cudaSuccess)
                return e;
            mem_bytes = need;
        }
        const unsigned n_seg = nb * ntpb;
        objs.resize(n_seg);
        for (unsigned b = 0; b < nb; b++)
            for (unsigned t = 0; t < ntpb; t++) {
                const unsigned alloc = (t != ntpb - 1) ? st.tex : last_alloc;
                cudaResourceDesc rd{};
                rd.resType = cudaResourceTypePitch2D;
                rd.res.pitch2D.devPtr = mem + (size_t)b * batch_bytes + (size_t)t * full_bytes;
                rd.res.pitch2D.desc = cudaCreateChannelDesc<float>();
                rd.res.pitch2D.width = D;
                rd.res.pitch2D.height = (size_t)alloc * D;
                rd.res.pitch2D.pitchInBytes = pitch;
                cudaTextureDesc td{};
                td.addressMode[0] = cudaAddressModeClamp;
                td.addressMode[1] = cudaAddressModeClamp;
                td.filterMode = cudaFilterModeLinear;
                td.readMode = cudaReadModeElementType;
                td.normalizedCoords = 0;
                cudaTextureObject_t o = 0;
                e = cudaCreateTextureObject(&o, &rd, &td, nullptr);
                if (e != cudaSuccess) {
                    objs.resize(b * ntpb + t);
                    destroy_objects();
                    return e;
                }
                objs[b * ntpb + t] = (unsigned long long)o;
            }
        if (d_objs_n < n_seg) {
            if (d_objs)
                cudaFree(d_objs);
            d_objs = nullptr;
            d_objs_n = 0;
            e = cudaMalloc(&d_objs, n_seg * sizeof(unsigned long long));
            if (e != cudaSuccess)
                return e;
            d_objs_n = n_seg;
        }
        e = cudaMemcpy(d_objs, objs.data(), n_seg * sizeof(unsigned long long), cudaMemcpyHostToDevice);
        if (e != cudaSuccess)
            return e;
        n = st.n;
        dim = D;
        batch = st.batch;
        tex = st.tex;
        pitch_ = pitch;
        full_bytes_ = full_bytes;
        batch_bytes_ = batch_bytes;
        n_batches = nb;
        device = dev;
    }
    return cudaSuccess;
}

cudaError_t TexStack::fill(const StackDesc& st, cudaStream_t stream)
{
    if (!mem || !d_objs || st.n != n || st.dim != dim || st.batch != batch || st.tex != tex)
        return cudaErrorInvalidValue;
    const size_t rows = (size_t)n_batches * batch * dim;
    if ((rows + 7) / 8 > 0x7FFFFFFFull)
        return cudaErrorInvalidValue;
    tex_fill_kernel<<<(unsigned)((rows + 7) / 8), 256, 0, stream>>>(st.img, n, dim, batch, tex, full_bytes_,
                                                                    batch_bytes_, pitch_, rows, mem);
    g_kernel_launches.fetch_add(1, std::memory_order_relaxed);
    return cudaGetLastError();
}

} // namespace gpuisac
