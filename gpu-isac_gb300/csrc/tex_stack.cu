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
#include <vector>

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

// tex_fill_kernel over a table of stacks (TexFillJob, ordered by row_begin
// from 0): one warp per destination row, persistent over hdr = {jobs, rows}
__global__ void __launch_bounds__(256)
tex_fill_jobs_kernel(const TexFillJob* __restrict__ jobs, const unsigned* __restrict__ hdr)
{
    const unsigned n_jobs = hdr[0], rows = hdr[1];
    for (unsigned r = blockIdx.x * 8 + (threadIdx.x >> 5); r < rows; r += gridDim.x * 8) {
        unsigned lo = 0, hi = n_jobs - 1;
        while (lo < hi) {
            const unsigned mid = (lo + hi + 1) >> 1;
            if (jobs[mid].row_begin <= r)
                lo = mid;
            else
                hi = mid - 1;
        }
        const TexFillJob& j = jobs[lo];
        const unsigned dim = j.dim, per_batch = j.batch * dim;
        const unsigned rl = r - j.row_begin;
        const unsigned b = rl / per_batch, rb = rl - b * per_batch;
        const unsigned t = rb / (j.tex * dim);
        const unsigned in_seg = rb - t * j.tex * dim;
        const unsigned jj = in_seg / dim, y = in_seg - jj * dim;
        unsigned g = b * j.batch + t * j.tex + jj;
        if (g >= j.n)
            g -= j.batch;
        float* dst = reinterpret_cast<float*>(j.mem + (size_t)b * j.batch_bytes + (size_t)t * j.full_bytes +
                                              (size_t)in_seg * j.pitch);
        const float* src = j.src + ((size_t)g * dim + y) * dim;
        for (unsigned x = threadIdx.x & 31; x < dim; x += 32)
            dst[x] = src[x];
    }
}

size_t round_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// where a stack's textures live: row pitch, bytes of a full texture, of a
// batch, of the whole layout; textures per batch, batches, images of a
// batch's last texture
struct TexGeometry {
    size_t pitch, full_bytes, batch_bytes, need;
    unsigned ntpb, nb, last_alloc;
};

cudaError_t tex_geometry(const StackDesc& st, int dev, TexGeometry& g)
{
    if (st.n == 0 || st.dim == 0 || st.batch == 0 || st.tex == 0 || st.batch > st.n)
        return cudaErrorInvalidValue;
    int tex_align = 512, pitch_align = 32;
    cudaDeviceGetAttribute(&tex_align, cudaDevAttrTextureAlignment, dev);
    cudaDeviceGetAttribute(&pitch_align, cudaDevAttrTexturePitchAlignment, dev);
    const unsigned D = st.dim;
    g.pitch = round_up((size_t)D * sizeof(float), (size_t)std::max(pitch_align, 4));
    g.ntpb = (st.batch + st.tex - 1) / st.tex;
    g.nb = (st.n + st.batch - 1) / st.batch;
    g.last_alloc = st.batch - (g.ntpb - 1) * st.tex;
    g.full_bytes = round_up((size_t)st.tex * D * g.pitch, (size_t)tex_align);
    const size_t last_bytes = round_up((size_t)g.last_alloc * D * g.pitch, (size_t)tex_align);
    g.batch_bytes = (size_t)(g.ntpb - 1) * g.full_bytes + last_bytes;
    g.need = (size_t)g.nb * g.batch_bytes;
    return cudaSuccess;
}

// one texture object per (batch, texture) segment of a layout at mem,
// appended to objs
cudaError_t create_tex_objects(unsigned char* mem, const StackDesc& st, const TexGeometry& g,
                               std::vector<unsigned long long>& objs)
{
    for (unsigned b = 0; b < g.nb; b++)
        for (unsigned t = 0; t < g.ntpb; t++) {
            const unsigned alloc = (t != g.ntpb - 1) ? st.tex : g.last_alloc;
            cudaResourceDesc rd{};
            rd.resType = cudaResourceTypePitch2D;
            rd.res.pitch2D.devPtr = mem + (size_t)b * g.batch_bytes + (size_t)t * g.full_bytes;
            rd.res.pitch2D.desc = cudaCreateChannelDesc<float>();
            rd.res.pitch2D.width = st.dim;
            rd.res.pitch2D.height = (size_t)alloc * st.dim;
            rd.res.pitch2D.pitchInBytes = g.pitch;
            cudaTextureDesc td{};
            td.addressMode[0] = cudaAddressModeClamp;
            td.addressMode[1] = cudaAddressModeClamp;
            td.filterMode = cudaFilterModeLinear;
            td.readMode = cudaReadModeElementType;
            td.normalizedCoords = 0;
            cudaTextureObject_t o = 0;
            const cudaError_t e = cudaCreateTextureObject(&o, &rd, &td, nullptr);
            if (e != cudaSuccess)
                return e;
            objs.push_back((unsigned long long)o);
        }
    return cudaSuccess;
}

} // namespace

void TexSet::destroy_objects()
{
    for (unsigned long long o : objs)
        cudaDestroyTextureObject((cudaTextureObject_t)o);
    objs.clear();
}

void TexSet::release()
{
    destroy_objects();
    if (mem)
        cudaFree(mem);
    mem = nullptr;
    mem_bytes = 0;
    jobs.clear();
    obj_first.clear();
    rows = 0;
}

cudaError_t TexSet::prepare(const std::vector<StackDesc>& stacks)
{
    destroy_objects();
    jobs.clear();
    obj_first.clear();
    rows = 0;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return e;
    std::vector<TexGeometry> geo(stacks.size());
    std::vector<size_t> off(stacks.size());
    size_t need = 0, total_rows = 0;
    for (size_t i = 0; i < stacks.size(); i++) {
        e = tex_geometry(stacks[i], dev, geo[i]);
        if (e != cudaSuccess)
            return e;
        off[i] = need;
        need += geo[i].need; // every part of a layout is a multiple of the texture alignment
        total_rows += (size_t)geo[i].nb * stacks[i].batch * stacks[i].dim;
    }
    if (total_rows > 0x7FFFFFFFull)
        return cudaErrorInvalidValue;
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
    size_t row = 0;
    for (size_t i = 0; i < stacks.size(); i++) {
        const StackDesc& st = stacks[i];
        const TexGeometry& g = geo[i];
        obj_first.push_back((unsigned)objs.size());
        e = create_tex_objects(mem + off[i], st, g, objs);
        if (e != cudaSuccess) {
            destroy_objects();
            return e;
        }
        TexFillJob j{};
        j.src = st.img;
        j.mem = mem + off[i];
        j.full_bytes = g.full_bytes;
        j.batch_bytes = g.batch_bytes;
        j.pitch = g.pitch;
        j.n = st.n;
        j.dim = st.dim;
        j.batch = st.batch;
        j.tex = st.tex;
        j.row_begin = (unsigned)row;
        jobs.push_back(j);
        row += (size_t)g.nb * st.batch * st.dim;
    }
    rows = (unsigned)row;
    return cudaSuccess;
}

cudaError_t launch_tex_fill_jobs(const TexFillJob* jobs, const unsigned* hdr, unsigned grid, cudaStream_t stream)
{
    if (grid == 0)
        return cudaSuccess;
    tex_fill_jobs_kernel<<<grid, 256, 0, stream>>>(jobs, hdr);
    g_kernel_launches.fetch_add(1, std::memory_order_relaxed);
    return cudaGetLastError();
}

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
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return e;
    TexGeometry g;
    e = tex_geometry(st, dev, g);
    if (e != cudaSuccess)
        return e;
    const bool same_layout = mem && g.need <= mem_bytes && dim == st.dim && batch == st.batch && tex == st.tex &&
                             n == st.n && pitch_ == g.pitch && device == dev;
    if (same_layout)
        return cudaSuccess;
    destroy_objects();
    if (g.need > mem_bytes) {
        if (mem)
            cudaFree(mem);
        mem = nullptr;
        mem_bytes = 0;
        e = cudaMalloc(&mem, g.need);
        if (e != cudaSuccess)
            return e;
        mem_bytes = g.need;
    }
    e = create_tex_objects(mem, st, g, objs);
    if (e != cudaSuccess) {
        destroy_objects();
        return e;
    }
    const size_t n_seg = objs.size();
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
    dim = st.dim;
    batch = st.batch;
    tex = st.tex;
    pitch_ = g.pitch;
    full_bytes_ = g.full_bytes;
    batch_bytes_ = g.batch_bytes;
    n_batches = g.nb;
    device = dev;
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
