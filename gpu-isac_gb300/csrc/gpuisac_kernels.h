// gpuisac_kernels.h -- host-side launchers of the alignment kernels.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

#include <atomic>
#include <vector>

#include "gpuisac_device.cuh"

namespace gpuisac {

constexpr unsigned kMaxRingNum = 88;    // rings supported by the kernels (reference tile fits shared memory)
constexpr unsigned kMaxShifts = 4096;   // shift grid entries supported

inline size_t polar_spectra_smem_bytes(unsigned ring_num)
{
    return (size_t)((ring_num + 1) / 2) * kPairStride * sizeof(float2) + kRingLen * sizeof(float2) +
           24 * sizeof(double);
}

// rings are padded to a multiple of this in the reference tile in shared memory
constexpr unsigned kRingPad = 8;
__host__ __device__ inline unsigned ring_pad(unsigned ring_num) { return (ring_num + kRingPad - 1) / kRingPad * kRingPad; }

// references per CTA of the CCF/peak kernel for a ring count
inline unsigned ccf_refs_per_cta(unsigned ring_num) { return ring_pad(ring_num) <= 40 ? 4u : 2u; }

size_t ccf_peak_smem_bytes(unsigned ring_num);

// kernels launched by this library since load (all launchers count here)
extern std::atomic<unsigned long long> g_kernel_launches;

// cudaFuncSetAttribute(MaxDynamicSharedMemorySize) applies to the current
// device only: opt `kernel` in to at least `bytes` of dynamic shared memory
// on the current device, once per (device, kernel, larger size); thread-safe
cudaError_t opt_in_smem(const void* kernel, int bytes);
template <typename K>
inline cudaError_t opt_in_smem_k(K* kernel, size_t bytes)
{
    return opt_in_smem(reinterpret_cast<const void*>(kernel), (int)bytes);
}
// the device's opt-in maximum per block (current device)
int smem_optin_max();

// A device stack laid out as the reference's textures hold it (batches of
// st.batch images in textures of st.tex images, stale slots of a short final
// batch filled from the previous batch), one texture object per segment
// (tex_stack.cu).  prepare() allocates the layout and creates the objects
// (kept while the geometry stays the same; not inside a stream capture);
// fill() copies st.img into every slot on `stream` (a kernel, capturable);
// build() is both.
struct TexStack {
    unsigned char* mem = nullptr;
    size_t mem_bytes = 0, pitch_ = 0, full_bytes_ = 0, batch_bytes_ = 0;
    std::vector<unsigned long long> objs;
    unsigned long long* d_objs = nullptr;
    size_t d_objs_n = 0;
    unsigned n = 0, dim = 0, batch = 0, tex = 0, n_batches = 0;
    int device = -1;
    cudaError_t prepare(const StackDesc& st);
    cudaError_t fill(const StackDesc& st, cudaStream_t stream);
    cudaError_t build(const StackDesc& st, cudaStream_t stream);
    // build(), or -- when it fails (no memory for the copy, say) -- nothing:
    // returns the objects, or null after releasing any partial allocation;
    // the caller then samples with the emulation (the same texels and
    // weights; the filtered value equal to the last bit or two)
    const unsigned long long* try_build(const StackDesc& st, cudaStream_t stream);
    const unsigned long long* objects() const { return d_objs; }
    void destroy_objects();
    void release();
};

// One stack's part of a TexSet fill: the destination layout and the rows
// row_begin .. of the launch (tex_fill_jobs_kernel)
struct TexFillJob {
    const float* src;
    unsigned char* mem;
    size_t full_bytes, batch_bytes, pitch;
    unsigned n, dim, batch, tex;
    unsigned row_begin;
};

// Many stacks laid out as the reference's textures hold them (each as a
// TexStack would), in one device region: prepare() lays them out (the region
// only grows), creates the texture objects (objs, stack i's first at
// obj_first[i]; the previous call's objects are destroyed) and the fill jobs
// (jobs, rows).  The caller uploads the jobs and objects and fills with
// launch_tex_fill_jobs, whose row count it reads from device memory.
struct TexSet {
    unsigned char* mem = nullptr;
    size_t mem_bytes = 0;
    std::vector<unsigned long long> objs;
    std::vector<unsigned> obj_first;
    std::vector<TexFillJob> jobs;
    unsigned rows = 0;
    cudaError_t prepare(const std::vector<StackDesc>& stacks);
    void destroy_objects();
    void release();
};

// hdr = {jobs, rows} in device memory; grid-stride over the rows, a warp per row
cudaError_t launch_tex_fill_jobs(const TexFillJob* jobs, const unsigned* hdr, unsigned grid, cudaStream_t stream);

// Whether the kernels sample through the texture unit (TexStack) where the
// caller has one: on unless the environment sets GPUISAC_TEXTURE=0.
bool texture_unit_enabled();

// Resample + normalise + ring FFT of n_img images x n_shift shifts: images
// img0 .. img0 + n_img - 1 of the stack, or img_list[0 .. n_img-1] (device)
// when a list is given.  out: [n_img][n_shift][ring_num][kSlots] float2
// (see polar_spectra.cu).  tex_objs: texture objects of st built by a
// TexStack (samples through the texture unit), or null (the emulation).
cudaError_t launch_polar_spectra(const StackDesc& st, const float2* tmpl, const float2* twiddle,
                                 unsigned ring_num, const int2* shift_int, unsigned n_shift,
                                 const float2* base, unsigned img0, unsigned n_img, int is_ref,
                                 float2* out, cudaStream_t stream, const unsigned* img_list = nullptr,
                                 const unsigned long long* tex_objs = nullptr);

// A run of consecutive spectra rows of one stack: images img0 .. img0 +
// n_img - 1 x n_shift shifts, written from `out` on ([n_img][n_shift] rows);
// rows row_begin .. of the launch that holds the job.
struct SpectraJob {
    StackDesc st;
    const unsigned long long* tex_objs; // texture objects of st, or null (the emulation)
    const float2* base;                 // base shifts by image index in st, or null
    const int2* shift_int;              // n_shift integer shifts
    float2* out;
    unsigned img0, n_img, n_shift;
    int is_ref;
    unsigned row_begin;
};

// The spectra of a job table: hdr = {first job, jobs, rows, lookup offset}
// in device memory (jobs ordered by row_begin from 0); lut + hdr[3] holds,
// per block of kJobLutRows rows, the index of the job holding the block's
// first row.  One CTA per row: `grid` must cover the rows (CTAs past them
// return); the same launch serves any table the device buffers hold.
constexpr unsigned kJobLutRows = 32;
cudaError_t launch_polar_spectra_jobs(const SpectraJob* jobs, const unsigned* hdr, const unsigned* lut,
                                      const float2* tmpl, const float2* twiddle, unsigned ring_num, unsigned grid,
                                      cudaStream_t stream);

// ---------------------------------------------------------------------------
// Rings of 512 samples (ring512.cu): spectra rows [ring][kSlots512] float2 in
// the basis of the 256-sample rows (slot 0 = (F[0], F[256])), and the CCF /
// inverse-FFT / peak search over them; tw512[e] = e^(-2 pi i e / 512).
constexpr int kRingLen512 = 512;
constexpr int kSlots512 = kRingLen512 / 2;
cudaError_t launch_polar_spectra512(const StackDesc& st, const float2* tmpl, const float2* tw512, unsigned ring_num,
                                    const int2* shift_int, unsigned n_shift, const float2* base, unsigned img0,
                                    unsigned n_img, int is_ref, float2* out, cudaStream_t stream,
                                    const unsigned long long* tex_objs);
// results for particle i of sbj_sp to column p_first + i of d_out / peak_out
// [n_ref][p_total]; base: base shifts by global particle index, or null
cudaError_t launch_ccf_peak512(const float2* sbj_sp, const float2* ref_sp, const float2* tw512, unsigned ring_num,
                               unsigned n_shift, unsigned n_ref, unsigned n_part, unsigned p_first, unsigned p_total,
                               const float2* shifts_f, const float2* base, float* d_out, float4* peak_out,
                               cudaStream_t stream);

// ---------------------------------------------------------------------------
// Operands of the tensor-core contraction (ccf_split.cu).  For every spectrum
// slot k the contraction is a GEMM over the rings: subject rows (one image
// row = particle x shift, two operand rows: the a and b parts of its spectra)
// against reference rows (one reference, two operand rows: u and v), with
// each FP32 value split into a BF16 high part and the BF16 rounding of the
// remainder.  A tile's operand for slot k is, in bytes,
//   [hl: hi, lo][kg: group of 8 rings][rg: group of 8 operand rows][8 rows][8 rings x 2 B]
// -- the canonical no-swizzle K-major layout of tcgen05 with 128-byte core
// matrices, K groups kg_stored = ceil(rings / 8) (rings beyond the count
// hold zero), rg row groups per tile.
//   subjects: tile = (particle, shift block), shift s of block b = s / block
//             at rows 2 (s % block) + {0: a, 1: b};
//   references: tile = block consecutive references, reference q at rows
//             2 (q % block) + {0: u, 1: v}, the ring weight (r+1) folded in.
struct OperandLayout {
    unsigned char* base = nullptr; // [tiles][kSlots][slot_bytes()]
    unsigned kg = 0;               // K groups stored
    unsigned rg = 0;               // row groups per tile
    unsigned block = 0;            // image rows per tile: shifts (subjects) or references
    unsigned n_blocks = 1;         // subjects: shift blocks per particle
    __host__ __device__ size_t slot_bytes() const { return (size_t)2 * kg * rg * 128; }
    __host__ __device__ size_t tile_bytes() const { return slot_bytes() * kSlots; }
};

// The same resampling and FFT, written as tensor-core operands (opnd.base
// set): subjects (is_ref = 0) as rows of particle tiles, references (is_ref)
// as rows of reference tiles; the spectra values are those
// launch_polar_spectra writes, bit for bit, before the split.
cudaError_t launch_polar_operands(const StackDesc& st, const float2* tmpl, const float2* twiddle,
                                  unsigned ring_num, const int2* shift_int, unsigned n_shift,
                                  const float2* base, unsigned img0, unsigned n_img, int is_ref,
                                  const OperandLayout& opnd, cudaStream_t stream,
                                  const unsigned long long* tex_objs = nullptr);

// CCF against every reference + inverse FFT + peak search for n_part particles
// whose spectra are in sbj_sp ([n_part][n_shift][ring_num][kSlots]); results
// for particle i go to column p_global0 + i of d_out [n_ref][p_total] and
// peak_out [n_ref][p_total] (angle, shift_x, shift_y, mirror).
// One alignment group as the CCF / peak kernels see it: the particles of the
// group present in the current spectra buffer against all its references.
struct CcfGroup {
    const float2* sbj_sp;   // [n_part][n_shift][ring_num][kSlots]
    const float2* ref_sp;   // [n_ref][ring_num][kSlots]
    const float2* base;     // base shifts, indexed by the particle's index in the group; or null
    float* d_out;           // [n_ref][p_total]
    float4* peak_out;       // [n_ref][p_total]
    unsigned p_first;       // index in the group of sbj_sp's first particle
    unsigned n_part;        // particles of the group in sbj_sp
    unsigned n_ref;         // references of the group
    unsigned p_total;       // particles in the group (row pitch of the outputs)
    unsigned item_begin;    // first work item of the group
    unsigned ref_tiles;     // reference tiles of the group
    const unsigned* ref_idx; // rows of ref_sp holding the group's references 0..n_ref-1; null = 0..n_ref-1
    unsigned rule;           // peak rule: kPeakMref or kPeakPreAlign
};

// Peak rules.  kPeakMref: the multi-reference search's (first strict maximum
// from -FLT_MAX, angle with the reference's float/double mixing).
// kPeakPreAlign: the pre-alignment's (first strict maximum from 0, so a
// table with no positive value keeps index 0; angle from the parabola in
// double precision).
enum { kPeakMref = 0, kPeakPreAlign = 1 };

// Work of one CCF launch: either one group (groups == null, `one`) or a
// device table of n_groups groups ordered by item_begin.  With dyn set, the
// table is groups + dyn[0] and its group and item counts are dyn[1], dyn[2]
// in device memory (a recorded launch then serves any table of the buffer);
// n_items is then only the host's bound for the grid.
struct CcfWork {
    const CcfGroup* groups;
    CcfGroup one;
    unsigned n_groups;
    unsigned n_items;
    const unsigned* dyn;
    // the warp-specialised kernel's work counter (device word, zeroed by the
    // launcher): its CTAs take their next items from it, so that they stay
    // together on the same particle blocks (their spectra read from L2 by
    // every reference tile); null: item = CTA + k x grid
    unsigned* item_counter;
    unsigned ppc;     // particles per work item
    unsigned max_ref; // most references of any group (0: not known); 1 selects the one-reference contraction
    // failure-path tests only (gpuisac_test_stall_ccf): the kernels that stage
    // with bulk copies issue none, and their bounded waits give up after
    // wait_iters tries (0: the default, about a second)
    unsigned test_stall;
    unsigned wait_iters;
};

// the contraction the next alignment calls of this thread use regardless of
// the process-wide mode (the autotuner times FP32 tile shapes this way);
// -1 clears
void contraction_force(int mode);

// the failure-path test settings every CCF launch carries (both 0 normally)
void ccf_test_settings(unsigned& stall, unsigned& wait_iters);

enum { kCcfGeneral = 0, kCcfTmem = 1, kCcfWs = 2 };
constexpr unsigned kCcfParticlesPerItem = 8;

// Tile shape of the CCF launch: kernel variant, contraction warps of the
// warp-specialised kernel, particles per work item.  Chosen per (ring count,
// shift count): GPUISAC_CCF_KERNEL / GPUISAC_CCF_WS_WARPS override, then a
// candidate forced on this thread by the autotuner while it times it, then
// the autotuner's recorded choice, then the default (ws, 8, 8).
struct CcfTile {
    int variant;
    int ws_warps;
    unsigned ppc;
};
CcfTile ccf_tile(unsigned ring_num, unsigned n_shift, bool aligned);
void ccf_tile_record(unsigned ring_num, unsigned n_shift, const CcfTile& t);
void ccf_tile_force(const CcfTile* t); // this thread only; nullptr clears
bool ccf_tile_lookup(unsigned ring_num, unsigned n_shift, CcfTile& t);
bool ccf_tile_allows_tmem(unsigned ring_num); // the single-phase tensor-memory kernel takes this ring count
// bumped whenever a choice is recorded (cached launch graphs compare it)
unsigned ccf_tile_generation();

// kernel variant for a ring count (aligned: spectra rows 16-byte aligned)
int ccf_variant(unsigned ring_num, bool aligned, unsigned n_shift = 0);
// references per work item of that variant
unsigned ccf_refs_per_item(unsigned ring_num, int variant);

// persistent launch over the work items of w
cudaError_t launch_ccf_peak_work(const CcfWork& w, int variant, const float2* twiddle, unsigned ring_num,
                                 unsigned n_shift, const float2* shifts_f, unsigned* err, cudaStream_t stream);

// err: device word set to non-zero if a kernel gave up waiting for its own
// asynchronous copies (bounded waits; the host checks it after the stream).
cudaError_t launch_ccf_peak(const float2* sbj_sp, const float2* ref_sp, const float2* twiddle,
                            unsigned ring_num, unsigned n_shift, unsigned n_ref, unsigned n_part,
                            unsigned p_global0, unsigned p_total, const float2* shifts_f,
                            const float2* base, float* d_out, float4* peak_out, unsigned* err,
                            cudaStream_t stream, unsigned rule = kPeakMref, unsigned* item_counter = nullptr);

// the checked build's failure records of each instrumented translation unit
// (count and first (site, index); read and cleared), zero in the normal build
void checked_read_spectra(unsigned& count, unsigned long long& first);
void checked_read_split(unsigned& count, unsigned long long& first);
void checked_read_ccf(unsigned& count, unsigned long long& first);
void checked_read_ring512(unsigned& count, unsigned long long& first);
void checked_read_averages(unsigned& count, unsigned long long& first);

} // namespace gpuisac
