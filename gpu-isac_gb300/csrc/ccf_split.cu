// ccf_split.cu -- the ring-summed cross-correlation on the tensor cores:
// BF16 hi/lo split operands (hi*hi + hi*lo + lo*hi, FP32 accumulation in
// tensor memory), then the inverse angular FFT and the peak search.
//
// Reference semantics: cu_ccf_mult_mref (cuda/gpu_aln_noref.cu:1483-1537),
// the C2R of every ccf-table entry (:2453-2461) and cu_aln_param_wizard
// (:1667-1794) -- the same as ccf_peak.cu, whose peak search and FFT this
// file shares (ccf_device.cuh); only the contraction's arithmetic differs.
//
// For every spectrum slot k the contraction is a GEMM over the rings:
//   D[(shift s, a|b)][(reference q, u|v)] = sum_r S[s][r][a|b] * R[q][r][u|v]
// whose four products per (shift, reference) pair are Re/Im of Z[k] and of
// Z[256-k] (polar_spectra.cu).  Every pair needs all 128 slots before its
// inverse FFT, 2 KB of accumulators, so MMA-sized tiles (thousands of pairs)
// cannot keep them on the SM: the pair spectra Z pass through HBM between two
// kernels, each launched once per particle chunk:
//
// ccf_mma_kernel    persistent; work item = (particle, shift block, reference
//                   tile); 576 threads: warp 0 issues the bulk copies of each
//                   slot's operands into a ring of shared-memory stages, one
//                   thread of warp 1 issues the 3 x K/16 tcgen05.mma of a slot
//                   (M = 128 lanes = 64 shifts x {a, b}, N = 2 x references)
//                   into one of two accumulators in tensor memory, and 16
//                   drain warps (four per lane quadrant) drain the other
//                   accumulator with tcgen05.ld and store every row's ring
//                   sums (sum u, sum v) per reference, the a and b rows of a
//                   shift side by side; the FFT kernel assembles Z[k] and
//                   Z[256-k] of each (shift, reference) pair from them.
// zfft_peak_kernel  persistent; work item = (particle, reference); the Z block
//                   of each shift block is bulk-copied into a shared buffer
//                   as soon as every 16-thread group has taken its shift's
//                   column of the previous one, each group running the
//                   inverse FFT and the peak search in its own workspace; a
//                   control warp merges the groups' bests at the item's end.
//
// Every wait is bounded (about a second); a kernel that gives up sets *err,
// lets its own copies and MMAs land, frees its tensor memory and returns.
#include <stdint.h>

#include <algorithm>

#include "ccf_device.cuh"
#include "gpuisac_device.cuh"
#include "gpuisac_kernels.h"
#include "gpuisac_split.h"

namespace gpuisac {

namespace {

// ---------------------------------------------------------------- helpers
__device__ __forceinline__ void mbar_arrive(uint64_t* bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

// bounded wait that also gives up once another role has aborted
__device__ __forceinline__ bool mbar_wait_abort(uint64_t* bar, uint32_t parity, volatile int* abort_flag,
                                                uint32_t tries)
{
    for (uint32_t it = 0; it < tries; it++) {
        if (mbar_try(bar, parity, 20000u))
            return true;
        if (*abort_flag)
            return false;
    }
    return false;
}

// shared-memory matrix descriptor (no swizzle): start address, leading (K)
// and stride (M/N) byte offsets in 16-byte units, version bits of tcgen05
__device__ __forceinline__ uint64_t mma_desc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}

__device__ __forceinline__ void mma_bf16(uint32_t d, uint64_t da, uint64_t db, uint32_t idesc, uint32_t acc)
{
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "setp.ne.u32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
                 "l"(da), "l"(db), "r"(idesc), "r"(acc)
                 : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
                 : "memory");
}

// instruction descriptor of kind::f16: F32 accumulator, BF16 A and B, both
// K-major, M = 128, N = n
__host__ __device__ constexpr uint32_t mma_idesc(uint32_t n)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((n >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
}

constexpr int kDrainWarps = 16;      // four per tensor-memory lane quadrant
constexpr int kDrainPerQuad = kDrainWarps / 4;
constexpr int kMmaThreads = 64 + 32 * kDrainWarps; // warp 0 copies, warp 1 MMA, warps 2.. drain
constexpr uint32_t kMmaTailPad = 2048; // 16 row groups x 128 bytes
constexpr uint32_t kAccStride = 256; // tensor-memory columns between the two accumulators
constexpr uint32_t kMmaTmemCols = 512;

} // namespace

// ============================================================================
__global__ void __launch_bounds__(kMmaThreads, 1) ccf_mma_kernel(SplitMmaWork w, unsigned* __restrict__ err)
{
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    const unsigned kge = w.kg + (w.kg & 1u);             // K groups the MMAs read (an odd count gets a zero group)
    const uint32_t a_bytes = kge * w.rga * 128u;         // one of A_hi / A_lo in a stage
    const uint32_t b_bytes = kge * w.rgb * 128u;         // one of B_hi / B_lo
    const uint32_t stage_bytes = 2u * (a_bytes + b_bytes);
    const uint32_t a_copy = w.kg * w.rga * 128u, b_copy = w.kg * w.rgb * 128u; // bytes copied per part
    // the barriers sit behind kMmaTailPad bytes: an M = 128 MMA reads 16 row
    // groups of A whatever the tile stores, and the rows beyond a short tile
    // (never drained) may run past the last stage
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw + (size_t)w.n_stages * stage_bytes + kMmaTailPad);
    uint64_t* full = bars;                  // [n_stages] operands landed
    uint64_t* empty = bars + w.n_stages;    // [n_stages] MMAs done with the stage
    uint64_t* accf = empty + w.n_stages;    // [2] accumulator written
    uint64_t* acce = accf + 2;              // [2] accumulator drained
    uint64_t* done = acce + 2;              // last MMAs finished (abort path)
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (blockIdx.x >= w.n_items)
        return;
    const uint32_t wlim = wait_tries(w.wait_iters);

    // the zero K group of an odd K-group count, in every part of every stage
    if (kge != w.kg) {
        for (unsigned st = 0; st < w.n_stages; st++) {
            unsigned char* sb = smem_raw + (size_t)st * stage_bytes;
            const uint32_t offs[4] = {a_copy, a_bytes + a_copy, 2 * a_bytes + b_copy, 2 * a_bytes + b_bytes + b_copy};
            const uint32_t lens[4] = {w.rga * 128u, w.rga * 128u, w.rgb * 128u, w.rgb * 128u};
            for (int part = 0; part < 4; part++)
                for (uint32_t i = tid * 16; i < lens[part]; i += kMmaThreads * 16)
                    *reinterpret_cast<uint4*>(sb + offs[part] + i) = make_uint4(0u, 0u, 0u, 0u);
        }
    }
    if (warp == 1)
        tmem_alloc(tmem_slot, kMmaTmemCols);
    if (tid == 0) {
        for (unsigned i = 0; i < w.n_stages; i++) {
            mbar_init(full + i, 1);
            mbar_init(empty + i, 1);
        }
        for (int i = 0; i < 2; i++) {
            mbar_init(accf + i, 1);
            mbar_init(acce + i, 32 * kDrainWarps);
        }
        mbar_init(done, 1);
        *abort_flag = 0;
        mbar_fence_init();
    }
    fence_proxy_async(); // the zero groups become visible to the tensor cores
    tmem_fence_before();
    __syncthreads();
    tmem_fence_after();
    const uint32_t tmem = *tmem_slot;

    bool failed = false;
    if (warp == 0) {
        // ================= operand copies =================
        if (lane == 0) {
            uint32_t it = 0;
            for (unsigned item = blockIdx.x; item < w.n_items && !failed; item += gridDim.x) {
                const unsigned t = item % w.n_rtiles, pb = item / w.n_rtiles; // pb = particle * n_blocks + block
                const unsigned char* a_src = w.sop + (size_t)pb * kSlots * w.sop_slot;
                const unsigned char* b_src = w.rop + (size_t)t * kSlots * w.rop_slot;
                for (unsigned k = 0; k < (unsigned)kSlots; k++, it++) {
                    const uint32_t st = it % w.n_stages;
                    if (it >= w.n_stages && !mbar_wait_abort(empty + st, ((it / w.n_stages) - 1u) & 1u, abort_flag, wlim)) {
                        failed = true;
                        break;
                    }
                    if (w.test_stall)
                        continue; // failure-path test: no copies
                    unsigned char* sb = smem_raw + (size_t)st * stage_bytes;
                    mbar_expect_tx(full + st, 2u * (a_copy + b_copy));
                    const unsigned char* as = a_src + (size_t)k * w.sop_slot;
                    const unsigned char* bs = b_src + (size_t)k * w.rop_slot;
                    // (checked build: an out-of-range copy is left out and the
                    // stage's bounded wait reports the call as failed)
                    const bool a_in = GPUISAC_IN_BOUNDS(kChkMmaA, (size_t)(as - w.sop) + 2 * a_copy - 1,
                                                        (size_t)w.n_part * w.n_blocks * kSlots * w.sop_slot);
                    const bool b_in = GPUISAC_IN_BOUNDS(kChkMmaB, (size_t)(bs - w.rop) + 2 * b_copy - 1,
                                                        (size_t)w.n_rtiles * kSlots * w.rop_slot);
                    if (a_in && b_in) {
                        bulk_g2s(sb, as, a_copy, full + st);
                        bulk_g2s(sb + a_bytes, as + a_copy, a_copy, full + st);
                        bulk_g2s(sb + 2 * a_bytes, bs, b_copy, full + st);
                        bulk_g2s(sb + 2 * a_bytes + b_bytes, bs + b_copy, b_copy, full + st);
                    }
                }
            }
            if (failed) {
                *abort_flag = 1;
                atomicExch(err, 1u);
            }
            // every issued copy has landed before the CTA ends: the last
            // n_stages stages' full phases (bounded; on the normal path the
            // MMA thread has already waited for them)
            const uint32_t issued = w.test_stall ? 0u : it;
            for (uint32_t j = issued > w.n_stages ? issued - w.n_stages : 0; j < issued; j++)
                mbar_wait(full + (j % w.n_stages), (j / w.n_stages) & 1u, wlim);
        }
    } else if (warp == 1) {
        // ================= MMA issue =================
        if (lane == 0) {
            const uint32_t idesc = mma_idesc(w.n_cols);
            const uint32_t ks = kge / 2; // K steps of 16 rings
            uint32_t it = 0;
            bool any = false;
            for (unsigned item = blockIdx.x; item < w.n_items && !failed; item += gridDim.x) {
                for (unsigned k = 0; k < (unsigned)kSlots; k++, it++) {
                    const uint32_t st = it % w.n_stages, buf = it & 1u;
                    if (!mbar_wait_abort(full + st, (it / w.n_stages) & 1u, abort_flag, wlim) ||
                        (it >= 2 && !mbar_wait_abort(acce + buf, ((it >> 1) - 1u) & 1u, abort_flag, wlim))) {
                        failed = true;
                        break;
                    }
                    tmem_fence_after();
                    const uint32_t sa = smem_addr(smem_raw + (size_t)st * stage_bytes);
                    const uint32_t sa_lo = sa + a_bytes, sb_hi = sa + 2 * a_bytes, sb_lo = sb_hi + b_bytes;
                    const uint32_t d = tmem + buf * kAccStride;
                    const uint32_t lbo_a = w.rga * 128u, lbo_b = w.rgb * 128u;
#pragma unroll 1
                    for (uint32_t j = 0; j < ks; j++) {
                        const uint32_t oa = 2 * j * lbo_a, ob = 2 * j * lbo_b;
                        const uint64_t ah = mma_desc(sa + oa, lbo_a, 128), al = mma_desc(sa_lo + oa, lbo_a, 128);
                        const uint64_t bh = mma_desc(sb_hi + ob, lbo_b, 128), bl = mma_desc(sb_lo + ob, lbo_b, 128);
                        mma_bf16(d, ah, bh, idesc, j > 0 ? 1u : 0u);
                        mma_bf16(d, ah, bl, idesc, 1u);
                        mma_bf16(d, al, bh, idesc, 1u);
                    }
                    mma_commit(empty + st);
                    mma_commit(accf + buf);
                    any = true;
                }
            }
            if (failed) {
                *abort_flag = 1;
                atomicExch(err, 1u);
                if (any) { // the MMAs already issued finish before the tensor memory is freed
                    mma_commit(done);
                    mbar_wait(done, 0, wlim);
                }
            }
        }
    } else {
        // ================= drain: accumulators -> Z =================
        // kDrainPerQuad warps per lane quadrant share a slot's columns: chunks
        // of 16 columns (8 references) go round-robin between them, the next
        // chunk's tensor-memory load in flight while the current one is
        // written out
        const int quad = warp & 3;                  // tensor-memory lanes 32 quad .. 32 quad + 31
        const unsigned part = (unsigned)(warp - 2) >> 2; // which chunks: part, part + kDrainPerQuad, ...
        const unsigned row = 32 * quad + lane;      // operand row = 2 shift + {0: a, 1: b}
        const unsigned sl = row >> 1;               // shift within the block
        uint32_t it = 0;
        for (unsigned item = blockIdx.x; item < w.n_items && !failed; item += gridDim.x) {
            const unsigned t = item % w.n_rtiles, pb = item / w.n_rtiles;
            const unsigned p = pb / w.n_blocks, b = pb - p * w.n_blocks;
            const unsigned q0 = t * w.rblock, nq = min(w.rblock, w.n_ref - q0);
            const unsigned s0 = b * w.block, nsb = min(w.block, w.n_shift - s0);
            const bool row_ok = sl < nsb;
            // ring sums of (p, q, b): [128 slots][zw shifts][a, b] float2, each
            // entry a row's (sum u, sum v); the 32 rows of a warp store 256
            // contiguous bytes per reference, and the FFT kernel assembles
            // Z[k] = (sum u a, sum u b) and Z[256-k] = (sum v b, sum v a)
            float2* zbase = w.z + ((size_t)(p * w.n_ref + q0) * w.n_blocks + b) * kRingLen * w.zw + row;
            const size_t zq = (size_t)w.n_blocks * kRingLen * w.zw; // between references
            const unsigned nchunk = (2 * nq + 15) / 16;
            const unsigned nj = nchunk > part ? (nchunk - part + kDrainPerQuad - 1) / kDrainPerQuad : 0;
            for (unsigned k = 0; k < (unsigned)kSlots; k++, it++) {
                const uint32_t buf = it & 1u;
                const bool ok = mbar_wait_abort(accf + buf, (it >> 1) & 1u, abort_flag, wlim);
                if (!__all_sync(0xffffffffu, ok)) {
                    failed = true;
                    break;
                }
                tmem_fence_after();
                const uint32_t taddr = tmem + ((uint32_t)(32 * quad) << 16) + buf * kAccStride;
                float2* const zrow = zbase + (size_t)k * 2 * w.zw;
                auto write_chunk = [&](const float (&r)[16], unsigned c) {
#pragma unroll
                    for (int j = 0; j < 8; j++) {
                        const unsigned ql = 8 * c + j;
                        if (row_ok && ql < nq &&
                            GPUISAC_IN_BOUNDS(kChkMmaZ, (size_t)(zrow + ql * zq - w.z),
                                              (size_t)w.n_part * w.n_ref * w.n_blocks * kRingLen * w.zw))
                            __stcs(zrow + ql * zq, make_float2(r[2 * j], r[2 * j + 1])); // streamed: read once
                    }
                };
                if (nj) {
                    float ra[16], rb[16];
                    tmem_ld16_async(taddr + 16 * part, ra);
                    tmem_wait_ld16(ra);
                    for (unsigned j = 0; j < nj; j += 2) {
                        const unsigned ca = part + kDrainPerQuad * j, cb = ca + kDrainPerQuad;
                        const bool more_b = j + 1 < nj;
                        if (more_b)
                            tmem_ld16_async(taddr + 16 * cb, rb);
                        write_chunk(ra, ca);
                        if (!more_b)
                            break;
                        tmem_wait_ld16(rb);
                        const bool more_a = j + 2 < nj;
                        if (more_a)
                            tmem_ld16_async(taddr + 16 * (cb + kDrainPerQuad), ra);
                        write_chunk(rb, cb);
                        if (more_a)
                            tmem_wait_ld16(ra);
                    }
                }
                tmem_fence_before();
                mbar_arrive(acce + buf);
            }
        }
        if (failed && lane == 0) {
            *abort_flag = 1;
            atomicExch(err, 1u);
        }
    }
    // release the tensor memory (all tcgen05 accesses of the CTA are done)
    tmem_fence_before();
    __syncthreads();
    tmem_fence_after();
    if (warp == 1)
        tmem_dealloc(tmem, kMmaTmemCols);
}

// ============================================================================
// inverse FFT + peak search of the pair spectra Z, one (particle, reference)
// per work item, one 16-thread group per shift of a block (w.block groups, up
// to kSplitMaxBlock = 49, in whole warps), plus one control warp.  The units
// (item, shift block) stream through one shared buffer of ring sums in
// kZfftParts parts (of 128 / kZfftParts slots each): the control warp copies a
// part of unit u + 1 in as soon as every group has taken its values of that
// part of unit u into registers (mbarriers `empty`), so several copies can be
// in flight and they overlap the FFTs; each group then transforms in its own
// workspace and runs on without waiting for the others.
// A finished item's group bests are parked in one of kZfftRing slot sets
// (mbarrier `parked`); the control warp merges them, writes the outputs and
// hands the set back (mbarrier `freed`).
constexpr int kZfftCtlThreads = 32;
constexpr unsigned kZfftRing = 4;
constexpr int kZfftParts = 2; // divides 8: a lane's 8 slots l + 16 m split evenly (4 parts: FFT kernel 261 -> 289 ms)
__host__ __device__ constexpr unsigned zfft_group_threads(unsigned groups) { return (16 * groups + 31) / 32 * 32; }
__host__ __device__ constexpr size_t zfft_zbuf_bytes(unsigned zw)
{
    return ((size_t)kRingLen * zw * sizeof(float2) + 15) / 16 * 16;
}

__global__ void __launch_bounds__(zfft_group_threads(kSplitMaxBlock) + kZfftCtlThreads, 1)
zfft_peak_kernel(SplitFftWork w, const float2* __restrict__ twiddle, unsigned* __restrict__ err)
{
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    const unsigned groups = w.block;
    const unsigned gthreads = 16 * groups;
    const bool ctl = threadIdx.x >= zfft_group_threads(groups);
    const size_t unit_elems = (size_t)kRingLen * w.zw;
    float2* const zb = reinterpret_cast<float2*>(smem_raw);                                // [128][zw][a, b]
    float2* const wsp = reinterpret_cast<float2*>(smem_raw + zfft_zbuf_bytes(w.zw));       // [groups][kPairStride]
    float2* const tw = wsp + (size_t)groups * kPairStride;                                 // [16][kTwRow]
    PeakSlot* const slots = reinterpret_cast<PeakSlot*>(tw + 16 * kTwRow);                 // [kZfftRing][64]
    uint64_t* const full = reinterpret_cast<uint64_t*>(slots + kZfftRing * 64); // [kZfftParts]
    uint64_t* const empty = full + kZfftParts;     // [kZfftParts]
    uint64_t* const parked = empty + kZfftParts;   // [kZfftRing]
    uint64_t* const freed = parked + kZfftRing;    // [kZfftRing]
    volatile int* const abort_flag = reinterpret_cast<volatile int*>(freed + kZfftRing);

    const int tid = threadIdx.x;
    const unsigned n_items = w.n_part * w.n_ref;
    if (blockIdx.x >= n_items)
        return;
    for (int i = tid; i < kRingLen; i += blockDim.x) { // lane l's inverse-FFT twiddles, row l
        const int tl = i >> 4, tj = i & 15;
        const float2 t = twiddle[(tl * tj) & (kRingLen - 1)];
        tw[tl * kTwRow + tj] = make_float2(t.x, t.y * -1.f);
    }
    if (tid == 0) {
        for (int h = 0; h < kZfftParts; h++) {
            mbar_init(full + h, 1);
            mbar_init(empty + h, gthreads);
        }
        for (unsigned i = 0; i < kZfftRing; i++) {
            mbar_init(parked + i, gthreads);
            mbar_init(freed + i, 1);
        }
        *abort_flag = 0;
        mbar_fence_init();
    }
    __syncthreads();

    // units of this CTA: (item, block), item = particle x reference
    const unsigned my_items = (n_items - blockIdx.x + gridDim.x - 1) / gridDim.x;
    const unsigned n_units = my_items * w.n_blocks;
    auto unit_item = [&](unsigned u) { return blockIdx.x + (u / w.n_blocks) * gridDim.x; };
    const uint32_t wlim = wait_tries(w.wait_iters);

    if (ctl) {
        // ---------------- control warp: copies, merges, outputs ----------------
        const int lane = tid & 31;
        const size_t half = unit_elems / kZfftParts; // one part: [128 / kZfftParts][zw][a, b]
        auto issue = [&](unsigned u, int h) {
            if (w.test_stall)
                return; // failure-path test: no copies
            const unsigned item = unit_item(u), b = u % w.n_blocks;
            const uint32_t bytes = (uint32_t)(half * sizeof(float2));
            const size_t at = ((size_t)item * w.n_blocks + b) * unit_elems + h * half;
            if (!GPUISAC_IN_BOUNDS(kChkZfftZ, at + half - 1, (size_t)n_items * w.n_blocks * unit_elems))
                return; // (checked build) the groups' bounded wait reports the failure
            fence_proxy_async();
            mbar_expect_tx(full + h, bytes);
            bulk_g2s(zb + h * half, w.z + at, bytes, full + h);
        };
        // the groups' parked bests of a finished item, reduced in the
        // reference's order (better(); equal entries: the lower group, which
        // holds the lower shifts), then the parabola and the outputs
        auto merge = [&](unsigned item, const PeakSlot* sl) {
            unsigned bi = (unsigned)lane < groups ? (unsigned)lane : 0u;
            float v = sl[bi].v;
            unsigned h = sl[bi].h, t = sl[bi].t;
            if ((unsigned)lane + 32 < groups) { // up to 64 groups: two per lane
                const PeakSlot& o = sl[lane + 32];
                if (better(o.v, o.h, o.t, v, h, t)) {
                    v = o.v;
                    h = o.h;
                    t = o.t;
                    bi = lane + 32;
                }
            }
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                const float v2 = __shfl_xor_sync(0xffffffffu, v, off);
                const unsigned h2 = __shfl_xor_sync(0xffffffffu, h, off), t2 = __shfl_xor_sync(0xffffffffu, t, off);
                const unsigned b2 = __shfl_xor_sync(0xffffffffu, bi, off);
                if (better(v2, h2, t2, v, h, t) || (v2 == v && h2 == h && t2 == t && b2 < bi)) {
                    v = v2;
                    h = h2;
                    t = t2;
                    bi = b2;
                }
            }
            if (lane == 0) {
                const PeakSlot& ps = sl[bi];
                const bool mirror = ps.h >= w.n_shift;
                const unsigned sidx = mirror ? ps.h - w.n_shift : ps.h;
                const float angle =
                    w.rule == kPeakPreAlign ? pre_peak_angle(ps.nb, ps.t, mirror) : peak_angle(ps.nb, ps.t, mirror);
                const unsigned p = item / w.n_ref, q = item - p * w.n_ref;
                const unsigned pg = w.p_first + p;
                const float bx = w.base ? w.base[pg].x : 0.f, by = w.base ? w.base[pg].y : 0.f;
                const float2 sf = w.shifts_f[sidx];
                const size_t o = (size_t)q * w.p_total + pg;
                if (GPUISAC_IN_BOUNDS(kChkZfftOut, o, (size_t)w.n_ref * w.p_total)) {
                    w.d_out[o] = ps.v;
                    w.peak_out[o] = make_float4(angle, bx + sf.x, by + sf.y, mirror ? 1.f : 0.f);
                }
            }
        };
        bool failed = false;
        unsigned issued[kZfftParts] = {}, n_done = 0; // units issued per part
        if (lane == 0 && n_units > 0)
            for (int h = 0; h < kZfftParts; h++)
                issue(0, h);
        if (n_units > 0)
            for (int h = 0; h < kZfftParts; h++)
                issued[h] = 1;
        for (unsigned u = 0; u < n_units; u++) {
            // every group holds its unit-u values of a part: the part takes unit u + 1
            bool ok = true;
#pragma unroll
            for (int h = 0; h < kZfftParts; h++) {
                if (lane == 0) {
                    ok = ok && mbar_wait_abort(empty + h, u & 1u, abort_flag, wlim);
                    if (ok && u + 1 < n_units)
                        issue(u + 1, h);
                }
                if (!__shfl_sync(0xffffffffu, ok, 0))
                    break;
                if (u + 1 < n_units)
                    issued[h] = u + 2;
            }
            if (!__shfl_sync(0xffffffffu, ok, 0)) {
                failed = true;
                break;
            }
            if (u % w.n_blocks == w.n_blocks - 1) {
                const unsigned set = n_done % kZfftRing;
                ok = mbar_wait_abort(parked + set, (n_done / kZfftRing) & 1u, abort_flag, wlim);
                if (!__all_sync(0xffffffffu, ok)) {
                    failed = true;
                    break;
                }
                merge(unit_item(u), slots + 64 * set);
                __syncwarp();
                if (lane == 0)
                    mbar_arrive(freed + set);
                n_done++;
            }
        }
        if (failed && lane == 0) {
            *abort_flag = 1;
            atomicExch(err, 1u);
            // the last copies issued land before the CTA ends (bounded)
            for (int h = 0; h < kZfftParts; h++)
                if (issued[h] && !w.test_stall)
                    mbar_wait(full + h, (issued[h] - 1) & 1u, wlim);
        }
        return;
    }

    // ---------------- FFT groups ----------------
    const int g = tid >> 4, l = tid & 15;
    if ((unsigned)g >= groups)
        return; // the unused half of the last warp
    const unsigned gmask = 0xffffu << (tid & 16);
    float2* const gz = wsp + (size_t)g * kPairStride;
    PeakState st;
    st.reset(w.rule);
    unsigned n_done = 0;
    for (unsigned u = 0; u < n_units; u++) {
        const unsigned b = u % w.n_blocks;
        const unsigned s0 = b * w.block, nsb = min(w.block, w.n_shift - s0);
        const bool has = (unsigned)g < nsb; // group-uniform
        // the ring sums e = (ua, va, ub, vb) of slot l + 16 m (m < 8) give
        // Z[k] = (ua, ub) for k = l + 16 m (input m) and Z[256 - k] =
        // (vb, va), input 15 - m of lane (16 - l) mod 16; lane 0 keeps its
        // own: Z[256 - 16 m] is its input 16 - m, and slot 0 (the real
        // (F[0], F[128]) products) gives Z[0] and Z[128].  Slots l + 16 m
        // are in part m / (8 / kZfftParts) of the buffer.
        float2 x[16];
        float p2 = 0.f;
        const float4* z4 = reinterpret_cast<const float4*>(zb);
        const int partner = (16 - l) & 15;
#pragma unroll
        for (int h = 0; h < kZfftParts; h++) {
            if (!mbar_wait_abort(full + h, u & 1u, abort_flag, wlim)) {
                *abort_flag = 1;
                atomicExch(err, 1u);
                return;
            }
            if (has) {
#pragma unroll
                for (int m = h * (8 / kZfftParts); m < (h + 1) * (8 / kZfftParts); m++) {
                    const float4 e = z4[(l + 16 * m) * w.zw + g];
                    x[m] = make_float2(e.x, e.z);
                    x[15 - m] =
                        make_float2(__shfl_sync(gmask, e.w, partner, 16), __shfl_sync(gmask, e.y, partner, 16));
                    if (l == 0) {
                        if (m == 0) {
                            const float p1 = 0.25f * (e.x + e.z + e.w + e.y);
                            p2 = 0.25f * (e.x - e.z + e.w - e.y);
                            x[0] = make_float2(p1, p1);
                        } else {
                            x[16 - m] = make_float2(e.w, e.y);
                        }
                    }
                }
            }
            mbar_arrive(empty + h);
        }
        if (has && l == 0)
            x[8] = make_float2(p2, p2);
        if (has)
            fft_peak_regs<true>(x, gz, tw + l * kTwRow, l, gmask, s0 + g, w.n_shift, st, w.rule);
        if (b == w.n_blocks - 1) {
            // every shift of the pair has been searched: park the group's best
            const unsigned set = n_done % kZfftRing;
            if (!mbar_wait_abort(freed + set, ((n_done / kZfftRing) & 1u) ^ 1u, abort_flag, wlim)) {
                *abort_flag = 1;
                atomicExch(err, 1u);
                return;
            }
            park_slot(slots + 64 * set, st, g, l);
            mbar_arrive(parked + set);
            st.reset(w.rule);
            n_done++;
        }
    }
}

// ============================================================================

GPUISAC_CHECKED_READER(checked_read_split)

static int device_sms()
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return std::max(sms, 1);
}


static size_t mma_stage_bytes(const SplitPlan& p)
{
    const unsigned kge = p.kg + (p.kg & 1u);
    return (size_t)2 * kge * (p.rga + p.rgb) * 128;
}

static size_t mma_smem(const SplitPlan& p) { return (size_t)p.n_stages * mma_stage_bytes(p) + kMmaTailPad + 256; }

static size_t fft_smem(const SplitPlan& p)
{
    return zfft_zbuf_bytes(p.zw) + (size_t)p.fft_groups * kPairStride * sizeof(float2) + 16 * kTwRow * sizeof(float2) +
           kZfftRing * 64 * sizeof(PeakSlot) + (2 * kZfftParts + 2 * kZfftRing) * sizeof(uint64_t) + 16;
}

bool split_plan(unsigned ring_num, unsigned n_shift, unsigned n_ref, SplitPlan& p)
{
    if (ring_num == 0 || ring_num > kMaxRingNum || n_shift == 0 || n_ref == 0)
        return false;
    p.n_blocks = (n_shift + kSplitMaxBlock - 1) / kSplitMaxBlock;
    p.block = (n_shift + p.n_blocks - 1) / p.n_blocks;
    p.zw = p.block | 1u; // odd row length: the FFT's column reads hit distinct banks
    p.kg = (ring_num + 7) / 8;
    p.rga = (2 * p.block + 7) / 8;
    p.rounds = 1;
    p.fft_groups = p.block;
    const size_t cap = std::min<size_t>((size_t)smem_optin_max(), 227 * 1024);
    // references per tile: as many as N = 2 x refs <= 256 allows with at
    // least two operand stages, tiles balanced
    for (unsigned maxq = 128; maxq >= 8; maxq /= 2) {
        const unsigned tiles = (n_ref + maxq - 1) / maxq;
        p.rblock = (n_ref + tiles - 1) / tiles;
        p.n_rtiles = (n_ref + p.rblock - 1) / p.rblock;
        p.n_cols = (2 * p.rblock + 15) / 16 * 16;
        p.rgb = p.n_cols / 8;
        p.n_stages = 0;
        const size_t sb = mma_stage_bytes(p);
        const unsigned fit = (unsigned)std::min<size_t>(4, (cap - kMmaTailPad - 256) / sb);
        if (fit >= 2) {
            p.n_stages = fit;
            break;
        }
    }
    if (p.n_stages < 2 || fft_smem(p) > cap)
        return false;
    p.sop_slot = (size_t)2 * p.kg * p.rga * 128;
    p.rop_slot = (size_t)2 * p.kg * p.rgb * 128;
    return true;
}

size_t split_sop_bytes(const SplitPlan& p, unsigned n_part) { return (size_t)n_part * p.n_blocks * kSlots * p.sop_slot; }
size_t split_rop_bytes(const SplitPlan& p) { return (size_t)p.n_rtiles * kSlots * p.rop_slot; }
size_t split_z_bytes(const SplitPlan& p, unsigned n_part, unsigned n_ref)
{
    return (size_t)n_part * n_ref * p.n_blocks * kRingLen * p.zw * sizeof(float2);
}

OperandLayout split_sbj_layout(const SplitPlan& p, unsigned char* base)
{
    OperandLayout o;
    o.base = base;
    o.kg = p.kg;
    o.rg = p.rga;
    o.block = p.block;
    o.n_blocks = p.n_blocks;
    return o;
}

OperandLayout split_ref_layout(const SplitPlan& p, unsigned char* base)
{
    OperandLayout o;
    o.base = base;
    o.kg = p.kg;
    o.rg = p.rgb;
    o.block = p.rblock;
    o.n_blocks = 1;
    return o;
}

cudaError_t launch_ccf_mma(const SplitPlan& p, const unsigned char* sop, const unsigned char* rop, float2* z,
                           unsigned n_part, unsigned n_ref, unsigned n_shift, unsigned* err, cudaStream_t stream)
{
    if (n_part == 0 || n_ref == 0)
        return cudaSuccess;
    SplitMmaWork mw;
    mw.sop = sop;
    mw.rop = rop;
    mw.z = z;
    mw.n_part = n_part;
    mw.n_blocks = p.n_blocks;
    mw.block = p.block;
    mw.n_shift = n_shift;
    mw.n_ref = n_ref;
    mw.rblock = p.rblock;
    mw.n_rtiles = p.n_rtiles;
    mw.kg = p.kg;
    mw.rga = p.rga;
    mw.rgb = p.rgb;
    mw.n_cols = p.n_cols;
    mw.n_stages = p.n_stages;
    mw.zw = p.zw;
    mw.sop_slot = p.sop_slot;
    mw.rop_slot = p.rop_slot;
    mw.n_items = n_part * p.n_blocks * p.n_rtiles;
    ccf_test_settings(mw.test_stall, mw.wait_iters);
    const size_t ms = mma_smem(p);
    cudaError_t e = opt_in_smem_k(ccf_mma_kernel, ms);
    if (e != cudaSuccess)
        return e;
    ccf_mma_kernel<<<std::min<unsigned>(mw.n_items, device_sms()), kMmaThreads, ms, stream>>>(mw, err);
    g_kernel_launches.fetch_add(1, std::memory_order_relaxed);
    return cudaGetLastError();
}

cudaError_t launch_zfft_peak(const SplitPlan& p, const float2* z, unsigned n_part, unsigned p_first,
                             unsigned p_total, unsigned n_ref, unsigned n_shift, const float2* twiddle,
                             const float2* shifts_f, const float2* base, float* d_out, float4* peak_out,
                             unsigned* err, cudaStream_t stream, unsigned rule)
{
    if (n_part == 0 || n_ref == 0)
        return cudaSuccess;
    SplitFftWork fw;
    fw.z = z;
    fw.n_part = n_part;
    fw.n_ref = n_ref;
    fw.n_shift = n_shift;
    fw.n_blocks = p.n_blocks;
    fw.block = p.block;
    fw.zw = p.zw;
    fw.p_first = p_first;
    fw.p_total = p_total;
    fw.shifts_f = shifts_f;
    fw.base = base;
    fw.d_out = d_out;
    fw.peak_out = peak_out;
    fw.rule = rule;
    ccf_test_settings(fw.test_stall, fw.wait_iters);
    const size_t fs = fft_smem(p);
    const unsigned grid = std::min<unsigned>(n_part * n_ref, device_sms());
    cudaError_t e;
    if ((e = opt_in_smem_k(zfft_peak_kernel, fs)) != cudaSuccess)
        return e;
    zfft_peak_kernel<<<grid, zfft_group_threads(p.fft_groups) + kZfftCtlThreads, fs, stream>>>(fw, twiddle, err);
    g_kernel_launches.fetch_add(1, std::memory_order_relaxed);
    return cudaGetLastError();
}

} // namespace gpuisac
