// ccf_peak.cu -- ring-weighted cross-correlation of every (particle, shift)
// against a tile of references, the inverse angular FFT and the peak search
// over reference x angle x shift x mirror, fused: the per-pair spectra never
// leave the SM.
//
// Reference semantics: cu_ccf_mult_mref (cuda/gpu_aln_noref.cu:1483-1537), the
// C2R of every ccf-table entry (:2453-2461), cu_aln_param_wizard (:1667-1794)
// and the host scatter of multi_ref_align (:516-541).
//
// Every kernel runs 16 (shift, reference) pairs per shift group (8 with 2
// shifts per group) through three stages:
//   contraction  the four sums that form Z[k] and Z[256-k] (Z = O + iM, see
//                polar_spectra.cu) for every slot k;
//   inverse FFT  16 groups of 16 threads, one 256-point FFT per pair; real part
//                = normal correlation, imaginary part = mirrored;
//   peak search  first strict maximum in the reference's scan order
//                (mirror-major, then shift, then angle), kept per pair slot
//                with the 7 samples around it; merged per reference at the
//                end of the particle, then the 7-point parabola.
//
// ccf_peak_ws_kernel<CW, NSI, QR> (up to 64 rings; the default): warp-
//   specialised, CW contraction warps with the 4 references in tensor memory
//   and the subject spectra staged by bulk async copies, and one 16-thread
//   FFT / peak group per pair running the previous shift group at the same
//   time; an item's (particle, shift) rows stream through the shift groups.
// ccf_peak_tmem_kernel (up to 36 rings): 4 references per CTA held in tensor
//   memory (lane = spectrum slot k, which is exactly the lane the thread
//   owning slot k may read), split by ring halves across the two 128-thread
//   halves (thread = slot k x half); the subject spectra of 4 shifts are
//   staged into shared memory by bulk async copies (mbarrier, bounded wait)
//   issued as soon as the previous contraction is done, so they overlap the
//   FFT phase; the halves exchange partial sums through shared memory.
// ccf_peak_kernel<QT> (any ring count up to the library maximum): QT
//   references in shared memory, subject spectra loaded into registers in
//   ring chunks.
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <map>
#include <mutex>

#include "ccf_device.cuh"
#include "gpuisac_device.cuh"
#include "gpuisac_kernels.h"

namespace gpuisac {

// spectra row of the group's q-th reference
__device__ __forceinline__ unsigned ref_row(const CcfGroup& g, unsigned q) { return g.ref_idx ? g.ref_idx[q] : q; }

// ---- work items ----
// Work item = (group, reference tile, block of up to ppc particles).  Items of
// a group are numbered reference tile fastest, so consecutive items (running
// on different SMs at the same time) read the same particles' spectra.
__device__ __forceinline__ bool decode_item(const CcfWork& w, unsigned item, int qt, CcfGroup& grp, unsigned& q0,
                                            unsigned& pb, unsigned& pe)
{
    if (item >= (w.dyn ? __ldg(w.dyn + 2) : w.n_items))
        return false;
    if (w.groups == nullptr) {
        grp = w.one;
    } else {
        const CcfGroup* groups = w.dyn ? w.groups + __ldg(w.dyn) : w.groups;
        unsigned lo = 0, hi = (w.dyn ? __ldg(w.dyn + 1) : w.n_groups) - 1; // last group with item_begin <= item
        while (lo < hi) {
            const unsigned mid = (lo + hi + 1) >> 1;
            if (groups[mid].item_begin <= item)
                lo = mid;
            else
                hi = mid - 1;
        }
        grp = groups[lo];
    }
    const unsigned local = item - grp.item_begin;
    const unsigned tile = local % grp.ref_tiles, blk = local / grp.ref_tiles;
    q0 = tile * (unsigned)qt;
    pb = blk * w.ppc;
    pe = min(grp.n_part, pb + w.ppc);
    return pb < pe;
}

// ring-half kernel: references in tensor memory, subject spectra staged into
// shared memory by bulk async copies (ring_num <= kTmaMaxRings); persistent
// over work items
constexpr int kTmemRingsPerHalf = 18;
constexpr uint32_t kTmemCols = 512;

__global__ void __launch_bounds__(256, 1)
ccf_peak_tmem_kernel(CcfWork w, const float2* __restrict__ twiddle, unsigned ring_num, unsigned n_shift,
                     const float2* __restrict__ shifts_f, unsigned* __restrict__ err)
{
    constexpr int QT = 4, NSI = 4;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const unsigned nrp = 2 * ((ring_num + 1) / 2); // rings per staged shift (one zero ring if odd)
    float2* sbuf = reinterpret_cast<float2*>(smem_raw);                // [NSI][nrp][kSlots]
    float2* zbuf = sbuf + (size_t)NSI * nrp * kSlots;                  // [16][kPairStride]
    float2* tw = zbuf + 16 * kPairStride;                              // [256]
    PeakSlot* slots = reinterpret_cast<PeakSlot*>(tw + kRingLen);      // [16]
    uint64_t* bar = reinterpret_cast<uint64_t*>(slots + 16);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bar + 1);

    const int tid = threadIdx.x;
    const int warp = tid >> 5;
    const int k = tid & (kSlots - 1);
    const int half = tid >> 7;

    unsigned item = blockIdx.x;
    CcfGroup grp;
    unsigned q0, pb, pe;
    if (!decode_item(w, item, QT, grp, q0, pb, pe))
        return;

    tw[tid] = twiddle[tid];
    for (unsigned i = tid; i < (unsigned)NSI * nrp * kSlots; i += 256)
        sbuf[i] = make_float2(0.f, 0.f); // the padding ring stays zero
    if (warp == 0)
        tmem_alloc(tmem_slot, kTmemCols);
    if (tid == 0) {
        mbar_init(bar, 1);
        mbar_fence_init();
    }
    tmem_fence_before();
    __syncthreads();
    tmem_fence_after();
    // lane k of the tensor memory holds slot k; columns: [ring][ref][u, v]
    const uint32_t tmem = *tmem_slot + ((uint32_t)(32 * (warp & 3)) << 16);
    const uint32_t row_bytes = ring_num * kSlots * sizeof(float2);

    const uint32_t wlim = wait_tries(w.wait_iters);
    // copies of shift group s0 of particle p of group g (called by thread 0)
    auto issue = [&](const CcfGroup& gg, unsigned p, unsigned s0) {
        const float2* sp = gg.sbj_sp;
        if (w.test_stall)
            return;
        unsigned nv = min((unsigned)NSI, n_shift - s0);
        fence_proxy_async();
        mbar_expect_tx(bar, nv * row_bytes);
        for (unsigned i = 0; i < nv; i++) {
            const size_t at = ((size_t)p * n_shift + s0 + i) * ring_num * kSlots;
            if (GPUISAC_IN_BOUNDS(kChkCcfRow, at + (size_t)ring_num * kSlots - 1,
                                  (size_t)gg.n_part * n_shift * ring_num * kSlots))
                bulk_g2s(sbuf + (size_t)i * nrp * kSlots, sp + at, row_bytes, bar);
        }
    };
    if (tid == 0)
        issue(grp, pb, 0);
    uint32_t phase = 0;
    bool failed = false;

    const int g = tid >> 4, l = tid & 15;
    const unsigned gmask = 0xffffu << (tid & 16);
    const int g_shift = g / QT;
    float2* gz = zbuf + g * kPairStride;

    while (!failed) {
        // this item's references -> tensor memory, columns [ring][ref][u, v]
        // of lane k; the two halves store alternate ring pairs and both read
        // every ring
        for (unsigned j = 2 * half; j < nrp; j += 4) {
#pragma unroll
            for (int jj = 0; jj < 2; jj++) {
                float v[8];
#pragma unroll
                for (int q = 0; q < QT; q++) {
                    float2 uv = make_float2(0.f, 0.f);
                    if (j + jj < ring_num && q0 + q < grp.n_ref)
                        uv = __ldg(&grp.ref_sp[((size_t)ref_row(grp, q0 + q) * ring_num + j + jj) * kSlots + k]);
                    v[2 * q] = uv.x;
                    v[2 * q + 1] = uv.y;
                }
                tmem_st8(tmem + (j + jj) * 8, v);
            }
        }
        tmem_wait_st();
        tmem_fence_before();
        __syncthreads();
        tmem_fence_after();
        // the item after this one, for the copies issued at its end
        CcfGroup ngrp;
        unsigned nq0 = 0, npb = 0, npe = 0;
        const bool has_next = decode_item(w, item + gridDim.x, QT, ngrp, nq0, npb, npe);

        for (unsigned p = pb; p < pe && !failed; p++) {
            PeakState st;
            st.reset(grp.rule);
            for (unsigned s0 = 0; s0 < n_shift; s0 += NSI) {
                // ---- wait for this group's spectra (bounded) ----
                const bool ok = mbar_wait(bar, phase, wlim);
                if (!__syncthreads_and(ok)) {
                    failed = true;
                    break;
                }
                phase ^= 1u;
                // ---- contraction: every ring, this half's 2 shifts x 4 references ----
                float acc[QT][2][4];
#pragma unroll
                for (int q = 0; q < QT; q++)
#pragma unroll
                    for (int i = 0; i < 2; i++)
#pragma unroll
                        for (int c = 0; c < 4; c++)
                            acc[q][i][c] = 0.f;
                const float2* sb = sbuf + (size_t)(2 * half) * nrp * kSlots + k;
                // rings j, j+1 from 16 columns; the next pair's load is in
                // flight while this pair is used
                auto ring_pair = [&](const float (&rv)[16], unsigned j) {
#pragma unroll
                    for (int jj = 0; jj < 2; jj++) {
                        if (j + jj < ring_num) {
                            const float2 a0 = sb[(size_t)(j + jj) * kSlots];
                            const float2 a1 = sb[(size_t)(nrp + j + jj) * kSlots];
#pragma unroll
                            for (int q = 0; q < QT; q++) {
                                const float u = rv[jj * 8 + 2 * q], vv = rv[jj * 8 + 2 * q + 1];
                                acc[q][0][0] = fmaf(u, a0.x, acc[q][0][0]);
                                acc[q][0][1] = fmaf(u, a0.y, acc[q][0][1]);
                                acc[q][0][2] = fmaf(vv, a0.y, acc[q][0][2]);
                                acc[q][0][3] = fmaf(vv, a0.x, acc[q][0][3]);
                                acc[q][1][0] = fmaf(u, a1.x, acc[q][1][0]);
                                acc[q][1][1] = fmaf(u, a1.y, acc[q][1][1]);
                                acc[q][1][2] = fmaf(vv, a1.y, acc[q][1][2]);
                                acc[q][1][3] = fmaf(vv, a1.x, acc[q][1][3]);
                            }
                        }
                    }
                };
                {
                    float ra[16], rb[16];
                    tmem_ld16_async(tmem, ra);
                    tmem_wait_ld16(ra);
                    for (unsigned j = 0; j < nrp; j += 4) {
                        const bool more_b = j + 2 < nrp;
                        if (more_b)
                            tmem_ld16_async(tmem + (j + 2) * 8, rb);
                        ring_pair(ra, j);
                        if (!more_b)
                            break;
                        tmem_wait_ld16(rb);
                        const bool more_a = j + 4 < nrp;
                        if (more_a)
                            tmem_ld16_async(tmem + (j + 4) * 8, ra);
                        ring_pair(rb, j + 2);
                        if (more_a)
                            tmem_wait_ld16(ra);
                    }
                }
                tmem_fence_before();
                __syncthreads(); // staging area read by everyone; previous FFT phase done with zbuf
                tmem_fence_after();
                // next copies overlap the FFT phase
                if (tid == 0) {
                    if (s0 + NSI < n_shift)
                        issue(grp, p, s0 + NSI);
                    else if (p + 1 < pe)
                        issue(grp, p + 1, 0);
                    else if (has_next)
                        issue(ngrp, npb, 0);
                }
#pragma unroll
                for (int ii = 0; ii < 2; ii++)
#pragma unroll
                    for (int q = 0; q < QT; q++)
                        write_z(zbuf + ((2 * half + ii) * QT + q) * kPairStride, k, acc[q][ii][0], acc[q][ii][1],
                                acc[q][ii][2], acc[q][ii][3]);
                __syncthreads();
                // ---- inverse FFT + peak search, one pair per 16-thread group ----
                const unsigned s = s0 + g_shift;
                // pairs of reference slots the group does not fill stay idle
                if (s < n_shift && q0 + (unsigned)(g % QT) < grp.n_ref)
                    fft_peak(gz, tw, l, gmask, s, n_shift, st, grp.rule);
            }
            if (failed)
                break;
            merge_write(slots, st, tid, g, l, QT, NSI, q0, grp.n_ref, n_shift, grp.p_first + p, grp.p_total, shifts_f,
                        grp.base, grp.d_out, grp.peak_out, grp.rule);
        }
        if (failed || !has_next)
            break;
        item += gridDim.x;
        grp = ngrp;
        q0 = nq0;
        pb = npb;
        pe = npe;
        tmem_fence_after();
    }
    if (failed && tid == 0) {
        atomicExch(err, 1u);
        if (!w.test_stall)
            mbar_wait(bar, phase, wlim); // let copies in flight land before leaving
    }
    // release the tensor memory (all tcgen05 accesses of the CTA are done)
    tmem_fence_before();
    __syncthreads();
    tmem_fence_after();
    if (warp == 0)
        tmem_dealloc(*tmem_slot, kTmemCols);
}

// ============================================================================
// warp-specialised tensor-memory kernel: 512 threads.  Threads 0..255 stage
// the subject spectra and run the contraction (references in tensor memory,
// as above); threads 256..511 run the inverse FFTs and the peak search of the
// previous shift group at the same time.  The two sides hand over the 16
// pair spectra through two shared-memory buffers guarded by named barriers
// (FULL: contraction -> FFT, EMPTY: FFT -> contraction).
constexpr int kWsBarC = 1;     // contraction side only (256 threads)
constexpr int kWsBarFull = 2;  // + buffer: 2, 3
constexpr int kWsBarEmpty = 4; // + buffer: 4, 5
constexpr int kWsBarF = 6;     // FFT side only (256 threads)

// CW contraction warps (slot k x NSI*128/(32 CW) shifts per thread) + one
// 16-thread FFT group per pair of the shift group (NSI shifts x 4 references).
// NSI = 4 up to kTmaMaxRings rings; NSI = 2 halves the staging area for up
// to kWsMaxRings rings (the references' tensor-memory columns bound both).
// QR: reference slots the contraction sums (4; 1 when every group of the
// launch has one reference -- the other slots' pairs stay idle).
template <int CW, int NSI, int QR>
__global__ void __launch_bounds__(32 * CW + NSI * 64, 1)
ccf_peak_ws_kernel(CcfWork w, const float2* __restrict__ twiddle, unsigned ring_num, unsigned n_shift,
                   const float2* __restrict__ shifts_f, unsigned* __restrict__ err)
{
    constexpr int QT = 4;
    constexpr int NP = NSI * QT;        // pairs per shift group
    constexpr int NC = 32 * CW;         // contraction threads
    constexpr int NF = 16 * NP;         // FFT / peak threads
    constexpr int NT = NC + NF;         // all threads
    constexpr int SPT = NSI * 128 / NC; // shifts per contraction thread
    static_assert((CW == 4 || CW == 8) && (NSI == 2 || NSI == 4) && SPT >= 1, "tile shape");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const unsigned nrp = 2 * ((ring_num + 1) / 2); // rings per staged shift (one zero ring if odd)
    float2* sbuf = reinterpret_cast<float2*>(smem_raw);                // [NSI][nrp][kSlots]
    float2* zbuf = sbuf + (size_t)NSI * nrp * kSlots;                  // [2][NP][kPairStride]
    float2* tw = zbuf + 2 * NP * kPairStride;                          // [16][kTwRow] per FFT lane
    PeakSlot* slots = reinterpret_cast<PeakSlot*>(tw + 16 * kTwRow);   // [16]
    uint64_t* bar = reinterpret_cast<uint64_t*>(slots + 16);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bar + 1);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
    // the item after the current one, by item parity: taken from the work
    // counter (w.item_counter) by the contraction side's thread 0, read by
    // both sides
    volatile unsigned* next_item = reinterpret_cast<volatile unsigned*>(abort_flag + 1);

    const int tid = threadIdx.x;
    const int warp = tid >> 5;
    const bool contraction_side = tid < NC;
    // An item's (particle, shift) rows run through the shift groups as one
    // stream, particle-major: with n_shift >= NSI a group may hold the end of
    // one particle and the start of the next, so no group is left part empty
    // at a particle's end.  Below NSI shifts every particle is padded to whole
    // groups.  Row v of the item is particle v / vstride, shift v % vstride.
    const unsigned vstride = n_shift >= (unsigned)NSI ? n_shift : (n_shift + NSI - 1) / NSI * NSI;

    unsigned item = blockIdx.x;
    CcfGroup grp;
    unsigned q0, pb, pe;
    if (!decode_item(w, item, QT, grp, q0, pb, pe))
        return;

    if (tid < kRingLen) { // lane l's inverse-FFT twiddles, row l
        const int tl = tid >> 4, tj = tid & 15;
        const float2 t = twiddle[(tl * tj) & (kRingLen - 1)];
        tw[tl * kTwRow + tj] = make_float2(t.x, t.y * -1.f);
    }
    for (unsigned i = tid; i < (unsigned)NSI * nrp * kSlots; i += NT)
        sbuf[i] = make_float2(0.f, 0.f); // the padding ring stays zero
    if (warp == 0)
        tmem_alloc(tmem_slot, kTmemCols);
    if (tid == 0) {
        mbar_init(bar, 1);
        mbar_fence_init();
        *abort_flag = 0;
    }
    tmem_fence_before();
    __syncthreads();
    tmem_fence_after();

    bool failed = false;
    uint32_t phase = 0;
    if (contraction_side) {
        // ================= contraction side =================
        const int k = tid & (kSlots - 1);
        const int half = tid >> 7; // which SPT shifts of the group (0 when CW = 4)
        // lane k of the tensor memory holds slot k; columns: [ring][ref][u, v]
        const uint32_t tmem = *tmem_slot + ((uint32_t)(32 * (warp & 3)) << 16);
        const uint32_t row_bytes = ring_num * kSlots * sizeof(float2);
        // the shift group of rows v0..v0+NSI-1 (item-local) of the item whose
        // particles start at p0 and number np
        const uint32_t wlim = wait_tries(w.wait_iters);
        // returns whether copies were issued
        auto issue = [&](const CcfGroup& gg, unsigned p0, unsigned np, unsigned v0) -> bool {
            const float2* sp = gg.sbj_sp;
            if (w.test_stall)
                return false;
            unsigned nv = 0;
            for (unsigned i = 0; i < (unsigned)NSI; i++) {
                const unsigned v = v0 + i, pl = v / vstride;
                nv += (pl < np && v - pl * vstride < n_shift) ? 1u : 0u;
            }
            fence_proxy_async();
            mbar_expect_tx(bar, nv * row_bytes);
            for (unsigned i = 0; i < (unsigned)NSI; i++) {
                const unsigned v = v0 + i, pl = v / vstride, sv = v - pl * vstride;
                const size_t at = ((size_t)(p0 + pl) * n_shift + sv) * ring_num * kSlots;
                if (pl < np && sv < n_shift &&
                    GPUISAC_IN_BOUNDS(kChkCcfRow, at + (size_t)ring_num * kSlots - 1,
                                      (size_t)gg.n_part * n_shift * ring_num * kSlots))
                    bulk_g2s(sbuf + (size_t)i * nrp * kSlots, sp + at, row_bytes, bar);
            }
            return true;
        };
        bool pending = false; // thread 0: copies in flight
        if (tid == 0)
            pending = issue(grp, pb, pe - pb, 0);
        unsigned it = 0, ii = 0;
        while (!failed) {
            if (tid == 0)
                next_item[ii & 1u] = w.item_counter ? gridDim.x + atomicAdd(w.item_counter, 1u) : item + gridDim.x;
            // this item's references -> tensor memory (both halves read every ring)
            for (unsigned j = 2 * half; j < nrp; j += 2 * (NC / 128)) {
#pragma unroll
                for (int jj = 0; jj < 2; jj++) {
                    float v[8];
#pragma unroll
                    for (int q = 0; q < QT; q++) {
                        float2 uv = make_float2(0.f, 0.f);
                        if (j + jj < ring_num && q0 + q < grp.n_ref)
                            uv = __ldg(&grp.ref_sp[((size_t)ref_row(grp, q0 + q) * ring_num + j + jj) * kSlots + k]);
                        v[2 * q] = uv.x;
                        v[2 * q + 1] = uv.y;
                    }
                    tmem_st8(tmem + (j + jj) * 8, v);
                }
            }
            tmem_wait_st();
            tmem_fence_before();
            nbar_sync(kWsBarC, NC);
            tmem_fence_after();
            CcfGroup ngrp;
            unsigned nq0 = 0, npb = 0, npe = 0;
            const unsigned nxt = next_item[ii & 1u];
            const bool has_next = decode_item(w, nxt, QT, ngrp, nq0, npb, npe);

            const unsigned nrows = (pe - pb) * vstride;
            for (unsigned v0 = 0; v0 < nrows && !failed; v0 += NSI, it++) {
                {
                    const unsigned b = it & 1u;
                    // ---- wait for this group's spectra (bounded) ----
                    const bool ok = mbar_wait(bar, phase, wlim);
                    if (ok && tid == 0)
                        pending = false;
                    if (!nbar_and(kWsBarC, NC, ok)) {
                        // hand the FFT side an empty buffer marked abort
                        failed = true;
                        nbar_sync(kWsBarEmpty + b, NT);
                        if (tid == 0)
                            *abort_flag = 1;
                        __threadfence_block();
                        nbar_arrive(kWsBarFull + b, NT);
                        break;
                    }
                    phase ^= 1u;
                    float acc[QR][SPT][4];
#pragma unroll
                    for (int q = 0; q < QR; q++)
#pragma unroll
                        for (int i = 0; i < SPT; i++)
#pragma unroll
                            for (int c = 0; c < 4; c++)
                                acc[q][i][c] = 0.f;
                    const float2* sb = sbuf + (size_t)(SPT * half) * nrp * kSlots + k;
                    // The zero ring that pads an odd ring count is summed like
                    // the others: it is zero in both the staging area and the
                    // tensor memory, and an accumulator that starts at +0 is
                    // never -0 under round-to-nearest, so adding 0 * 0 leaves
                    // every sum bit for bit as it was (and the loop has no
                    // per-ring branch).
                    auto ring_pair = [&](const float (&rv)[16], unsigned j) {
                        float2 pa[2][SPT];
#pragma unroll
                        for (int jj = 0; jj < 2; jj++)
#pragma unroll
                            for (int i = 0; i < SPT; i++)
                                pa[jj][i] = sb[(size_t)(i * nrp + j + jj) * kSlots];
#pragma unroll
                        for (int jj = 0; jj < 2; jj++) {
#pragma unroll
                            for (int q = 0; q < QR; q++) {
                                const float u = rv[jj * 8 + 2 * q], vv = rv[jj * 8 + 2 * q + 1];
#pragma unroll
                                for (int i = 0; i < SPT; i++) {
                                    const float2 a = pa[jj][i];
                                    acc[q][i][0] = fmaf(u, a.x, acc[q][i][0]);
                                    acc[q][i][1] = fmaf(u, a.y, acc[q][i][1]);
                                    acc[q][i][2] = fmaf(vv, a.y, acc[q][i][2]);
                                    acc[q][i][3] = fmaf(vv, a.x, acc[q][i][3]);
                                }
                            }
                        }
                    };
                    {
                        // four rings per iteration, the next ring pair's
                        // columns in flight; the load after the last pair
                        // re-reads that pair (address clamped inside the
                        // allocation) instead of a branch; an odd last pair
                        // of rings follows the loop
                        float ra[16], rb[16];
                        tmem_ld16_async(tmem, ra);
                        tmem_wait_ld16(ra);
                        const unsigned n4 = nrp >> 2;
                        for (unsigned t = 0; t < n4; t++) {
                            const unsigned j = 4 * t;
                            tmem_ld16_async(tmem + (j + 2) * 8, rb);
                            ring_pair(ra, j);
                            tmem_wait_ld16(rb);
                            tmem_ld16_async(tmem + min(j + 4, nrp - 2) * 8, ra);
                            ring_pair(rb, j + 2);
                            tmem_wait_ld16(ra);
                        }
                        if (nrp & 2u)
                            ring_pair(ra, nrp - 2);
                    }
                    tmem_fence_before();
                    nbar_sync(kWsBarC, NC); // the staging area is consumed
                    tmem_fence_after();
                    if (tid == 0) {
                        if (v0 + NSI < nrows)
                            pending = issue(grp, pb, pe - pb, v0 + NSI);
                        else if (has_next)
                            pending = issue(ngrp, npb, npe - npb, 0);
                    }
                    // ---- hand the pair spectra to the FFT side ----
                    float2* zb = zbuf + (size_t)b * NP * kPairStride;
                    nbar_sync(kWsBarEmpty + b, NT);
#pragma unroll
                    for (int ii = 0; ii < SPT; ii++)
#pragma unroll
                        for (int q = 0; q < QR; q++)
                            write_z(zb + ((SPT * half + ii) * QT + q) * kPairStride, k, acc[q][ii][0], acc[q][ii][1],
                                    acc[q][ii][2], acc[q][ii][3]);
                    __threadfence_block();
                    nbar_arrive(kWsBarFull + b, NT);
                }
            }
            if (failed || !has_next)
                break;
            item = nxt;
            ii++;
            grp = ngrp;
            q0 = nq0;
            pb = npb;
            pe = npe;
            // the next item's references overwrite tensor memory: every
            // contraction of this item is done
            tmem_fence_before();
            nbar_sync(kWsBarC, NC);
            tmem_fence_after();
        }
        if (failed && tid == 0) {
            atomicExch(err, 1u);
            if (pending)
                mbar_wait(bar, phase, wlim); // let copies in flight land before leaving (bounded)
        }
    } else {
        // ================= FFT / peak side =================
        const int ftid = tid - NC;
        const int g = ftid >> 4, l = ftid & 15;
        const unsigned gmask = 0xffffu << (ftid & 16);
        const int g_shift = g / QT;
        // both buffers start empty
        nbar_arrive(kWsBarEmpty + 0, NT);
        nbar_arrive(kWsBarEmpty + 1, NT);
        unsigned it = 0, ii = 0;
        while (!failed) {
            // st: the slot's running best of particle pb + pc, the particle of
            // the shift group's first row.  In the group that holds pc's last
            // row, a slot whose row already belongs to pc + 1 parks its best
            // of pc before starting afresh, the others after their row; then
            // the slots are merged for pc.
            const unsigned nrows = (pe - pb) * vstride;
            unsigned pc = 0;
            PeakState st;
            st.reset(grp.rule);
            for (unsigned v0 = 0; v0 < nrows; v0 += NSI, it++) {
                const unsigned b = it & 1u;
                nbar_sync(kWsBarFull + b, NT);
                if (*abort_flag) {
                    failed = true;
                    break;
                }
                float2* gz = zbuf + (size_t)b * NP * kPairStride + g * kPairStride;
                const unsigned v = v0 + g_shift, pl = v / vstride, s = v - pl * vstride;
                const bool last = (pc + 1) * vstride <= v0 + NSI; // pc's last row is in this group
                const bool next = pl != pc;                        // the same on both groups of a warp
                if (last && next) {
                    park_slot(slots, st, g, l);
                    st.reset(grp.rule);
                }
                // pairs of reference slots the group does not fill stay idle
                if (v < nrows && s < n_shift && q0 + (unsigned)(g % QT) < grp.n_ref)
                    fft_peak<true>(gz, tw + l * kTwRow, l, gmask, s, n_shift, st, grp.rule);
                __threadfence_block();
                nbar_arrive(kWsBarEmpty + b, NT);
                if (last) {
                    if (!next) {
                        park_slot(slots, st, g, l);
                        st.reset(grp.rule);
                    }
                    merge_slots<kWsBarF, NF>(slots, ftid, QT, NSI, q0, grp.n_ref, n_shift, grp.p_first + pb + pc,
                                             grp.p_total, shifts_f, grp.base, grp.d_out, grp.peak_out, grp.rule);
                    pc++;
                }
            }
            if (failed)
                break;
            // (written by the contraction side before this item's first full buffer)
            CcfGroup ngrp;
            unsigned nq0 = 0, npb = 0, npe = 0;
            const unsigned nxt = next_item[ii & 1u];
            if (!decode_item(w, nxt, QT, ngrp, nq0, npb, npe))
                break;
            item = nxt;
            ii++;
            grp = ngrp;
            q0 = nq0;
            pb = npb;
            pe = npe;
        }
    }
    // release the tensor memory (all tcgen05 accesses of the CTA are done)
    tmem_fence_before();
    __syncthreads();
    tmem_fence_after();
    if (warp == 0)
        tmem_dealloc(*tmem_slot, kTmemCols);
}

// ============================================================================
// general kernel: references in shared memory, subject spectra in registers;
// persistent over work items
template <int QT>
__global__ void __launch_bounds__(256, 1)
ccf_peak_kernel(CcfWork w, const float2* __restrict__ twiddle, unsigned ring_num, unsigned n_shift,
                const float2* __restrict__ shifts_f)
{
    constexpr int NSI = 16 / QT; // shifts per iteration
    constexpr int RPT = QT / 2;  // references per thread
    constexpr int RC = 32 / NSI; // rings per register chunk
    static_assert(RC <= (int)kRingPad && kRingPad % RC == 0, "ring chunk must divide the padding");

    extern __shared__ __align__(16) unsigned char smem_raw[];
    const unsigned nrp = ring_pad(ring_num);
    float2* rsp = reinterpret_cast<float2*>(smem_raw);    // [QT][nrp][kSlots]
    float2* zbuf = rsp + (size_t)QT * nrp * kSlots;       // [16][kPairStride]
    float2* tw = zbuf + 16 * kPairStride;                  // [256]
    PeakSlot* slots = reinterpret_cast<PeakSlot*>(tw + kRingLen); // [16]

    const int tid = threadIdx.x;
    const int k = tid & (kSlots - 1);
    const int half = tid >> 7;
    tw[tid] = twiddle[tid];

    const int g = tid >> 4, l = tid & 15;
    const unsigned gmask = 0xffffu << (tid & 16);
    const int g_shift = g / QT;
    float2* gz = zbuf + g * kPairStride;
    const unsigned n_chunks = nrp / RC;

    for (unsigned item = blockIdx.x;; item += gridDim.x) {
        CcfGroup grp;
        unsigned q0, pb, pe;
        if (!decode_item(w, item, QT, grp, q0, pb, pe))
            break;
        __syncthreads(); // previous item is done with the reference tile
        // reference tile -> shared memory (zero padded rings / missing refs)
        for (unsigned idx = tid; idx < (unsigned)QT * nrp * kSlots; idx += 256) {
            unsigned qq = idx / (nrp * kSlots);
            unsigned rem = idx - qq * nrp * kSlots;
            unsigned r = rem / kSlots, kk = rem - r * kSlots;
            float2 v = make_float2(0.f, 0.f);
            if (q0 + qq < grp.n_ref && r < ring_num)
                v = __ldg(&grp.ref_sp[((size_t)ref_row(grp, q0 + qq) * ring_num + r) * kSlots + kk]);
            rsp[idx] = v;
        }
        __syncthreads();

        for (unsigned p = pb; p < pe; p++) {
            PeakState st;
            st.reset(grp.rule);
            for (unsigned s0 = 0; s0 < n_shift; s0 += NSI) {
                float acc[RPT][NSI][4];
#pragma unroll
                for (int j = 0; j < RPT; j++)
#pragma unroll
                    for (int i = 0; i < NSI; i++)
#pragma unroll
                        for (int c = 0; c < 4; c++)
                            acc[j][i][c] = 0.f;

                const float2* srow[NSI];
                bool svalid[NSI];
#pragma unroll
                for (int i = 0; i < NSI; i++) {
                    unsigned s = s0 + i;
                    svalid[i] = s < n_shift;
                    srow[i] = grp.sbj_sp + ((size_t)p * n_shift + (svalid[i] ? s : 0)) * ring_num * kSlots + k;
                }
                // ring chunks in two register buffers used alternately: the next
                // chunk's loads are in flight while the current one is consumed
                float2 bufa[NSI][RC], bufb[NSI][RC];
                auto load = [&](float2 (&dst)[NSI][RC], unsigned r0) {
#pragma unroll
                    for (int i = 0; i < NSI; i++)
#pragma unroll
                        for (int rr = 0; rr < RC; rr++)
                            dst[i][rr] = (svalid[i] && r0 + rr < ring_num)
                                             ? __ldg(srow[i] + (size_t)(r0 + rr) * kSlots)
                                             : make_float2(0.f, 0.f);
                };
                auto consume = [&](const float2 (&src)[NSI][RC], unsigned r0) {
#pragma unroll
                    for (int j = 0; j < RPT; j++) {
                        const float2* rq = rsp + ((size_t)(half * RPT + j) * nrp + r0) * kSlots + k;
#pragma unroll
                        for (int rr = 0; rr < RC; rr++) {
                            const float2 uv = rq[rr * kSlots];
#pragma unroll
                            for (int i = 0; i < NSI; i++) {
                                const float2 ab = src[i][rr];
                                acc[j][i][0] = fmaf(uv.x, ab.x, acc[j][i][0]);
                                acc[j][i][1] = fmaf(uv.x, ab.y, acc[j][i][1]);
                                acc[j][i][2] = fmaf(uv.y, ab.y, acc[j][i][2]);
                                acc[j][i][3] = fmaf(uv.y, ab.x, acc[j][i][3]);
                            }
                        }
                    }
                };
                load(bufa, 0);
                for (unsigned c = 0; c < n_chunks; c += 2) {
                    if (c + 1 < n_chunks)
                        load(bufb, (c + 1) * RC);
                    consume(bufa, c * RC);
                    if (c + 1 < n_chunks) {
                        if (c + 2 < n_chunks)
                            load(bufa, (c + 2) * RC);
                        consume(bufb, (c + 1) * RC);
                    }
                }

                __syncthreads(); // previous FFT phase is done with zbuf
#pragma unroll
                for (int j = 0; j < RPT; j++)
#pragma unroll
                    for (int i = 0; i < NSI; i++)
                        write_z(zbuf + (i * QT + half * RPT + j) * kPairStride, k, acc[j][i][0], acc[j][i][1],
                                acc[j][i][2], acc[j][i][3]);
                __syncthreads();

                const unsigned s = s0 + g_shift;
                // pairs of reference slots the group does not fill stay idle
                if (s < n_shift && q0 + (unsigned)(g % QT) < grp.n_ref)
                    fft_peak(gz, tw, l, gmask, s, n_shift, st, grp.rule);
            }
            merge_write(slots, st, tid, g, l, QT, NSI, q0, grp.n_ref, n_shift, grp.p_first + p, grp.p_total, shifts_f,
                        grp.base, grp.d_out, grp.peak_out, grp.rule);
        }
    }
}

// ============================================================================
constexpr unsigned kTmaMaxRings = 2 * kTmemRingsPerHalf;

static size_t tma_smem_bytes(unsigned ring_num)
{
    unsigned nrp = 2 * ((ring_num + 1) / 2);
    return (size_t)4 * nrp * kSlots * sizeof(float2) + 16 * kPairStride * sizeof(float2) +
           kRingLen * sizeof(float2) + 16 * sizeof(PeakSlot) + 16;
}

// rings the warp-specialised kernel takes with 2 shifts per group: the 4
// references' (u, v) columns of every ring fill the 512 tensor-memory columns
constexpr unsigned kWsMaxRings = 64;

static unsigned ws_shifts_per_group(unsigned ring_num) { return ring_num <= kTmaMaxRings ? 4u : 2u; }

static size_t ws_smem_bytes(unsigned ring_num)
{
    const unsigned nrp = 2 * ((ring_num + 1) / 2), nsi = ws_shifts_per_group(ring_num);
    return (size_t)nsi * nrp * kSlots * sizeof(float2) + 2 * nsi * 4 * kPairStride * sizeof(float2) +
           16 * kTwRow * sizeof(float2) + 16 * sizeof(PeakSlot) + 16 + 16; // barrier, tensor-memory slot, abort, next items
}

template <int CW, int NSI, int QR>
static cudaError_t launch_ws(const CcfWork& w, unsigned grid, const float2* twiddle, unsigned ring_num,
                             unsigned n_shift, const float2* shifts_f, unsigned* err, cudaStream_t stream)
{
    cudaError_t e = set_max_smem(ccf_peak_ws_kernel<CW, NSI, QR>);
    if (e != cudaSuccess)
        return e;
    ccf_peak_ws_kernel<CW, NSI, QR><<<grid, 32 * CW + NSI * 64, ws_smem_bytes(ring_num), stream>>>(
        w, twiddle, ring_num, n_shift, shifts_f, err);
    return cudaSuccess;
}

// shared memory of the general kernel (references in shared memory) at any
// ring count
size_t ccf_peak_smem_bytes(unsigned ring_num)
{
    unsigned qt = ccf_refs_per_cta(ring_num);
    return (size_t)qt * ring_pad(ring_num) * kSlots * sizeof(float2) + 16 * kPairStride * sizeof(float2) +
           kRingLen * sizeof(float2) + 16 * sizeof(PeakSlot);
}

unsigned ccf_refs_per_item(unsigned ring_num, int variant)
{
    if ((variant == kCcfTmem && ring_num <= kTmaMaxRings) || (variant == kCcfWs && ring_num <= kWsMaxRings))
        return 4;
    return ccf_refs_per_cta(ring_num);
}

namespace {
std::mutex g_tile_mu;
std::map<std::pair<unsigned, unsigned>, CcfTile> g_tiles;
std::atomic<unsigned> g_tile_gen{0};
thread_local const CcfTile* t_forced = nullptr;
} // namespace

void ccf_tile_record(unsigned ring_num, unsigned n_shift, const CcfTile& t)
{
    std::lock_guard<std::mutex> lk(g_tile_mu);
    g_tiles[{ring_num, n_shift}] = t;
    g_tile_gen.fetch_add(1);
}

bool ccf_tile_lookup(unsigned ring_num, unsigned n_shift, CcfTile& t)
{
    std::lock_guard<std::mutex> lk(g_tile_mu);
    auto it = g_tiles.find({ring_num, n_shift});
    if (it == g_tiles.end())
        return false;
    t = it->second;
    return true;
}

void ccf_tile_force(const CcfTile* t) { t_forced = t; }

bool ccf_tile_allows_tmem(unsigned ring_num) { return ring_num <= kTmaMaxRings; }

unsigned ccf_tile_generation() { return g_tile_gen.load(); }

CcfTile ccf_tile(unsigned ring_num, unsigned n_shift, bool aligned)
{
    CcfTile t{kCcfWs, 8, kCcfParticlesPerItem};
    if (t_forced)
        t = *t_forced;
    else
        ccf_tile_lookup(ring_num, n_shift, t);
    // GPUISAC_CCF_KERNEL=general selects the general kernel for every ring
    // count, =tmem the single-phase tensor-memory kernel, =ws the
    // warp-specialised one; GPUISAC_CCF_WS_WARPS=4|8 its contraction warps
    const char* sel = getenv("GPUISAC_CCF_KERNEL");
    if (sel && strcmp(sel, "general") == 0)
        t.variant = kCcfGeneral;
    else if (sel && strcmp(sel, "tmem") == 0)
        t.variant = kCcfTmem;
    else if (sel && strcmp(sel, "ws") == 0)
        t.variant = kCcfWs;
    const char* cw = getenv("GPUISAC_CCF_WS_WARPS");
    if (cw && (strcmp(cw, "4") == 0 || strcmp(cw, "8") == 0))
        t.ws_warps = cw[0] - '0';
    if (!aligned || ring_num > kWsMaxRings)
        t.variant = kCcfGeneral;
    else if (ring_num > kTmaMaxRings && t.variant == kCcfTmem)
        t.variant = kCcfWs; // the single-phase kernel stages 4 shifts: up to kTmaMaxRings rings
    if (t.ws_warps != 4)
        t.ws_warps = 8;
    if (t.ppc == 0)
        t.ppc = kCcfParticlesPerItem;
    return t;
}

int ccf_variant(unsigned ring_num, bool aligned, unsigned n_shift) { return ccf_tile(ring_num, n_shift, aligned).variant; }

template <typename K>
static cudaError_t set_max_smem(K kernel)
{
    return opt_in_smem_k(kernel, (size_t)smem_optin_max());
}

static unsigned persistent_grid(unsigned n_items, unsigned ctas_per_sm)
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    unsigned cap = (unsigned)std::max(sms, 1) * std::max(ctas_per_sm, 1u);
    return std::max(1u, std::min(n_items, cap));
}

namespace {
std::atomic<unsigned> g_test_stall{0}, g_test_wait_iters{0};
} // namespace

GPUISAC_CHECKED_READER(checked_read_ccf)

void ccf_test_settings(unsigned& stall, unsigned& wait_iters)
{
    stall = g_test_stall.load();
    wait_iters = g_test_wait_iters.load();
}

cudaError_t launch_ccf_peak_work(const CcfWork& w_in, int variant, const float2* twiddle, unsigned ring_num,
                                 unsigned n_shift, const float2* shifts_f, unsigned* err, cudaStream_t stream)
{
    if (w_in.n_items == 0)
        return cudaSuccess;
    CcfWork w = w_in;
    ccf_test_settings(w.test_stall, w.wait_iters);
    const unsigned grid = persistent_grid(w.n_items, 1);
    if (variant != kCcfWs)
        w.item_counter = nullptr; // (the other kernels take items CTA + k x grid)
    else if (w.item_counter) {
        cudaError_t e = cudaMemsetAsync(w.item_counter, 0, sizeof(unsigned), stream);
        if (e != cudaSuccess)
            return e;
    }
    if (variant == kCcfWs) {
        const bool four = ccf_tile(ring_num, n_shift, true).ws_warps == 4;
        const bool one_ref = w.max_ref == 1;
        cudaError_t e;
        if (ring_num <= kTmaMaxRings) {
            if (one_ref)
                e = launch_ws<8, 4, 1>(w, grid, twiddle, ring_num, n_shift, shifts_f, err, stream);
            else
                e = four ? launch_ws<4, 4, 4>(w, grid, twiddle, ring_num, n_shift, shifts_f, err, stream)
                         : launch_ws<8, 4, 4>(w, grid, twiddle, ring_num, n_shift, shifts_f, err, stream);
        } else {
            if (one_ref)
                e = launch_ws<8, 2, 1>(w, grid, twiddle, ring_num, n_shift, shifts_f, err, stream);
            else
                e = four ? launch_ws<4, 2, 4>(w, grid, twiddle, ring_num, n_shift, shifts_f, err, stream)
                         : launch_ws<8, 2, 4>(w, grid, twiddle, ring_num, n_shift, shifts_f, err, stream);
        }
        if (e != cudaSuccess)
            return e;
    } else if (variant == kCcfTmem) {
        cudaError_t e = set_max_smem(ccf_peak_tmem_kernel);
        if (e != cudaSuccess)
            return e;
        ccf_peak_tmem_kernel<<<grid, 256, tma_smem_bytes(ring_num), stream>>>(w, twiddle, ring_num, n_shift, shifts_f,
                                                                              err);
    } else if (ccf_refs_per_cta(ring_num) == 4) {
        cudaError_t e = set_max_smem(ccf_peak_kernel<4>);
        if (e != cudaSuccess)
            return e;
        ccf_peak_kernel<4><<<grid, 256, ccf_peak_smem_bytes(ring_num), stream>>>(w, twiddle, ring_num, n_shift,
                                                                               shifts_f);
    } else {
        cudaError_t e = set_max_smem(ccf_peak_kernel<2>);
        if (e != cudaSuccess)
            return e;
        ccf_peak_kernel<2><<<grid, 256, ccf_peak_smem_bytes(ring_num), stream>>>(w, twiddle, ring_num, n_shift,
                                                                               shifts_f);
    }
    g_kernel_launches.fetch_add(1, std::memory_order_relaxed);
    return cudaGetLastError();
}

cudaError_t launch_ccf_peak(const float2* sbj_sp, const float2* ref_sp, const float2* twiddle, unsigned ring_num,
                            unsigned n_shift, unsigned n_ref, unsigned n_part, unsigned p_global0, unsigned p_total,
                            const float2* shifts_f, const float2* base, float* d_out, float4* peak_out,
                            unsigned* err, cudaStream_t stream, unsigned rule, unsigned* item_counter)
{
    if (n_part == 0 || n_ref == 0)
        return cudaSuccess;
    // bulk copies need 16-byte aligned sources (every row is a multiple of 1 KiB)
    const bool aligned = ((uintptr_t)sbj_sp & 15) == 0 && err != nullptr;
    const CcfTile tile = ccf_tile(ring_num, n_shift, aligned);
    const int variant = tile.variant;
    const unsigned qt = ccf_refs_per_item(ring_num, variant);
    CcfWork w{};
    w.groups = nullptr;
    w.n_groups = 1;
    w.ppc = tile.ppc;
    CcfGroup& g = w.one;
    g.sbj_sp = sbj_sp;
    g.ref_sp = ref_sp;
    g.base = base;
    g.d_out = d_out;
    g.peak_out = peak_out;
    g.p_first = p_global0;
    g.n_part = n_part;
    g.n_ref = n_ref;
    g.p_total = p_total;
    g.item_begin = 0;
    g.ref_tiles = (n_ref + qt - 1) / qt;
    g.rule = rule;
    w.n_items = g.ref_tiles * ((n_part + w.ppc - 1) / w.ppc);
    w.max_ref = n_ref;
    w.item_counter = item_counter;
    return launch_ccf_peak_work(w, variant, twiddle, ring_num, n_shift, shifts_f, err, stream);
}

} // namespace gpuisac

extern "C" void gpuisac_test_stall_ccf(unsigned int wait_iters)
{
    gpuisac::g_test_wait_iters.store(wait_iters);
    gpuisac::g_test_stall.store(wait_iters ? 1u : 0u);
}
