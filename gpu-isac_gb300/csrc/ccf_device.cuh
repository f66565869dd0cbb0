// ccf_device.cuh -- device pieces shared by the CCF / inverse-FFT / peak
// kernels (ccf_peak.cu, the FP32 contraction; ccf_split.cu, the tensor-core
// contraction): the peak search in the reference's scan order with its
// 7-point parabola, the named-barrier, mbarrier and bulk-copy helpers, and
// the tensor-memory helpers.
#pragma once

#include <stdint.h>

#include "gpuisac_device.cuh"
#include "gpuisac_kernels.h"

namespace gpuisac {

namespace {

struct PeakSlot {
    float v;
    unsigned h;
    unsigned t;
    float nb[7];
};

__device__ __forceinline__ bool better(float v, unsigned h, unsigned t, float bv, unsigned bh, unsigned bt)
{
    return v > bv || (v == bv && (h < bh || (h == bh && t < bt)));
}

// Reference: angle from the peak index and the 7-point parabola,
// cuda/gpu_aln_noref.cu:1773-1793 (same float/double mixing).
// (ring_len: samples per ring, the reference's cfg->ring_len)
__device__ float peak_angle(const float* x, unsigned tau, bool mirror, unsigned ring_len = kRingLen)
{
    float c2 = (float)(49. * x[0] + 6. * x[1] - 21. * x[2] - 32. * x[3] - 27. * x[4] - 6. * x[5] + 31. * x[6]);
    float c3 = (float)(5. * x[0] - 3. * x[2] - 4. * x[3] - 3. * x[4] + 5. * x[6]);
    float step = (float)(360.0 / (double)(float)ring_len);
    float angle = step * (float)tau;
    if (c3 != 0.0)
        angle = (float)((double)angle + (double)step * ((double)c2 / (2.0 * (double)c3) - 4));
    angle = (float)(360.0 - (double)angle);
    if (mirror)
        angle = (float)((double)angle + 180.0);
    if (angle >= 360.0)
        angle = (float)((double)angle - 360.0);
    return angle;
}

// Reference: the pre-alignment's angle, CcfResultTable::compute_alignment_param
// and interpolate_angle (cuda/gpu_aln_noref.cu:2463-2513, 2535-2577): the
// parabola and the angle in double precision, stored as float; 180 degrees
// added (and 360 taken off) for mirrors only.
__device__ float pre_peak_angle(const float* xf, unsigned tau, bool mirror)
{
    double x[7];
#pragma unroll
    for (int i = 0; i < 7; i++)
        x[i] = (double)xf[i];
    const double c2 = 49. * x[0] + 6. * x[1] - 21. * x[2] - 32. * x[3] - 27. * x[4] - 6. * x[5] + 31. * x[6];
    const double c3 = 5. * x[0] - 3. * x[2] - 4. * x[3] - 3. * x[4] + 5. * x[6];
    const double step = 360.0 / (double)kRingLen;
    double a = step * (double)tau;
    if (c3 != 0.0)
        a = a + step * (c2 / (2.0 * c3) - 4);
    float angle = (float)(360.0 - a);
    if (mirror) {
        angle = (float)((double)angle + 180.0);
        if (angle >= 360.0)
            angle = (float)((double)angle - 360.0);
    }
    return angle;
}

// running best of one pair slot, replicated over its 16-thread group
// (lanes 0..6 also hold the 7 samples around the peak)
struct PeakState {
    float bv;
    unsigned bh, bt;
    float nb;
    __device__ void reset(unsigned rule = kPeakMref)
    {
        // the pre-alignment's scan starts from 0 at index 0
        bv = rule == kPeakPreAlign ? 0.f : -3.40282e+038f;
        bh = 0;
        bt = 0;
        nb = 0.f;
    }
};

// Z[k] and Z[256-k] of one pair from the four ring sums at slot k
// (slot 0 carried (F[0], F[128]): recover the two real products)
__device__ __forceinline__ void write_z(float2* zp, int k, float a1, float a2, float a3, float a4)
{
    if (k == 0) {
        const float p1 = 0.25f * (a1 + a2 + a3 + a4);
        const float p2 = 0.25f * (a1 - a2 + a3 - a4);
        zp[0] = make_float2(p1, p1);
        zp[kSlots] = make_float2(p2, p2);
    } else {
        zp[k] = make_float2(a1, a2);
        zp[kRingLen - k] = make_float2(a3, a4);
    }
}

// inverse FFT of the pair spectrum this thread holds (x[m] = Z[l + 16 m]) and
// the peak search of both mirrors; gz is the group's workspace of
// kPairStride float2 (kTwl: tw is this thread's row of precomputed twiddles,
// fft256_group_twl)
template <bool kTwl = false>
__device__ __forceinline__ void fft_peak_regs(float2 (&x)[16], float2* gz, const float2* tw, int l, unsigned gmask,
                                              unsigned s, unsigned n_shift, PeakState& st, unsigned rule = kPeakMref)
{
    if (kTwl)
        fft256_group_twl<+1>(x, gz, tw, gmask);
    else
        fft256_group<+1>(x, gz, tw, l, gmask);
    float* wf = reinterpret_cast<float*>(gz);
    if (rule == kPeakPreAlign && s == 0 && st.bv == 0.f && st.bh == 0 && st.bt == 0) {
        // the starting index (normal, shift 0, angle 0) stays the answer when
        // no value beats 0: keep its 7 neighbours
        __syncwarp(gmask);
#pragma unroll
        for (int k2 = 0; k2 < 16; k2++)
            wf[l + 16 * k2] = x[perm16(k2)].x;
        __syncwarp(gmask);
        if (l < 7)
            st.nb = wf[((unsigned)l - 3u) & (kRingLen - 1)];
        __syncwarp(gmask);
    }
    // group maximum of each mirror first (the two reductions side by side);
    // the first index is only needed when a candidate can replace the
    // running best
    float vm[2] = {x[perm16(0)].x, x[perm16(0)].y};
#pragma unroll
    for (int k2 = 1; k2 < 16; k2++) {
        vm[0] = fmaxf(vm[0], x[perm16(k2)].x);
        vm[1] = fmaxf(vm[1], x[perm16(k2)].y);
    }
#pragma unroll
    for (int off = 8; off > 0; off >>= 1) {
        const float o0 = __shfl_xor_sync(gmask, vm[0], off), o1 = __shfl_xor_sync(gmask, vm[1], off);
        vm[0] = fmaxf(vm[0], o0);
        vm[1] = fmaxf(vm[1], o1);
    }
    // lane 0's values for the whole group keep every branch below
    // group-uniform, NaN inputs included
    vm[0] = __shfl_sync(gmask, vm[0], 0, 16);
    vm[1] = __shfl_sync(gmask, vm[1], 0, 16);
    // this transform's better mirror in the reference's order (at equal
    // maxima the normal one: its scan index is lower), then against the
    // running best -- the same result as offering both in turn, with one
    // index search and one gather of the neighbours
    const bool mir = vm[1] > vm[0] || vm[0] != vm[0];
    const float v = mir ? vm[1] : vm[0];
    if (!(v >= st.bv))
        return;
    unsigned t = 0xffffffffu;
#pragma unroll
    for (int k2 = 15; k2 >= 0; k2--)
        if ((mir ? x[perm16(k2)].y : x[perm16(k2)].x) == v)
            t = l + 16 * k2;
#pragma unroll
    for (int off = 8; off > 0; off >>= 1)
        t = min(t, __shfl_xor_sync(gmask, t, off));
    t = __shfl_sync(gmask, t, 0, 16);
    const unsigned hc = mir ? n_shift + s : s;
    if (t < (unsigned)kRingLen && better(v, hc, t, st.bv, st.bh, st.bt)) {
        st.bv = v;
        st.bh = hc;
        st.bt = t;
        __syncwarp(gmask);
#pragma unroll
        for (int k2 = 0; k2 < 16; k2++)
            wf[l + 16 * k2] = mir ? x[perm16(k2)].y : x[perm16(k2)].x;
        __syncwarp(gmask);
        if (l < 7)
            st.nb = wf[(t + (unsigned)l - 3u) & (kRingLen - 1)];
        __syncwarp(gmask);
    }
}

// the same for the pair spectrum in gz (Z[0..255], natural order)
template <bool kTwl = false>
__device__ __forceinline__ void fft_peak(float2* gz, const float2* tw, int l, unsigned gmask, unsigned s,
                                         unsigned n_shift, PeakState& st, unsigned rule = kPeakMref)
{
    float2 x[16];
#pragma unroll
    for (int m = 0; m < 16; m++)
        x[m] = gz[l + 16 * m];
    fft_peak_regs<kTwl>(x, gz, tw, l, gmask, s, n_shift, st, rule);
}

// named barrier `id` over n threads (id 0 with n = blockDim is __syncthreads)
__device__ __forceinline__ void nbar_sync(int id, int n) { asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory"); }
__device__ __forceinline__ void nbar_arrive(int id, int n)
{
    asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(n) : "memory");
}
// barrier `id` over n threads that returns whether p held on every one of them
__device__ __forceinline__ bool nbar_and(int id, int n, bool p)
{
    uint32_t r;
    asm volatile("{\n\t.reg .pred pi, po;\n\t"
                 "setp.ne.u32 pi, %1, 0;\n\t"
                 "bar.red.and.pred po, %2, %3, pi;\n\t"
                 "selp.u32 %0, 1, 0, po;\n\t}"
                 : "=r"(r)
                 : "r"((uint32_t)p), "r"(id), "r"(n)
                 : "memory");
    return r != 0;
}
// the barrier of the N threads that run the FFT / peak phase
template <int BAR, int N = 256>
__device__ __forceinline__ void phase_sync()
{
    if (BAR == 0)
        __syncthreads();
    else
        nbar_sync(BAR, N);
}

// merge the nsi shift slots of each of the qt references and write the
// outputs of particle p (the N threads of the FFT phase call, synchronised
// by barrier BAR; threads < qt write)
// the running best of pair slot g into the shared slot array
__device__ __forceinline__ void park_slot(PeakSlot* slots, const PeakState& st, int g, int l)
{
    if (l == 0) {
        slots[g].v = st.bv;
        slots[g].h = st.bh;
        slots[g].t = st.bt;
    }
    if (l < 7)
        slots[g].nb[l] = st.nb;
}

// the merge and the writes from slots every pair slot has parked
template <int BAR = 0, int N = 256>
__device__ __forceinline__ void merge_slots(PeakSlot* slots, int tid, int qt, int nsi, unsigned q0, unsigned n_ref,
                                            unsigned n_shift, unsigned pg, unsigned p_total, const float2* shifts_f,
                                            const float2* base, float* d_out, float4* peak_out,
                                            unsigned rule = kPeakMref)
{
    phase_sync<BAR, N>();
    if (tid < qt && q0 + tid < n_ref) {
        int best = tid;
        for (int i = 1; i < nsi; i++) {
            const int c = i * qt + tid;
            if (better(slots[c].v, slots[c].h, slots[c].t, slots[best].v, slots[best].h, slots[best].t))
                best = c;
        }
        const PeakSlot& ps = slots[best];
        const bool mirror = ps.h >= n_shift;
        const unsigned sidx = mirror ? ps.h - n_shift : ps.h;
        const float angle =
            rule == kPeakPreAlign ? pre_peak_angle(ps.nb, ps.t, mirror) : peak_angle(ps.nb, ps.t, mirror);
        const float bx = base ? base[pg].x : 0.f;
        const float by = base ? base[pg].y : 0.f;
        const float2 sf = shifts_f[sidx];
        const size_t o = (size_t)(q0 + tid) * p_total + pg;
        if (GPUISAC_IN_BOUNDS(kChkMergeOut, o, (size_t)n_ref * p_total)) {
            d_out[o] = ps.v;
            peak_out[o] = make_float4(angle, bx + sf.x, by + sf.y, mirror ? 1.f : 0.f);
        }
    }
    phase_sync<BAR, N>();
}

template <int BAR = 0, int N = 256>
__device__ __forceinline__ void merge_write(PeakSlot* slots, const PeakState& st, int tid, int g, int l, int qt,
                                            int nsi, unsigned q0, unsigned n_ref, unsigned n_shift, unsigned pg,
                                            unsigned p_total, const float2* shifts_f, const float2* base,
                                            float* d_out, float4* peak_out, unsigned rule = kPeakMref)
{
    phase_sync<BAR, N>();
    park_slot(slots, st, g, l);
    merge_slots<BAR, N>(slots, tid, qt, nsi, q0, n_ref, n_shift, pg, p_total, shifts_f, base, d_out, peak_out, rule);
}

// ---- mbarrier + bulk async copy (inline PTX) ----
__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

// try_wait suspends the thread until the phase completes or the hinted time
// (ns) has passed, leaving the issue slots to the other warps meanwhile
__device__ __forceinline__ bool mbar_try(uint64_t* bar, uint32_t parity, uint32_t hint_ns)
{
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(smem_addr(bar)), "r"(parity), "r"(hint_ns)
                 : "memory");
    return ok != 0;
}
// bounded wait: gives up after `tries` tries of at most 20 us (by default
// 2^16, about a second)
constexpr uint32_t kWaitTries = 1u << 16;
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t tries = kWaitTries)
{
    for (uint32_t it = 0; it < tries; it++)
        if (mbar_try(bar, parity, 20000u))
            return true;
    return false;
}
// the limit a work descriptor asks for (0: the default)
__device__ __forceinline__ uint32_t wait_tries(uint32_t asked) { return asked ? asked : kWaitTries; }

__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

} // namespace

// ============================================================================
// ---- tensor memory (inline PTX) ----
namespace {
__device__ __forceinline__ void tmem_alloc(uint32_t* dst_smem, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(dst_smem)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tmem_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tmem_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// each thread of the warp writes 8 consecutive columns of its own lane
__device__ __forceinline__ void tmem_st8(uint32_t taddr, const float (&v)[8])
{
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"r"(taddr),
                 "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])),
                 "r"(__float_as_uint(v[3])), "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])),
                 "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7]))
                 : "memory");
}
__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }
// 16 consecutive columns of the thread's own lane, left in flight: the
// registers are valid after tmem_wait_ld16 on the same array, which takes
// them as operands so that no use is scheduled before the wait
__device__ __forceinline__ void tmem_ld16_async(uint32_t taddr, float (&v)[16])
{
    uint32_t* r = reinterpret_cast<uint32_t*>(v);
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, "
                 "%13, %14, %15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                   "=r"(r[15])
                 : "r"(taddr)
                 : "memory");
}
__device__ __forceinline__ void tmem_wait_ld16(float (&v)[16])
{
    uint32_t* r = reinterpret_cast<uint32_t*>(v);
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                   "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]),
                   "+r"(r[15])
                 :
                 : "memory");
}
} // namespace

} // namespace gpuisac
