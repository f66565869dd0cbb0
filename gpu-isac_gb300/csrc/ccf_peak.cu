// ccf_peak.cu -- ring-weighted cross-correlation of every (particle, shift)
// against a tile of references, the inverse angular FFT and the peak search
// over reference x angle x shift x mirror, fused: the per-pair spectra never
// leave the SM.
//
// Reference semantics: cu_ccf_mult_mref (cuda/gpu_aln_noref.cu:1483-1537), the
// C2R of every ccf-table entry (:2453-2461), cu_aln_param_wizard (:1667-1794)
// and the host scatter of multi_ref_align (:516-541).
//
// CTA = 256 threads, one tile of QT references (spectra resident in shared
// memory), a run of particles.  Per iteration NSI = 16/QT shifts x QT refs =
// 16 (shift, ref) pairs:
//   contraction  thread (k = tid%128, half = tid/128) holds the subject
//                spectra of NSI shifts at slot k and accumulates, for its
//                QT/2 references, the four sums that form Z[k] and Z[256-k];
//   inverse FFT  16 groups of 16 threads, one 256-point FFT per pair; real part
//                = normal correlation, imaginary part = mirrored;
//   peak search  first strict maximum in the reference's scan order
//                (mirror-major, then shift, then angle), kept per pair slot
//                with the 7 samples around it; merged per reference at the
//                end of the particle, then the 7-point parabola.
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
__device__ float peak_angle(const float* x, unsigned tau, bool mirror)
{
    float c2 = (float)(49. * x[0] + 6. * x[1] - 21. * x[2] - 32. * x[3] - 27. * x[4] - 6. * x[5] + 31. * x[6]);
    float c3 = (float)(5. * x[0] - 3. * x[2] - 4. * x[3] - 3. * x[4] + 5. * x[6]);
    float step = (float)(360.0 / (double)(float)kRingLen);
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

} // namespace

template <int QT>
__global__ void __launch_bounds__(256, 1)
ccf_peak_kernel(const float2* __restrict__ sbj_sp, const float2* __restrict__ ref_sp,
                const float2* __restrict__ twiddle, unsigned ring_num, unsigned n_shift, unsigned n_ref,
                unsigned n_part, unsigned part_per_cta, unsigned p_global0, unsigned p_total,
                const float2* __restrict__ shifts_f, const float2* __restrict__ base,
                float* __restrict__ d_out, float4* __restrict__ peak_out)
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
    const unsigned q0 = blockIdx.x * QT;

    tw[tid] = twiddle[tid];
    // reference tile -> shared memory (zero padded rings / missing refs)
    for (unsigned idx = tid; idx < (unsigned)QT * nrp * kSlots; idx += 256) {
        unsigned qq = idx / (nrp * kSlots);
        unsigned rem = idx - qq * nrp * kSlots;
        unsigned r = rem / kSlots, kk = rem - r * kSlots;
        float2 v = make_float2(0.f, 0.f);
        if (q0 + qq < n_ref && r < ring_num)
            v = __ldg(&ref_sp[((size_t)(q0 + qq) * ring_num + r) * kSlots + kk]);
        rsp[idx] = v;
    }
    __syncthreads();

    const int g = tid >> 4, l = tid & 15;
    const unsigned gmask = 0xffffu << (tid & 16);
    const int g_shift = g / QT;
    float2* gz = zbuf + g * kPairStride;
    const unsigned n_chunks = nrp / RC;

    for (unsigned pi = 0; pi < part_per_cta; pi++) {
        const unsigned p = blockIdx.y * part_per_cta + pi;
        if (p >= n_part)
            break;
        float bv = -3.40282e+038f;
        unsigned bh = 0, bt = 0;
        float nb = 0.f;

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
                srow[i] = sbj_sp + ((size_t)p * n_shift + (svalid[i] ? s : 0)) * ring_num * kSlots + k;
            }
            float2 cur[NSI][RC], nxt[NSI][RC];
#pragma unroll
            for (int i = 0; i < NSI; i++)
#pragma unroll
                for (int rr = 0; rr < RC; rr++)
                    cur[i][rr] = (svalid[i] && (unsigned)rr < ring_num) ? __ldg(srow[i] + rr * kSlots)
                                                                        : make_float2(0.f, 0.f);
            for (unsigned c = 0; c < n_chunks; c++) {
                const unsigned r0 = c * RC;
                if (c + 1 < n_chunks) {
                    const unsigned r1 = r0 + RC;
#pragma unroll
                    for (int i = 0; i < NSI; i++)
#pragma unroll
                        for (int rr = 0; rr < RC; rr++)
                            nxt[i][rr] = (svalid[i] && r1 + rr < ring_num)
                                             ? __ldg(srow[i] + (size_t)(r1 + rr) * kSlots)
                                             : make_float2(0.f, 0.f);
                }
#pragma unroll
                for (int j = 0; j < RPT; j++) {
                    const float2* rq = rsp + ((size_t)(half * RPT + j) * nrp + r0) * kSlots + k;
#pragma unroll
                    for (int rr = 0; rr < RC; rr++) {
                        const float2 uv = rq[rr * kSlots];
#pragma unroll
                        for (int i = 0; i < NSI; i++) {
                            const float2 ab = cur[i][rr];
                            acc[j][i][0] = fmaf(uv.x, ab.x, acc[j][i][0]);
                            acc[j][i][1] = fmaf(uv.x, ab.y, acc[j][i][1]);
                            acc[j][i][2] = fmaf(uv.y, ab.y, acc[j][i][2]);
                            acc[j][i][3] = fmaf(uv.y, ab.x, acc[j][i][3]);
                        }
                    }
                }
#pragma unroll
                for (int i = 0; i < NSI; i++)
#pragma unroll
                    for (int rr = 0; rr < RC; rr++)
                        cur[i][rr] = nxt[i][rr];
            }

            __syncthreads(); // previous FFT phase is done with zbuf
#pragma unroll
            for (int j = 0; j < RPT; j++) {
#pragma unroll
                for (int i = 0; i < NSI; i++) {
                    float2* zp = zbuf + (i * QT + half * RPT + j) * kPairStride;
                    const float a1 = acc[j][i][0], a2 = acc[j][i][1], a3 = acc[j][i][2], a4 = acc[j][i][3];
                    if (k == 0) {
                        // slot 0 carried (F[0], F[128]): recover the two real products
                        const float p1 = 0.25f * (a1 + a2 + a3 + a4);
                        const float p2 = 0.25f * (a1 - a2 + a3 - a4);
                        zp[0] = make_float2(p1, p1);
                        zp[kSlots] = make_float2(p2, p2);
                    } else {
                        zp[k] = make_float2(a1, a2);
                        zp[kRingLen - k] = make_float2(a3, a4);
                    }
                }
            }
            __syncthreads();

            // ---- inverse FFT + peak search, one pair per 16-thread group ----
            const unsigned s = s0 + g_shift;
            if (s < n_shift) {
                float2 x[16];
#pragma unroll
                for (int m = 0; m < 16; m++)
                    x[m] = gz[l + 16 * m];
                fft256_group<+1>(x, gz, tw, l, gmask);
                float* wf = reinterpret_cast<float*>(gz);
#pragma unroll
                for (int mir = 0; mir < 2; mir++) {
                    float v = mir ? x[0].y : x[0].x;
                    unsigned t = l;
#pragma unroll
                    for (int k2 = 1; k2 < 16; k2++) {
                        const float c = mir ? x[k2].y : x[k2].x;
                        if (c > v) {
                            v = c;
                            t = l + 16 * k2;
                        }
                    }
#pragma unroll
                    for (int off = 8; off > 0; off >>= 1) {
                        const float ov = __shfl_xor_sync(gmask, v, off);
                        const unsigned ot = __shfl_xor_sync(gmask, t, off);
                        if (ov > v || (ov == v && ot < t)) {
                            v = ov;
                            t = ot;
                        }
                    }
                    // lane 0's result for the whole group, so the branch below
                    // stays group-uniform even for NaN inputs
                    v = __shfl_sync(gmask, v, 0, 16);
                    t = __shfl_sync(gmask, t, 0, 16);
                    const unsigned hc = mir ? n_shift + s : s;
                    if (better(v, hc, t, bv, bh, bt)) {
                        bv = v;
                        bh = hc;
                        bt = t;
                        __syncwarp(gmask);
#pragma unroll
                        for (int k2 = 0; k2 < 16; k2++)
                            wf[l + 16 * k2] = mir ? x[k2].y : x[k2].x;
                        __syncwarp(gmask);
                        if (l < 7)
                            nb = wf[(t + (unsigned)l - 3u) & (kRingLen - 1)];
                        __syncwarp(gmask);
                    }
                }
            }
        }

        // ---- merge the NSI shift slots of each reference, write results ----
        __syncthreads();
        if (l == 0) {
            slots[g].v = bv;
            slots[g].h = bh;
            slots[g].t = bt;
        }
        if (l < 7)
            slots[g].nb[l] = nb;
        __syncthreads();
        if (tid < QT && q0 + tid < n_ref) {
            int best = tid;
#pragma unroll
            for (int i = 1; i < NSI; i++) {
                const int c = i * QT + tid;
                if (better(slots[c].v, slots[c].h, slots[c].t, slots[best].v, slots[best].h, slots[best].t))
                    best = c;
            }
            const PeakSlot& ps = slots[best];
            const bool mirror = ps.h >= n_shift;
            const unsigned sidx = mirror ? ps.h - n_shift : ps.h;
            const float angle = peak_angle(ps.nb, ps.t, mirror);
            const unsigned pg = p_global0 + p;
            const float bx = base ? base[pg].x : 0.f;
            const float by = base ? base[pg].y : 0.f;
            const float2 sf = shifts_f[sidx];
            const size_t o = (size_t)(q0 + tid) * p_total + pg;
            d_out[o] = ps.v;
            peak_out[o] = make_float4(angle, bx + sf.x, by + sf.y, mirror ? 1.f : 0.f);
        }
        __syncthreads();
    }
}

size_t ccf_peak_smem_bytes(unsigned ring_num)
{
    unsigned qt = ccf_refs_per_cta(ring_num);
    return (size_t)qt * ring_pad(ring_num) * kSlots * sizeof(float2) + 16 * kPairStride * sizeof(float2) +
           kRingLen * sizeof(float2) + 16 * sizeof(PeakSlot);
}

template <int QT>
static cudaError_t launch_qt(const float2* sbj_sp, const float2* ref_sp, const float2* twiddle, unsigned ring_num,
                             unsigned n_shift, unsigned n_ref, unsigned n_part, unsigned p_global0,
                             unsigned p_total, const float2* shifts_f, const float2* base, float* d_out,
                             float4* peak_out, cudaStream_t stream)
{
    static int configured = 0;
    size_t smem = ccf_peak_smem_bytes(ring_num);
    if (!configured) {
        int dev = 0, max_optin = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        cudaError_t e = cudaFuncSetAttribute(ccf_peak_kernel<QT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             max_optin);
        if (e != cudaSuccess)
            return e;
        configured = 1;
    }
    const unsigned ref_tiles = (n_ref + QT - 1) / QT;
    const unsigned ppc = 8;
    dim3 grid(ref_tiles, (n_part + ppc - 1) / ppc);
    ccf_peak_kernel<QT><<<grid, 256, smem, stream>>>(sbj_sp, ref_sp, twiddle, ring_num, n_shift, n_ref, n_part, ppc,
                                                     p_global0, p_total, shifts_f, base, d_out, peak_out);
    g_kernel_launches.fetch_add(1, std::memory_order_relaxed);
    return cudaGetLastError();
}

cudaError_t launch_ccf_peak(const float2* sbj_sp, const float2* ref_sp, const float2* twiddle, unsigned ring_num,
                            unsigned n_shift, unsigned n_ref, unsigned n_part, unsigned p_global0, unsigned p_total,
                            const float2* shifts_f, const float2* base, float* d_out, float4* peak_out,
                            cudaStream_t stream)
{
    if (n_part == 0 || n_ref == 0)
        return cudaSuccess;
    if (ccf_refs_per_cta(ring_num) == 4)
        return launch_qt<4>(sbj_sp, ref_sp, twiddle, ring_num, n_shift, n_ref, n_part, p_global0, p_total, shifts_f,
                            base, d_out, peak_out, stream);
    return launch_qt<2>(sbj_sp, ref_sp, twiddle, ring_num, n_shift, n_ref, n_part, p_global0, p_total, shifts_f, base,
                        d_out, peak_out, stream);
}

} // namespace gpuisac
