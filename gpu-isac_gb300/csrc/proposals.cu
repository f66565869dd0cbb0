// proposals.cu -- the exhaustive shift x angle x mirror search restricted to
// a list of references per particle.
//
// gpuisac_align_proposals_device aligns each selected particle against its own
// k references (a proposal list, or every reference for a fallback) with the
// same kernels and the same stacked-image semantics as the full
// multi-reference alignment: each (particle, reference) result equals the
// corresponding entry of a full alignment of the stack.  Particles keep their
// index in the whole stack (texture grouping of the reference), whichever
// subset is selected.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <mutex>
#include <vector>

#include "../../include/gpu_aln_pack.h"
#include "gpuisac_kernels.h"
#include "host_geometry.h"

using namespace gpuisac;

namespace {

int fail(int code, const char* msg)
{
    record_error(code, msg);
    return code;
}

#define P_CK(expr)                                                                        \
    do {                                                                                  \
        cudaError_t e_ = (expr);                                                          \
        if (e_ != cudaSuccess) {                                                          \
            char m_[384];                                                                 \
            snprintf(m_, sizeof(m_), "%s (%s) in the proposal alignment", cudaGetErrorString(e_), #expr); \
            return fail(1, m_);                                                           \
        }                                                                                 \
    } while (0)

template <typename T>
struct Buf {
    T* p = nullptr;
    size_t n = 0;
    cudaError_t ensure(size_t count)
    {
        if (count <= n)
            return cudaSuccess;
        if (p)
            cudaFree(p);
        p = nullptr;
        n = 0;
        cudaError_t e = cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T));
        if (e == cudaSuccess)
            n = count;
        return e;
    }
};

struct PropState {
    std::mutex mu;
    Buf<float2> tw, tmpl, shifts_f, ref_sp, sbj_sp;
    Buf<int2> shifts_i, zero;
    Buf<CcfGroup> table;
    Buf<unsigned> err, sel;
    TexStack ref_tex, sbj_tex;
} g_prop;

} // namespace

extern "C" int gpuisac_align_proposals_device(const AlignConfig* cfg, const float* sbj, const float* ref,
                                              const float* base_shift, const unsigned int* part_idx,
                                              unsigned int n_sel, const unsigned int* proposals, unsigned int k,
                                              float* d_out, float* peak_out, void* stream)
{
    HostGeometry geo;
    int rc = host_geometry(cfg, geo);
    if (rc)
        return rc;
    if (!sbj || !ref || !proposals || !d_out || !peak_out)
        return fail(2, "NULL device pointer");
    if (k == 0 || k > geo.R)
        return fail(2, "proposal length must be 1..ref_num");
    if (!part_idx && n_sel != geo.P)
        return fail(2, "without a particle list every particle is selected (n_sel must equal sbj_num)");
    if (n_sel == 0)
        return 0;
    std::lock_guard<std::mutex> lk(g_prop.mu);
    PropState& S = g_prop;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int dev = 0;
    P_CK(cudaGetDevice(&dev));
    const unsigned NR = geo.NR, Sn = geo.S, D = geo.D;
    const size_t row_elems = (size_t)NR * kSlots;
    const unsigned tex = texture_images(dev, D);
    const int variant = ccf_variant(NR, true, Sn);
    const unsigned qt = ccf_refs_per_item(NR, variant);

    P_CK(S.tw.ensure(kRingLen));
    P_CK(S.tmpl.ensure(geo.tmpl.size()));
    P_CK(S.shifts_f.ensure(Sn));
    P_CK(S.shifts_i.ensure(Sn));
    P_CK(S.zero.ensure(1));
    P_CK(S.err.ensure(2)); // the timeout flag and the CCF kernel's work counter
    P_CK(S.ref_sp.ensure(row_elems * geo.R));
    P_CK(S.table.ensure(n_sel));
    const int2 zero = make_int2(0, 0);
    P_CK(cudaMemcpy(S.tw.p, geo.tw.data(), kRingLen * sizeof(float2), cudaMemcpyHostToDevice));
    P_CK(cudaMemcpy(S.tmpl.p, geo.tmpl.data(), geo.tmpl.size() * sizeof(float2), cudaMemcpyHostToDevice));
    P_CK(cudaMemcpy(S.shifts_f.p, geo.shifts_f.data(), Sn * sizeof(float2), cudaMemcpyHostToDevice));
    P_CK(cudaMemcpy(S.shifts_i.p, geo.shifts_i.data(), Sn * sizeof(int2), cudaMemcpyHostToDevice));
    P_CK(cudaMemcpy(S.zero.p, &zero, sizeof(int2), cudaMemcpyHostToDevice));
    P_CK(cudaMemsetAsync(S.err.p, 0, sizeof(unsigned), st));

    // selected particles (host copy of the list, for the per-particle groups)
    std::vector<unsigned> sel(n_sel);
    if (part_idx) {
        P_CK(cudaMemcpy(sel.data(), part_idx, n_sel * sizeof(unsigned), cudaMemcpyDeviceToHost));
        for (unsigned i = 0; i < n_sel; i++)
            if (sel[i] >= geo.P)
                return fail(2, "particle index outside the stack");
    } else {
        for (unsigned i = 0; i < n_sel; i++)
            sel[i] = i;
    }

    // every proposal must name a reference of the stack (the kernels trust them)
    {
        std::vector<unsigned> prop((size_t)n_sel * k);
        P_CK(cudaMemcpy(prop.data(), proposals, prop.size() * sizeof(unsigned), cudaMemcpyDeviceToHost));
        for (unsigned v : prop)
            if (v >= geo.R)
                return fail(2, "proposal names a reference outside the stack");
    }

    // reference spectra: every reference, stacked as the reference stacks them
    StackDesc refs{ref, geo.R, D, std::max(1u, std::min(geo.R, 100u)), tex};
    const unsigned long long *ref_tx = nullptr, *sbj_tx = nullptr;
    if (texture_unit_enabled())
        ref_tx = S.ref_tex.try_build(refs, st);
    P_CK(launch_polar_spectra(refs, S.tmpl.p, S.tw.p, NR, S.zero.p, 1, nullptr, 0, geo.R, 1, S.ref_sp.p, st, nullptr,
                              ref_tx));

    // one group per selected particle: 1 particle x its k references
    const unsigned tiles = (k + qt - 1) / qt;
    std::vector<CcfGroup> table(n_sel);
    size_t free_b = 0, total_b = 0;
    P_CK(cudaMemGetInfo(&free_b, &total_b));
    const size_t per_part = row_elems * Sn * sizeof(float2);
    const unsigned chunk =
        (unsigned)std::max<size_t>(1, std::min<size_t>((size_t)(0.4 * (double)free_b) / per_part, 16384));
    P_CK(S.sbj_sp.ensure(row_elems * Sn * std::min(chunk, n_sel)));
    const float2* bs = reinterpret_cast<const float2*>(base_shift);
    StackDesc sbjs{sbj, geo.P, D, geo.sbj_batch, tex};
    if (texture_unit_enabled())
        sbj_tx = S.sbj_tex.try_build(sbjs, st);
    const unsigned* sel_dev = part_idx;
    for (unsigned c0 = 0; c0 < n_sel; c0 += chunk) {
        const unsigned n = std::min(chunk, n_sel - c0);
        for (unsigned i = 0; i < n; i++) {
            CcfGroup g{};
            const unsigned p = sel[c0 + i];
            g.sbj_sp = S.sbj_sp.p + (size_t)i * row_elems * Sn;
            g.ref_sp = S.ref_sp.p;
            g.ref_idx = proposals + (size_t)(c0 + i) * k;
            g.base = bs ? bs + p : nullptr;
            g.d_out = d_out + (size_t)(c0 + i) * k;
            g.peak_out = reinterpret_cast<float4*>(peak_out) + (size_t)(c0 + i) * k;
            g.p_first = 0;
            g.n_part = 1;
            g.n_ref = k;
            g.p_total = 1;
            g.item_begin = i * tiles;
            g.ref_tiles = tiles;
            table[c0 + i] = g;
        }
        P_CK(cudaMemcpyAsync(S.table.p + c0, table.data() + c0, n * sizeof(CcfGroup), cudaMemcpyHostToDevice, st));
        P_CK(launch_polar_spectra(sbjs, S.tmpl.p, S.tw.p, NR, S.shifts_i.p, Sn, bs, c0, n, 0, S.sbj_sp.p, st,
                                  sel_dev ? sel_dev + c0 : nullptr, sbj_tx));
        CcfWork w{};
        w.groups = S.table.p + c0;
        w.n_groups = n;
        w.n_items = n * tiles;
        w.ppc = 1;
        w.item_counter = S.err.p + 1;
        P_CK(launch_ccf_peak_work(w, variant, S.tw.p, NR, Sn, S.shifts_f.p, S.err.p, st));
    }
    P_CK(cudaStreamSynchronize(st)); // the host table must outlive its copies
    unsigned flag = 0;
    P_CK(cudaMemcpy(&flag, S.err.p, sizeof(unsigned), cudaMemcpyDeviceToHost));
    return flag ? fail(1, "a kernel timed out waiting for its own asynchronous copies") : 0;
}

// ============================================================ learned search

namespace {

// One warp per row i of d [n][kk] (candidates cand[i][j], or j itself when
// cand is null): the best entry (ties: the smaller reference index, NaN never
// wins), written to particle dst[i] (or i).  Optionally the gap to the
// runner-up candidate (+inf with one candidate) and the fallback flag
// gap < gap_margin.
__global__ void best_of_kernel(const float* __restrict__ d, const float4* __restrict__ pk,
                               const unsigned* __restrict__ cand, unsigned kk, unsigned n,
                               const unsigned* __restrict__ dst, int* __restrict__ best_ref,
                               float* __restrict__ best_peak, float4* __restrict__ best_param,
                               float* __restrict__ best_gap, float gap_margin, unsigned* __restrict__ fb)
{
    const unsigned i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (i >= n)
        return;
    const float* row = d + (size_t)i * kk;
    const unsigned* crow = cand ? cand + (size_t)i * kk : nullptr;
    const unsigned kNone = 0xffffffffu;
    float bv = -INFINITY;
    unsigned br = kNone, bj = kNone;
    for (unsigned j = lane; j < kk; j += 32) {
        const float v = row[j];
        const unsigned r = crow ? crow[j] : j;
        if (v != v)
            continue;
        if (br == kNone || v > bv || (v == bv && r < br)) {
            bv = v;
            br = r;
            bj = j;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        const float ov = __shfl_xor_sync(0xffffffffu, bv, o);
        const unsigned orr = __shfl_xor_sync(0xffffffffu, br, o);
        const unsigned oj = __shfl_xor_sync(0xffffffffu, bj, o);
        if (orr != kNone && (br == kNone || ov > bv || (ov == bv && orr < br))) {
            bv = ov;
            br = orr;
            bj = oj;
        }
    }
    float sv = -INFINITY;
    for (unsigned j = lane; j < kk; j += 32)
        if (j != bj && row[j] == row[j])
            sv = fmaxf(sv, row[j]);
    for (int o = 16; o > 0; o >>= 1)
        sv = fmaxf(sv, __shfl_xor_sync(0xffffffffu, sv, o));
    if (lane == 0) {
        const unsigned o = dst ? dst[i] : i;
        if (br == kNone) { // every entry NaN: keep the first
            bj = 0;
            br = crow ? crow[0] : 0;
            bv = row[0];
        }
        best_ref[o] = (int)br;
        best_peak[o] = bv;
        best_param[o] = pk[(size_t)i * kk + bj];
        const float gap = bv - sv;
        if (best_gap)
            best_gap[o] = gap;
        if (fb)
            fb[o] = (gap >= gap_margin) ? 0u : 1u;
    }
}

struct LearnState {
    std::mutex mu;
    Buf<float2> tw, tmpl, shifts_f, ref_sp, sbj_sp;
    Buf<int2> shifts_i, zero;
    Buf<CcfGroup> table;
    Buf<unsigned> err, prop, fb_list, fb_flag;
    Buf<float> X, H, Z, E, nrm, G, Smax, dk, dfb;
    Buf<float4> pkk, pfb;
    TexStack ref_tex, sbj_tex;
} g_learn;

} // namespace

extern "C" int gpuisac_learned_align_device(const AlignConfig* cfg, const float* sbj, const float* ref,
                                            const float* base_shift, const GpuisacProposalNet* net,
                                            const float* ref_emb, unsigned int k, float gap_margin, int* best_ref,
                                            float* best_peak, float* best_param, float* best_gap,
                                            unsigned int* fallback, unsigned long long* pairs, void* stream)
{
    const gpuisac::NvtxRange nvtx_range("gpuisac:learned_align");
    HostGeometry geo;
    int rc = host_geometry(cfg, geo);
    if (rc)
        return rc;
    if (!sbj || !ref || !net || !ref_emb || !best_ref || !best_peak || !best_param)
        return fail(2, "NULL pointer");
    if (!net->mu || !net->inv_sd || !net->W1 || !net->b1 || !net->W2 || !net->b2)
        return fail(2, "NULL network weight");
    if (net->nk == 0 || net->nk > kSlots || net->hidden == 0 || net->emb == 0)
        return fail(2, "network shape out of range (nk 1..128, hidden and emb >= 1)");
    if (k == 0 || k > geo.R || k > 64 || geo.R > 1024)
        return fail(2, "k must be 1..min(64, ref_num), ref_num <= 1024");
    if (pairs)
        *pairs = 0;
    std::lock_guard<std::mutex> lk(g_learn.mu);
    LearnState& S = g_learn;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int dev = 0;
    P_CK(cudaGetDevice(&dev));
    const unsigned NR = geo.NR, Sn = geo.S, D = geo.D, R = geo.R, P = geo.P;
    const unsigned n_in = NR * net->nk, hid = net->hidden, emb = net->emb;
    const size_t row_elems = (size_t)NR * kSlots;
    const unsigned tex = texture_images(dev, D);
    const int variant = ccf_variant(NR, true, Sn);
    const unsigned qt = ccf_refs_per_item(NR, variant);

    P_CK(S.tw.ensure(kRingLen));
    P_CK(S.tmpl.ensure(geo.tmpl.size()));
    P_CK(S.shifts_f.ensure(Sn));
    P_CK(S.shifts_i.ensure(Sn));
    P_CK(S.zero.ensure(1));
    P_CK(S.err.ensure(2)); // the timeout flag and the CCF kernel's work counter
    P_CK(S.ref_sp.ensure(row_elems * R));
    const int2 zero = make_int2(0, 0);
    P_CK(cudaMemcpy(S.tw.p, geo.tw.data(), kRingLen * sizeof(float2), cudaMemcpyHostToDevice));
    P_CK(cudaMemcpy(S.tmpl.p, geo.tmpl.data(), geo.tmpl.size() * sizeof(float2), cudaMemcpyHostToDevice));
    P_CK(cudaMemcpy(S.shifts_f.p, geo.shifts_f.data(), Sn * sizeof(float2), cudaMemcpyHostToDevice));
    P_CK(cudaMemcpy(S.shifts_i.p, geo.shifts_i.data(), Sn * sizeof(int2), cudaMemcpyHostToDevice));
    P_CK(cudaMemcpy(S.zero.p, &zero, sizeof(int2), cudaMemcpyHostToDevice));
    P_CK(cudaMemsetAsync(S.err.p, 0, sizeof(unsigned), st));

    // reference spectra for the search (reference basis, every reference)
    StackDesc refs{ref, R, D, std::max(1u, std::min(R, 100u)), tex};
    const unsigned long long *ref_tx = nullptr, *sbj_tx = nullptr;
    if (texture_unit_enabled())
        ref_tx = S.ref_tex.try_build(refs, st);
    P_CK(launch_polar_spectra(refs, S.tmpl.p, S.tw.p, NR, S.zero.p, 1, nullptr, 0, R, 1, S.ref_sp.p, st, nullptr,
                              ref_tx));

    // chunk of particles: spectra at every shift, network activations over
    // every (particle, shift) row, scores, proposals and both searches
    const size_t per_part = row_elems * Sn * sizeof(float2) +
                            (size_t)Sn * (n_in + hid + 2 * emb + 1 + R) * sizeof(float) +
                            (size_t)R * (sizeof(float) + sizeof(float) + sizeof(float4)) +
                            (size_t)k * (sizeof(unsigned) + sizeof(float) + sizeof(float4)) + 64;
    size_t free_b = 0, total_b = 0;
    P_CK(cudaMemGetInfo(&free_b, &total_b));
    const unsigned chunk = (unsigned)std::min<size_t>(
        P, std::max<size_t>(1, std::min<size_t>((size_t)(0.4 * (double)free_b) / per_part, 16384)));
    const size_t rows_max = (size_t)chunk * Sn;
    P_CK(S.sbj_sp.ensure(row_elems * rows_max));
    P_CK(S.X.ensure(rows_max * n_in));
    P_CK(S.H.ensure(rows_max * hid));
    P_CK(S.Z.ensure(rows_max * emb));
    P_CK(S.E.ensure(rows_max * emb));
    P_CK(S.nrm.ensure(rows_max));
    P_CK(S.G.ensure(rows_max * R));
    P_CK(S.Smax.ensure((size_t)chunk * R));
    P_CK(S.prop.ensure((size_t)chunk * k));
    P_CK(S.dk.ensure((size_t)chunk * k));
    P_CK(S.pkk.ensure((size_t)chunk * k));
    P_CK(S.fb_flag.ensure(chunk));
    P_CK(S.fb_list.ensure(chunk));
    P_CK(S.dfb.ensure((size_t)chunk * R));
    P_CK(S.pfb.ensure((size_t)chunk * R));
    P_CK(S.table.ensure(chunk));

    const float2* bs = reinterpret_cast<const float2*>(base_shift);
    StackDesc sbjs{sbj, P, D, geo.sbj_batch, tex};
    if (texture_unit_enabled())
        sbj_tx = S.sbj_tex.try_build(sbjs, st);
    std::vector<CcfGroup> table(chunk);
    std::vector<unsigned> flags(chunk), fbl;
    unsigned long long n_pairs = 0;
    float4* bparam = reinterpret_cast<float4*>(best_param);
    const unsigned tiles_k = (k + qt - 1) / qt, tiles_all = (R + qt - 1) / qt;

    auto ccf = [&](unsigned n_groups, unsigned tiles) -> int {
        P_CK(cudaMemcpyAsync(S.table.p, table.data(), n_groups * sizeof(CcfGroup), cudaMemcpyHostToDevice, st));
        CcfWork w{};
        w.groups = S.table.p;
        w.n_groups = n_groups;
        w.n_items = n_groups * tiles;
        w.ppc = 1;
        w.item_counter = S.err.p + 1;
        P_CK(launch_ccf_peak_work(w, variant, S.tw.p, NR, Sn, S.shifts_f.p, S.err.p, st));
        return 0;
    };
#define NN_CK(expr)                                                                      \
    do {                                                                                 \
        if ((expr) != 0)                                                                 \
            return fail(1, "network kernel launch failed in the learned search (" #expr ")"); \
    } while (0)

    // the network's GEMMs on the tensor cores (BF16 operands) unless
    // GPUISAC_NN_FP32 is set or a shape or address rules out 16-byte staging
    auto al16 = [](const void* p) { return ((uintptr_t)p & 15) == 0; };
    const char* fp32 = getenv("GPUISAC_NN_FP32");
    const bool tensor_cores = !(fp32 && fp32[0] && fp32[0] != '0') && n_in % 4 == 0 && hid % 4 == 0 &&
                              emb % 4 == 0 && al16(net->W1) && al16(net->W2) && al16(ref_emb);
    for (unsigned c0 = 0; c0 < P; c0 += chunk) {
        const unsigned n = std::min(chunk, P - c0);
        const long rows = (long)n * Sn;
        // 1. subject spectra at every shift
        P_CK(launch_polar_spectra(sbjs, S.tmpl.p, S.tw.p, NR, S.shifts_i.p, Sn, bs, c0, n, 0, S.sbj_sp.p, st, nullptr,
                                  sbj_tx));
        // 2. standardised ring features of every (particle, shift) row
        NN_CK(gpuisac_nn_features(reinterpret_cast<const float*>(S.sbj_sp.p), (unsigned)rows, NR, net->nk, net->mu,
                                  net->inv_sd, S.X.p, st));
        // 3. embeddings (BF16 tensor cores, bias and ReLU in the epilogue; FP32
        // CUDA-core GEMMs where the shapes do not allow the 16-byte staging)
        if (tensor_cores) {
            NN_CK(gpuisac_nn_gemm_bf16((int)rows, (int)hid, (int)n_in, 1.f, S.X.p, n_in, net->W1, n_in, net->b1, 1,
                                       S.H.p, hid, S.err.p, st));
            NN_CK(gpuisac_nn_gemm_bf16((int)rows, (int)emb, (int)hid, 1.f, S.H.p, hid, net->W2, hid, net->b2, 0,
                                       S.Z.p, emb, S.err.p, st));
        } else {
            NN_CK(gpuisac_nn_gemm((int)rows, (int)hid, (int)n_in, 1.f, S.X.p, n_in, 1, net->W1, 1, n_in, 0.f, S.H.p,
                                  hid, st));
            NN_CK(gpuisac_nn_bias_act(S.H.p, net->b1, rows, (int)hid, 1, st));
            NN_CK(gpuisac_nn_gemm((int)rows, (int)emb, (int)hid, 1.f, S.H.p, hid, 1, net->W2, 1, hid, 0.f, S.Z.p,
                                  emb, st));
            NN_CK(gpuisac_nn_bias_act(S.Z.p, net->b2, rows, (int)emb, 0, st));
        }
        NN_CK(gpuisac_nn_l2norm(S.Z.p, rows, (int)emb, S.E.p, S.nrm.p, st));
        // 4. similarity to every reference, best over shifts, top k
        if (tensor_cores)
            NN_CK(gpuisac_nn_gemm_bf16((int)rows, (int)R, (int)emb, 1.f, S.E.p, emb, ref_emb, emb, nullptr, 0, S.G.p,
                                       R, S.err.p, st));
        else
            NN_CK(gpuisac_nn_gemm((int)rows, (int)R, (int)emb, 1.f, S.E.p, emb, 1, ref_emb, 1, emb, 0.f, S.G.p, R,
                                  st));
        NN_CK(gpuisac_nn_group_max(S.G.p, n, (int)Sn, (int)R, S.Smax.p, st));
        NN_CK(gpuisac_nn_topk(S.Smax.p, n, (int)R, (int)k, S.prop.p, st));
        // 5. exhaustive search of every particle over its proposals
        for (unsigned i = 0; i < n; i++) {
            CcfGroup g{};
            g.sbj_sp = S.sbj_sp.p + (size_t)i * row_elems * Sn;
            g.ref_sp = S.ref_sp.p;
            g.ref_idx = S.prop.p + (size_t)i * k;
            g.base = bs ? bs + c0 + i : nullptr;
            g.d_out = S.dk.p + (size_t)i * k;
            g.peak_out = S.pkk.p + (size_t)i * k;
            g.n_part = 1;
            g.n_ref = k;
            g.p_total = 1;
            g.item_begin = i * tiles_k;
            g.ref_tiles = tiles_k;
            table[i] = g;
        }
        if ((rc = ccf(n, tiles_k)) != 0)
            return rc;
        best_of_kernel<<<(n + 7) / 8, 256, 0, st>>>(S.dk.p, S.pkk.p, S.prop.p, k, n, nullptr, best_ref + c0,
                                                     best_peak + c0, bparam + c0, best_gap ? best_gap + c0 : nullptr,
                                                     gap_margin, S.fb_flag.p);
        g_kernel_launches.fetch_add(1, std::memory_order_relaxed);
        P_CK(cudaGetLastError());
        n_pairs += (unsigned long long)n * k;
        // 6. particles below the margin: every reference
        P_CK(cudaMemcpyAsync(flags.data(), S.fb_flag.p, n * sizeof(unsigned), cudaMemcpyDeviceToHost, st));
        P_CK(cudaStreamSynchronize(st));
        if (fallback)
            P_CK(cudaMemcpyAsync(fallback + c0, S.fb_flag.p, n * sizeof(unsigned), cudaMemcpyDeviceToDevice, st));
        fbl.clear();
        for (unsigned i = 0; i < n; i++)
            if (flags[i])
                fbl.push_back(i);
        const unsigned nf = (unsigned)fbl.size();
        if (nf) {
            for (unsigned j = 0; j < nf; j++) {
                const unsigned i = fbl[j];
                CcfGroup g{};
                g.sbj_sp = S.sbj_sp.p + (size_t)i * row_elems * Sn;
                g.ref_sp = S.ref_sp.p;
                g.ref_idx = nullptr;
                g.base = bs ? bs + c0 + i : nullptr;
                g.d_out = S.dfb.p + (size_t)j * R;
                g.peak_out = S.pfb.p + (size_t)j * R;
                g.n_part = 1;
                g.n_ref = R;
                g.p_total = 1;
                g.item_begin = j * tiles_all;
                g.ref_tiles = tiles_all;
                table[j] = g;
            }
            P_CK(cudaMemcpyAsync(S.fb_list.p, fbl.data(), nf * sizeof(unsigned), cudaMemcpyHostToDevice, st));
            if ((rc = ccf(nf, tiles_all)) != 0)
                return rc;
            best_of_kernel<<<(nf + 7) / 8, 256, 0, st>>>(S.dfb.p, S.pfb.p, nullptr, R, nf, S.fb_list.p,
                                                          best_ref + c0, best_peak + c0, bparam + c0, nullptr, 0.f,
                                                          nullptr);
            g_kernel_launches.fetch_add(1, std::memory_order_relaxed);
            P_CK(cudaGetLastError());
            n_pairs += (unsigned long long)nf * R;
        }
        P_CK(cudaStreamSynchronize(st)); // the host table is rewritten by the next chunk
    }
#undef NN_CK
    if (pairs)
        *pairs = n_pairs;
    unsigned flag = 0;
    P_CK(cudaMemcpy(&flag, S.err.p, sizeof(unsigned), cudaMemcpyDeviceToHost));
    return flag ? fail(1, "a kernel timed out waiting for its own asynchronous copies") : 0;
}
