// groups.cu -- many independent alignment groups in one go.
//
// ISAC aligns uneven groups (generations, per-class subsets) one
// init / multi_ref_align / clear cycle at a time (bin/sp_isac2_gpu.py:937-1032
// per call).  gpuisac_multi_ref_align_groups_device runs all of them at once:
// reference spectra for every group, particle spectra in waves that pack
// consecutive groups into one buffer, and one persistent CCF / peak launch per
// wave whose work items span every group of the wave.  The launch sequence
// is captured in a CUDA graph the first time a given call is made and
// replayed when the same call is repeated.  Every group's results equal a
// separate multi-reference alignment of that group (the per-group image
// stacking of the reference is kept: each group is its own stack).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
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

#define G_CK(expr)                                                                        \
    do {                                                                                  \
        cudaError_t e_ = (expr);                                                          \
        if (e_ != cudaSuccess) {                                                          \
            char m_[384];                                                                 \
            snprintf(m_, sizeof(m_), "%s (%s) in the grouped alignment", cudaGetErrorString(e_), #expr); \
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

struct Segment {
    unsigned group;
    unsigned a, b;   // particles [a, b) of the group
    size_t row;      // first spectra row (particle) of the segment in the wave buffer
};

struct Wave {
    std::vector<Segment> segs;
    unsigned rows = 0;          // particles in the wave
    unsigned table_first = 0;   // first CcfGroup entry of the wave
    unsigned n_items = 0;
};

// the last call's plan and graph, replayed when the same call comes again
struct Plan {
    std::vector<unsigned char> key;
    cudaGraphExec_t exec = nullptr;
    cudaGraph_t graph = nullptr;
    cudaStream_t stream = nullptr;
};

struct GroupState {
    std::mutex mu;
    Buf<float2> tw, tmpl, shifts_f, ref_sp, sbj_sp;
    Buf<int2> shifts_i, zero;
    Buf<CcfGroup> table;
    Buf<unsigned> err;
    Plan plan;
    std::vector<TexStack> ref_tex, sbj_tex; // each group's stacks as textures
    std::vector<float2> h_tw, h_tmpl, h_sf;
    std::vector<int2> h_si;
} g_groups;

void drop_plan(Plan& pl)
{
    if (pl.exec)
        cudaGraphExecDestroy(pl.exec);
    if (pl.graph)
        cudaGraphDestroy(pl.graph);
    pl.exec = nullptr;
    pl.graph = nullptr;
    pl.key.clear();
}

void append(std::vector<unsigned char>& k, const void* p, size_t n)
{
    const unsigned char* c = static_cast<const unsigned char*>(p);
    k.insert(k.end(), c, c + n);
}

} // namespace

extern "C" int gpuisac_multi_ref_align_groups_device(const AlignConfig* cfg, const GpuisacGroup* groups,
                                                     unsigned int n_groups, const float* sbj, const float* ref,
                                                     const float* base_shift, float* d_out, float* peak_out,
                                                     void* stream)
{
    HostGeometry geo;
    int rc = host_geometry(cfg, geo);
    if (rc)
        return rc;
    if (n_groups == 0)
        return 0;
    if (!groups || !sbj || !ref || !d_out || !peak_out)
        return fail(2, "NULL group table or device pointer");
    for (unsigned i = 0; i < n_groups; i++) {
        const GpuisacGroup& g = groups[i];
        if ((size_t)g.sbj_offset + g.sbj_num > geo.P || (size_t)g.ref_offset + g.ref_num > geo.R) {
            char m[200];
            snprintf(m, sizeof(m), "group %u reaches outside the stacks (sbj %u+%u of %u, ref %u+%u of %u)", i,
                     g.sbj_offset, g.sbj_num, geo.P, g.ref_offset, g.ref_num, geo.R);
            return fail(2, m);
        }
    }
    std::lock_guard<std::mutex> lk(g_groups.mu);
    GroupState& S = g_groups;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int dev = 0;
    G_CK(cudaGetDevice(&dev));

    // the same call again: replay its graph
    std::vector<unsigned char> key;
    append(key, cfg, offsetof(AlignConfig, aln_type));
    append(key, groups, sizeof(GpuisacGroup) * n_groups);
    const void* ptrs[5] = {sbj, ref, base_shift, d_out, peak_out};
    append(key, ptrs, sizeof(ptrs));
    append(key, &dev, sizeof(dev));
    append(key, &st, sizeof(st));
    const CcfTile key_tile = ccf_tile(geo.NR, geo.S, true); // another tile shape records a new graph
    append(key, &key_tile, sizeof(key_tile));
    bool hw = texture_unit_enabled();
    append(key, &hw, sizeof(hw));
    if (S.plan.exec && S.plan.key == key) {
        G_CK(cudaMemsetAsync(S.err.p, 0, sizeof(unsigned), st));
        G_CK(cudaGraphLaunch(S.plan.exec, st));
        G_CK(cudaStreamSynchronize(st));
        unsigned flag = 0;
        G_CK(cudaMemcpy(&flag, S.err.p, sizeof(unsigned), cudaMemcpyDeviceToHost));
        return flag ? fail(1, "a kernel timed out waiting for its own asynchronous copies") : 0;
    }
    drop_plan(S.plan);

    // ---- plan: tables, reference spectra rows, waves ----
    const unsigned NR = geo.NR, Sn = geo.S, D = geo.D;
    const size_t row_elems = (size_t)NR * kSlots;
    const unsigned tex = texture_images(dev, D);
    const CcfTile tile = ccf_tile(NR, Sn, true);
    const int variant = tile.variant;
    const unsigned qt = ccf_refs_per_item(NR, variant);
    const unsigned ppc = tile.ppc;

    // every group's stacks as the reference's textures (allocated and bound
    // here; filled inside the recorded sequence)
    auto ref_desc = [&](const GpuisacGroup& g) {
        return StackDesc{ref + (size_t)g.ref_offset * D * D, g.ref_num, D, std::max(1u, std::min(g.ref_num, 100u)),
                         tex};
    };
    auto sbj_desc = [&](const GpuisacGroup& g) {
        AlignConfig gc = *cfg;
        gc.sbj_num = g.sbj_num;
        gc.ref_num = g.ref_num;
        return StackDesc{sbj + (size_t)g.sbj_offset * D * D, g.sbj_num, D, reference_batch(&gc), tex};
    };
    for (size_t i = n_groups; i < S.ref_tex.size(); i++) {
        S.ref_tex[i].release();
        S.sbj_tex[i].release();
    }
    S.ref_tex.resize(n_groups);
    S.sbj_tex.resize(n_groups);
    // (a texture set that cannot be made -- no memory for the copies, say --
    // leaves the whole plan on the emulation, which computes the same taps)
    for (unsigned gi = 0; hw && gi < n_groups; gi++) {
        const GpuisacGroup& g = groups[gi];
        if (g.ref_num == 0 || g.sbj_num == 0)
            continue;
        if (S.ref_tex[gi].prepare(ref_desc(g)) != cudaSuccess ||
            S.sbj_tex[gi].prepare(sbj_desc(g)) != cudaSuccess) {
            (void)cudaGetLastError();
            for (unsigned gj = 0; gj < n_groups; gj++) {
                S.ref_tex[gj].release();
                S.sbj_tex[gj].release();
            }
            hw = false;
        }
    }

    size_t free_b = 0, total_b = 0;
    G_CK(cudaMemGetInfo(&free_b, &total_b));
    const size_t per_part = row_elems * Sn * sizeof(float2);
    const size_t budget = (size_t)(0.4 * (double)free_b);
    const unsigned wave_cap = (unsigned)std::max<size_t>(1, std::min<size_t>(budget / per_part, 16384));

    std::vector<Wave> waves;
    std::vector<CcfGroup> table;
    {
        Wave cur;
        for (unsigned gi = 0; gi < n_groups; gi++) {
            const GpuisacGroup& g = groups[gi];
            if (g.sbj_num == 0 || g.ref_num == 0)
                continue;
            unsigned a = 0;
            while (a < g.sbj_num) {
                if (cur.rows == wave_cap) {
                    waves.push_back(cur);
                    cur = Wave();
                }
                const unsigned b = std::min(g.sbj_num, a + (wave_cap - cur.rows));
                cur.segs.push_back(Segment{gi, a, b, cur.rows});
                cur.rows += b - a;
                a = b;
            }
        }
        if (cur.rows)
            waves.push_back(cur);
    }
    // each group gets its own reference-spectra rows: a reference's sample
    // positions depend on its slot in its group's texture, so groups that
    // share references still need their own spectra
    std::vector<size_t> ref_row(n_groups, 0);
    size_t ref_rows = 0;
    for (unsigned gi = 0; gi < n_groups; gi++) {
        ref_row[gi] = ref_rows;
        ref_rows += groups[gi].ref_num;
    }
    G_CK(S.sbj_sp.ensure(row_elems * Sn * (size_t)wave_cap));
    G_CK(S.ref_sp.ensure(row_elems * std::max<size_t>(ref_rows, 1)));
    for (Wave& w : waves) {
        w.table_first = (unsigned)table.size();
        unsigned items = 0;
        for (const Segment& sg : w.segs) {
            const GpuisacGroup& g = groups[sg.group];
            CcfGroup c{};
            c.sbj_sp = S.sbj_sp.p + sg.row * row_elems * Sn;
            c.ref_sp = S.ref_sp.p + ref_row[sg.group] * row_elems;
            c.base = base_shift ? reinterpret_cast<const float2*>(base_shift) + g.sbj_offset : nullptr;
            c.d_out = d_out + g.out_offset;
            c.peak_out = reinterpret_cast<float4*>(peak_out) + g.out_offset;
            c.p_first = sg.a;
            c.n_part = sg.b - sg.a;
            c.n_ref = g.ref_num;
            c.p_total = g.sbj_num;
            c.item_begin = items;
            c.ref_tiles = (g.ref_num + qt - 1) / qt;
            items += c.ref_tiles * ((c.n_part + ppc - 1) / ppc);
            table.push_back(c);
        }
        w.n_items = items;
    }

    // ---- device tables (uploaded before the graph is recorded) ----
    G_CK(S.tw.ensure(kRingLen));
    G_CK(S.tmpl.ensure(geo.tmpl.size()));
    G_CK(S.shifts_f.ensure(Sn));
    G_CK(S.shifts_i.ensure(Sn));
    G_CK(S.zero.ensure(1));
    G_CK(S.err.ensure(1));
    G_CK(S.table.ensure(std::max<size_t>(table.size(), 1)));
    S.h_tw = geo.tw;
    S.h_tmpl = geo.tmpl;
    S.h_sf = geo.shifts_f;
    S.h_si = geo.shifts_i;
    const int2 zero = make_int2(0, 0);
    G_CK(cudaMemcpy(S.tw.p, S.h_tw.data(), kRingLen * sizeof(float2), cudaMemcpyHostToDevice));
    G_CK(cudaMemcpy(S.tmpl.p, S.h_tmpl.data(), S.h_tmpl.size() * sizeof(float2), cudaMemcpyHostToDevice));
    G_CK(cudaMemcpy(S.shifts_f.p, S.h_sf.data(), Sn * sizeof(float2), cudaMemcpyHostToDevice));
    G_CK(cudaMemcpy(S.shifts_i.p, S.h_si.data(), Sn * sizeof(int2), cudaMemcpyHostToDevice));
    G_CK(cudaMemcpy(S.zero.p, &zero, sizeof(int2), cudaMemcpyHostToDevice));
    if (!table.empty())
        G_CK(cudaMemcpy(S.table.p, table.data(), table.size() * sizeof(CcfGroup), cudaMemcpyHostToDevice));

    // ---- record the launch sequence into a graph ----
    cudaStream_t cap = nullptr;
    G_CK(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    G_CK(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = cudaSuccess;
    for (unsigned gi = 0; gi < n_groups && e == cudaSuccess; gi++) {
        const GpuisacGroup& g = groups[gi];
        if (g.ref_num == 0 || g.sbj_num == 0)
            continue;
        const StackDesc rs = ref_desc(g);
        if (hw) {
            e = S.ref_tex[gi].fill(rs, cap);
            if (e == cudaSuccess)
                e = S.sbj_tex[gi].fill(sbj_desc(g), cap);
            if (e != cudaSuccess)
                break;
        }
        e = launch_polar_spectra(rs, S.tmpl.p, S.tw.p, NR, S.zero.p, 1, nullptr, 0, g.ref_num, 1,
                                 S.ref_sp.p + ref_row[gi] * row_elems, cap, nullptr,
                                 hw ? S.ref_tex[gi].objects() : nullptr);
    }
    for (const Wave& w : waves) {
        for (const Segment& sg : w.segs) {
            if (e != cudaSuccess)
                break;
            const GpuisacGroup& g = groups[sg.group];
            const StackDesc ss = sbj_desc(g);
            const float2* bs = base_shift ? reinterpret_cast<const float2*>(base_shift) + g.sbj_offset : nullptr;
            e = launch_polar_spectra(ss, S.tmpl.p, S.tw.p, NR, S.shifts_i.p, Sn, bs, sg.a, sg.b - sg.a, 0,
                                     S.sbj_sp.p + sg.row * row_elems * Sn, cap, nullptr,
                                     hw ? S.sbj_tex[sg.group].objects() : nullptr);
        }
        if (e != cudaSuccess)
            break;
        CcfWork cw{};
        cw.groups = S.table.p + w.table_first;
        cw.n_groups = (unsigned)w.segs.size();
        cw.n_items = w.n_items;
        cw.ppc = ppc;
        e = launch_ccf_peak_work(cw, variant, S.tw.p, NR, Sn, S.shifts_f.p, S.err.p, cap);
    }
    cudaGraph_t graph = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(cap, &graph);
    cudaStreamDestroy(cap);
    if (e != cudaSuccess || e2 != cudaSuccess) {
        if (graph)
            cudaGraphDestroy(graph);
        char m[256];
        snprintf(m, sizeof(m), "recording the grouped alignment failed: %s",
                 cudaGetErrorString(e != cudaSuccess ? e : e2));
        return fail(1, m);
    }
    S.plan.graph = graph;
    G_CK(cudaGraphInstantiate(&S.plan.exec, graph, 0));
    S.plan.key = key;
    G_CK(cudaMemsetAsync(S.err.p, 0, sizeof(unsigned), st));
    G_CK(cudaGraphLaunch(S.plan.exec, st));
    G_CK(cudaStreamSynchronize(st));
    unsigned flag = 0;
    G_CK(cudaMemcpy(&flag, S.err.p, sizeof(unsigned), cudaMemcpyDeviceToHost));
    return flag ? fail(1, "a kernel timed out waiting for its own asynchronous copies") : 0;
}
