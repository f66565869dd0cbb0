// groups.cu -- many independent alignment groups in one go.
//
// ISAC aligns uneven groups (generations, per-class subsets) one
// init / multi_ref_align / clear cycle at a time (bin/sp_isac2_gpu.py:937-1032
// per call).  gpuisac_multi_ref_align_groups_device runs all of them at once
// with a launch sequence whose shape does not depend on the groups:
//
//   one texture fill over every group's stacks (each group is its own stack,
//     laid out as the reference's textures hold it),
//   per wave of particles: one spectra launch (the first wave's also computes
//     every group's reference spectra) and one persistent CCF / peak launch
//     whose work items span every group of the wave.
//
// Every launch reads its work from device tables (spectra jobs, CCF group
// tables, row and item counts), so the sequence recorded into a CUDA graph
// for a number of waves is replayed by any later call with that many waves:
// a new set of groups rewrites the tables and the texture objects and
// launches the recorded graph -- 1 + 2 x waves launches, no re-capture.
// Every group's results equal a separate multi-reference alignment of that
// group.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
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
    unsigned rows = 0; // particles in the wave
};

// Capacities of the device table region; they only grow (rounded up to
// powers of two), so that a recorded graph outlives calls of other sizes.
struct Caps {
    unsigned waves = 0, groups = 0, jobs = 0, fills = 0, objs = 0, luts = 0;
    unsigned rows = 0; // spectra rows of the largest wave (the spectra launches' grid)
};

// Table region: [hdr words][CcfGroup x groups][SpectraJob x jobs][TexFillJob x fills][texture objects x objs]
// [job lookup x luts].  hdr: per wave kHdrWave words -- CCF {first group,
// groups, items}, spectra {first job, jobs, rows, lookup offset} -- then the
// fill's {jobs, rows}.
constexpr unsigned kHdrWave = 7;
struct Layout {
    size_t hdr = 0, groups = 0, jobs = 0, fills = 0, objs = 0, luts = 0, bytes = 0;
};

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

Layout layout_of(const Caps& c)
{
    Layout l;
    size_t o = 0;
    l.hdr = o;
    o = align_up(o + (kHdrWave * (size_t)c.waves + 2) * sizeof(unsigned), 256);
    l.groups = o;
    o = align_up(o + (size_t)c.groups * sizeof(CcfGroup), 256);
    l.jobs = o;
    o = align_up(o + (size_t)c.jobs * sizeof(SpectraJob), 256);
    l.fills = o;
    o = align_up(o + (size_t)c.fills * sizeof(TexFillJob), 256);
    l.objs = o;
    o = align_up(o + (size_t)c.objs * sizeof(unsigned long long), 256);
    l.luts = o;
    o = align_up(o + (size_t)c.luts * sizeof(unsigned), 256);
    l.bytes = o;
    return l;
}

unsigned pow2_at_least(size_t v, unsigned lo)
{
    unsigned p = lo;
    while (p < v)
        p <<= 1;
    return p;
}

// a recorded launch sequence and what it was recorded for
struct Rec {
    std::vector<unsigned char> key;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

struct GroupState {
    std::mutex mu;
    Buf<float2> tw, tmpl, shifts_f, ref_sp, sbj_sp;
    Buf<int2> shifts_i, zero;
    Buf<unsigned char> tables;
    Buf<unsigned> err;
    Caps caps;
    TexSet texs;
    std::vector<unsigned char> h_tables;
    std::vector<Rec> recs; // most recent last
    GpuisacGroupStats stats{};
} g_groups;

constexpr size_t kMaxRecs = 4;

void append(std::vector<unsigned char>& k, const void* p, size_t n)
{
    const unsigned char* c = static_cast<const unsigned char*>(p);
    k.insert(k.end(), c, c + n);
}

double ms_since(std::chrono::steady_clock::time_point t0)
{
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

} // namespace

extern "C" int gpuisac_groups_stats(GpuisacGroupStats* out)
{
    if (!out)
        return fail(2, "gpuisac_groups_stats: NULL output");
    std::lock_guard<std::mutex> lk(g_groups.mu);
    *out = g_groups.stats;
    return 0;
}

extern "C" int gpuisac_multi_ref_align_groups_device(const AlignConfig* cfg, const GpuisacGroup* groups,
                                                     unsigned int n_groups, const float* sbj, const float* ref,
                                                     const float* base_shift, float* d_out, float* peak_out,
                                                     void* stream)
{
    const gpuisac::NvtxRange nvtx_range("gpuisac:multi_ref_align_groups");
    const auto t_call = std::chrono::steady_clock::now();
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
    S.stats = GpuisacGroupStats{};
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int dev = 0, sms = 0;
    G_CK(cudaGetDevice(&dev));
    G_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));

    const unsigned NR = geo.NR, Sn = geo.S, D = geo.D;
    const size_t row_elems = (size_t)NR * kSlots;
    const unsigned tex = texture_images(dev, D);
    const CcfTile tile = ccf_tile(NR, Sn, true);
    const unsigned qt = ccf_refs_per_item(NR, tile.variant);
    const unsigned ppc = tile.ppc;

    // ---- the groups' stacks as the reference's textures ----
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
    std::vector<unsigned> live; // groups with work
    for (unsigned gi = 0; gi < n_groups; gi++)
        if (groups[gi].sbj_num && groups[gi].ref_num)
            live.push_back(gi);
    if (live.empty())
        return 0;
    bool hw = texture_unit_enabled();
    if (hw) {
        std::vector<StackDesc> stacks;
        for (unsigned gi : live) {
            stacks.push_back(ref_desc(groups[gi]));
            stacks.push_back(sbj_desc(groups[gi]));
        }
        // (a texture set that cannot be made -- no memory for the copies,
        // say -- leaves the call on the emulation: the same texels and
        // weights, the filtered value equal to the last bit or two)
        if (S.texs.prepare(stacks) != cudaSuccess) {
            (void)cudaGetLastError();
            S.texs.release();
            hw = false;
        }
    }

    // ---- waves of particles, as many as the spectra buffer needs ----
    size_t free_b = 0, total_b = 0;
    G_CK(cudaMemGetInfo(&free_b, &total_b));
    const size_t per_part = row_elems * Sn * sizeof(float2);
    const size_t held = S.sbj_sp.n * sizeof(float2);
    const size_t budget = (size_t)(0.45 * (double)(free_b + held));
    // (waves of 32768 particles: 15 at 4.8e5 particles, as fast as smaller
    // waves and 2 % faster than waves of 65536)
    size_t cap_parts = std::min<size_t>(budget / per_part, 32768);
    if (const char* e = std::getenv("GPUISAC_GROUP_WAVE")) // particles per wave, smaller (tests of many waves)
        cap_parts = std::min<size_t>(cap_parts, (size_t)std::strtoul(e, nullptr, 10));
    const unsigned wave_cap = (unsigned)std::max<size_t>(1, cap_parts);
    std::vector<Wave> waves;
    {
        Wave cur;
        for (unsigned gi : live) {
            const GpuisacGroup& g = groups[gi];
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
    const unsigned W = (unsigned)waves.size();
    size_t max_rows = 0, n_segs = 0;
    for (const Wave& w : waves) {
        max_rows = std::max<size_t>(max_rows, w.rows);
        n_segs += w.segs.size();
    }
    // each group gets its own reference-spectra rows: a reference's sample
    // positions depend on its slot in its group's texture, so groups that
    // share references still need their own spectra
    std::vector<size_t> ref_row(n_groups, 0);
    size_t ref_rows = 0;
    for (unsigned gi : live) {
        ref_row[gi] = ref_rows;
        ref_rows += groups[gi].ref_num;
    }
    G_CK(S.sbj_sp.ensure(row_elems * Sn * max_rows));
    G_CK(S.ref_sp.ensure(row_elems * ref_rows));
    G_CK(S.tw.ensure(kRingLen));
    G_CK(S.tmpl.ensure(geo.tmpl.size()));
    G_CK(S.shifts_f.ensure(Sn));
    G_CK(S.shifts_i.ensure(Sn));
    G_CK(S.zero.ensure(1));
    G_CK(S.err.ensure(2)); // the timeout flag and the CCF kernels' work counter

    // spectra rows of each wave (the first also computes the reference rows)
    std::vector<size_t> wave_rows(W);
    size_t lut_total = 0, rows_max = 0;
    for (unsigned w = 0; w < W; w++) {
        wave_rows[w] = (size_t)waves[w].rows * Sn + (w == 0 ? ref_rows : 0);
        if (wave_rows[w] > 0xFFFFFFFFull)
            return fail(2, "a wave of the grouped alignment has more than 2^32 spectra rows");
        lut_total += (wave_rows[w] + kJobLutRows - 1) / kJobLutRows;
        rows_max = std::max(rows_max, wave_rows[w]);
    }

    // ---- device tables ----
    Caps need;
    need.waves = pow2_at_least(W, 4);
    need.groups = pow2_at_least(n_segs, 256);
    need.jobs = pow2_at_least(live.size() + n_segs, 256);
    need.fills = pow2_at_least(2 * live.size(), 256);
    need.objs = pow2_at_least(hw ? S.texs.objs.size() : 1, 1024);
    need.luts = pow2_at_least(lut_total, 4096);
    need.rows = (unsigned)std::min<size_t>(0x7FFFFFFFull, (rows_max + 65535) / 65536 * 65536);
    Caps caps = S.caps;
    caps.waves = std::max(caps.waves, need.waves);
    caps.groups = std::max(caps.groups, need.groups);
    caps.jobs = std::max(caps.jobs, need.jobs);
    caps.fills = std::max(caps.fills, need.fills);
    caps.objs = std::max(caps.objs, need.objs);
    caps.luts = std::max(caps.luts, need.luts);
    caps.rows = std::max(caps.rows, need.rows);
    const Layout L = layout_of(caps);
    G_CK(S.tables.ensure(L.bytes));
    S.caps = caps;
    unsigned char* const dt = S.tables.p;
    std::vector<unsigned char>& ht = S.h_tables;
    ht.assign(L.bytes, 0);
    unsigned* hdr = reinterpret_cast<unsigned*>(ht.data() + L.hdr);
    CcfGroup* htab = reinterpret_cast<CcfGroup*>(ht.data() + L.groups);
    SpectraJob* hjob = reinterpret_cast<SpectraJob*>(ht.data() + L.jobs);
    TexFillJob* hfill = reinterpret_cast<TexFillJob*>(ht.data() + L.fills);
    unsigned* hlut = reinterpret_cast<unsigned*>(ht.data() + L.luts);
    const unsigned long long* d_objs = reinterpret_cast<const unsigned long long*>(dt + L.objs);
    if (hw) {
        std::copy(S.texs.objs.begin(), S.texs.objs.end(), reinterpret_cast<unsigned long long*>(ht.data() + L.objs));
        std::copy(S.texs.jobs.begin(), S.texs.jobs.end(), hfill);
        hdr[kHdrWave * caps.waves] = (unsigned)S.texs.jobs.size();
        hdr[kHdrWave * caps.waves + 1] = S.texs.rows;
    }
    // the stack index of group gi's references in the texture set is 2 k,
    // its particles' 2 k + 1, for its place k among the live groups
    std::vector<unsigned> live_pos(n_groups, 0);
    for (size_t k = 0; k < live.size(); k++)
        live_pos[live[k]] = (unsigned)k;
    auto objs_of = [&](unsigned gi, bool is_ref) -> const unsigned long long* {
        return hw ? d_objs + S.texs.obj_first[2 * live_pos[gi] + (is_ref ? 0 : 1)] : nullptr;
    };
    const float2* bs_all = reinterpret_cast<const float2*>(base_shift);
    unsigned n_tab = 0, n_job = 0, n_lut = 0;
    for (unsigned w = 0; w < W; w++) {
        const Wave& wv = waves[w];
        const unsigned job_first = n_job;
        unsigned rows = 0;
        if (w == 0) {
            for (unsigned gi : live) {
                const GpuisacGroup& g = groups[gi];
                SpectraJob& j = hjob[n_job++];
                j.st = ref_desc(g);
                j.tex_objs = objs_of(gi, true);
                j.base = nullptr;
                j.shift_int = S.zero.p;
                j.out = S.ref_sp.p + ref_row[gi] * row_elems;
                j.img0 = 0;
                j.n_img = g.ref_num;
                j.n_shift = 1;
                j.is_ref = 1;
                j.row_begin = rows;
                rows += g.ref_num;
            }
        }
        const unsigned tab_first = n_tab;
        unsigned items = 0;
        for (const Segment& sg : wv.segs) {
            const GpuisacGroup& g = groups[sg.group];
            const float2* bs = bs_all ? bs_all + g.sbj_offset : nullptr;
            SpectraJob& j = hjob[n_job++];
            j.st = sbj_desc(g);
            j.tex_objs = objs_of(sg.group, false);
            j.base = bs;
            j.shift_int = S.shifts_i.p;
            j.out = S.sbj_sp.p + sg.row * row_elems * Sn;
            j.img0 = sg.a;
            j.n_img = sg.b - sg.a;
            j.n_shift = Sn;
            j.is_ref = 0;
            j.row_begin = rows;
            rows += j.n_img * Sn;

            CcfGroup& c = htab[n_tab++];
            c.sbj_sp = j.out;
            c.ref_sp = S.ref_sp.p + ref_row[sg.group] * row_elems;
            c.base = bs;
            c.d_out = d_out + g.out_offset;
            c.peak_out = reinterpret_cast<float4*>(peak_out) + g.out_offset;
            c.p_first = sg.a;
            c.n_part = sg.b - sg.a;
            c.n_ref = g.ref_num;
            c.p_total = g.sbj_num;
            c.item_begin = items;
            c.ref_tiles = (g.ref_num + qt - 1) / qt;
            c.ref_idx = nullptr;
            c.rule = kPeakMref;
            items += c.ref_tiles * ((c.n_part + ppc - 1) / ppc);
        }
        // the job holding the first row of every block of kJobLutRows rows
        const unsigned lut_first = n_lut;
        for (unsigned b = 0, jj = job_first; (size_t)b * kJobLutRows < rows; b++) {
            while (jj + 1 < n_job && hjob[jj + 1].row_begin <= b * kJobLutRows)
                jj++;
            hlut[n_lut++] = jj;
        }
        unsigned* h = hdr + kHdrWave * w;
        h[0] = tab_first;
        h[1] = n_tab - tab_first;
        h[2] = items;
        h[3] = job_first;
        h[4] = n_job - job_first;
        h[5] = rows;
        h[6] = lut_first;
    }
    G_CK(cudaMemcpy(S.tw.p, geo.tw.data(), kRingLen * sizeof(float2), cudaMemcpyHostToDevice));
    G_CK(cudaMemcpy(S.tmpl.p, geo.tmpl.data(), geo.tmpl.size() * sizeof(float2), cudaMemcpyHostToDevice));
    G_CK(cudaMemcpy(S.shifts_f.p, geo.shifts_f.data(), Sn * sizeof(float2), cudaMemcpyHostToDevice));
    G_CK(cudaMemcpy(S.shifts_i.p, geo.shifts_i.data(), Sn * sizeof(int2), cudaMemcpyHostToDevice));
    const int2 zero = make_int2(0, 0);
    G_CK(cudaMemcpy(S.zero.p, &zero, sizeof(int2), cudaMemcpyHostToDevice));
    G_CK(cudaMemcpy(dt, ht.data(), L.bytes, cudaMemcpyHostToDevice));
    S.stats.plan_ms = ms_since(t_call);

    // ---- the recorded sequence for this shape, or a new recording ----
    // one CTA per spectra row of the largest wave the tables can describe
    const unsigned spec_grid = caps.rows;
    const unsigned fill_grid = (unsigned)std::max(1, sms) * 8;
    std::vector<unsigned char> key;
    const void* ptrs[9] = {dt, S.tw.p, S.tmpl.p, S.shifts_f.p, S.shifts_i.p, S.zero.p, S.err.p, nullptr, nullptr};
    append(key, ptrs, sizeof(ptrs));
    const unsigned shape[8] = {(unsigned)dev, NR, Sn, W, caps.waves, spec_grid, hw ? 1u : 0u, ccf_tile_generation()};
    append(key, shape, sizeof(shape));
    append(key, &tile, sizeof(tile));
    append(key, &caps, sizeof(caps)); // the table layout
    size_t ri = 0;
    while (ri < S.recs.size() && S.recs[ri].key != key)
        ri++;
    if (ri == S.recs.size()) {
        const auto t_rec = std::chrono::steady_clock::now();
        cudaStream_t cap = nullptr;
        G_CK(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
        G_CK(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
        const unsigned* d_hdr = reinterpret_cast<const unsigned*>(dt + L.hdr);
        cudaError_t e = cudaSuccess;
        if (hw)
            e = launch_tex_fill_jobs(reinterpret_cast<const TexFillJob*>(dt + L.fills), d_hdr + kHdrWave * caps.waves,
                                     fill_grid, cap);
        for (unsigned w = 0; w < W && e == cudaSuccess; w++) {
            e = launch_polar_spectra_jobs(reinterpret_cast<const SpectraJob*>(dt + L.jobs), d_hdr + kHdrWave * w + 3,
                                          reinterpret_cast<const unsigned*>(dt + L.luts), S.tmpl.p, S.tw.p, NR,
                                          spec_grid, cap);
            if (e != cudaSuccess)
                break;
            CcfWork cw{};
            cw.groups = reinterpret_cast<const CcfGroup*>(dt + L.groups);
            cw.dyn = d_hdr + kHdrWave * w;
            cw.n_groups = 1;
            cw.n_items = 0xFFFFFFFFu; // a grid over every SM; the items come from dyn
            cw.ppc = ppc;
            cw.item_counter = S.err.p + 1;
            e = launch_ccf_peak_work(cw, tile.variant, S.tw.p, NR, Sn, S.shifts_f.p, S.err.p, cap);
        }
        cudaGraph_t graph = nullptr;
        const cudaError_t e2 = cudaStreamEndCapture(cap, &graph);
        cudaStreamDestroy(cap);
        if (e != cudaSuccess || e2 != cudaSuccess) {
            if (graph)
                cudaGraphDestroy(graph);
            char m[256];
            snprintf(m, sizeof(m), "recording the grouped alignment failed: %s",
                     cudaGetErrorString(e != cudaSuccess ? e : e2));
            return fail(1, m);
        }
        Rec r;
        r.key = key;
        r.graph = graph;
        e = cudaGraphInstantiate(&r.exec, graph, 0);
        if (e != cudaSuccess) {
            cudaGraphDestroy(graph);
            G_CK(e);
        }
        if (S.recs.size() == kMaxRecs) {
            cudaGraphExecDestroy(S.recs.front().exec);
            cudaGraphDestroy(S.recs.front().graph);
            S.recs.erase(S.recs.begin());
        }
        S.recs.push_back(r);
        ri = S.recs.size() - 1;
        S.stats.record_ms = ms_since(t_rec);
        S.stats.graphs_recorded = 1;
        // the launchers counted the launches they recorded; they run below
        g_kernel_launches.fetch_sub((hw ? 1u : 0u) + 2 * W, std::memory_order_relaxed);
    }
    S.stats.waves = W;
    S.stats.graph_launches = (hw ? 1u : 0u) + 2 * W;
    G_CK(cudaMemsetAsync(S.err.p, 0, sizeof(unsigned), st));
    G_CK(cudaGraphLaunch(S.recs[ri].exec, st));
    g_kernel_launches.fetch_add(S.stats.graph_launches, std::memory_order_relaxed);
    G_CK(cudaStreamSynchronize(st));
    unsigned flag = 0;
    G_CK(cudaMemcpy(&flag, S.err.p, sizeof(unsigned), cudaMemcpyDeviceToHost));
    return flag ? fail(1, "a kernel timed out waiting for its own asynchronous copies") : 0;
}
