// autotune.cu -- chooses the CCF launch's tile shape by timing.
//
// gpuisac_autotune_ccf times every candidate tile shape (kernel variant,
// contraction warps of the warp-specialised kernel, particles per work item)
// on a sample of the caller's own stacks through the device entry point, and
// records the fastest for the call's (ring count, shift count).  Every
// candidate runs the same arithmetic in the same order, so the choice changes
// only the speed, never a result.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/gpu_aln_pack.h"
#include "gpuisac_kernels.h"
#include "host_geometry.h"

using namespace gpuisac;

namespace {

const char* variant_name(int v) { return v == kCcfWs ? "ws" : (v == kCcfTmem ? "tmem" : "general"); }

std::string tile_text(const CcfTile& t)
{
    char b[64];
    if (t.variant == kCcfWs)
        snprintf(b, sizeof(b), "ws%d/ppc%u", t.ws_warps, t.ppc);
    else
        snprintf(b, sizeof(b), "%s/ppc%u", variant_name(t.variant), t.ppc);
    return b;
}

void copy_text(const std::string& s, char* buf, size_t len)
{
    if (!buf || len == 0)
        return;
    size_t n = std::min(len - 1, s.size());
    memcpy(buf, s.data(), n);
    buf[n] = 0;
}

} // namespace

extern "C" int gpuisac_autotune_ccf(const AlignConfig* cfg, const float* sbj, const float* ref,
                                    unsigned int n_sample, char* report, size_t report_len, void* stream)
{
    HostGeometry geo;
    int rc = host_geometry(cfg, geo);
    if (rc)
        return rc;
    if (!sbj || !ref) {
        record_error(2, "NULL device pointer");
        return 2;
    }
    const unsigned n = std::min(geo.P, n_sample ? n_sample : 2048u);
    AlignConfig c = *cfg;
    c.sbj_num = n;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    float *d = nullptr, *pk = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    auto cleanup = [&]() {
        ccf_tile_force(nullptr);
        contraction_force(-1);
        if (d)
            cudaFree(d);
        if (pk)
            cudaFree(pk);
        if (e0)
            cudaEventDestroy(e0);
        if (e1)
            cudaEventDestroy(e1);
    };
    if (cudaMalloc(&d, (size_t)geo.R * n * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&pk, (size_t)geo.R * n * 4 * sizeof(float)) != cudaSuccess ||
        cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        cleanup();
        record_error(1, "cannot allocate the autotuner's buffers");
        return 1;
    }
    std::vector<CcfTile> cand;
    const unsigned ppcs[3] = {4, 8, 16};
    if (ccf_tile(geo.NR, geo.S, true).variant != kCcfGeneral) {
        for (unsigned ppc : ppcs) {
            cand.push_back({kCcfWs, 8, ppc});
            cand.push_back({kCcfWs, 4, ppc});
            if (ccf_tile_allows_tmem(geo.NR))
                cand.push_back({kCcfTmem, 8, ppc});
        }
    } else {
        for (unsigned ppc : ppcs)
            cand.push_back({kCcfGeneral, 8, ppc});
    }
    std::string rep;
    float best_ms = 1e30f;
    CcfTile best = cand[0];
    // the candidates are tile shapes of the FP32 CCF kernels: time them with
    // that contraction whatever the process-wide mode
    contraction_force(GPUISAC_CONTRACTION_FP32);
    for (size_t i = 0; i < cand.size(); i++) {
        ccf_tile_force(&cand[i]);
        float ms = 1e30f;
        for (int r = 0; r < (i == 0 ? 3 : 2); r++) { // the first candidate also warms the work space
            cudaEventRecord(e0, st);
            rc = gpuisac_multi_ref_align_device(&c, sbj, ref, nullptr, d, pk, stream);
            cudaEventRecord(e1, st);
            if (rc) {
                cleanup();
                return rc;
            }
            cudaEventSynchronize(e1);
            float t = 0.f;
            cudaEventElapsedTime(&t, e0, e1);
            ms = std::min(ms, t);
        }
        char b[96];
        snprintf(b, sizeof(b), "%s%s %.3f ms", rep.empty() ? "" : "; ", tile_text(cand[i]).c_str(), ms);
        rep += b;
        if (ms < best_ms) {
            best_ms = ms;
            best = cand[i];
        }
    }
    cleanup();
    ccf_tile_record(geo.NR, geo.S, best);
    rep += "; chosen " + tile_text(best);
    copy_text(rep, report, report_len);
    return 0;
}

extern "C" int gpuisac_ccf_tile_name(unsigned int ring_num, unsigned int n_shift, char* buf, size_t len)
{
    copy_text(tile_text(ccf_tile(ring_num, n_shift, true)), buf, len);
    return 0;
}
