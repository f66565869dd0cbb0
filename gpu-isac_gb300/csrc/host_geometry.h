// host_geometry.h -- host-side helpers of align_abi.cu shared with other
// translation units of this library.
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <vector>

#include "../../include/gpu_aln_pack.h"

namespace gpuisac {

// A named NVTX range for the lifetime of the object: the entry points and the
// particle chunks of the pipeline show up by name in a timeline or an
// ncu --nvtx capture (header-only NVTX; no cost without a tool attached).
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

// failure-path tests (gpuisac_test_fail_alloc): true while injected failures
// of workspace allocations are pending; each call consumes one
bool take_injected_alloc_failure();

struct HostGeometry {
    unsigned P = 0, R = 0, D = 0, NR = 0, S = 0;
    std::vector<float2> shifts_f; // the reference's float shift grid
    std::vector<int2> shifts_i;   // truncated to int, as the resample kernel receives them
    std::vector<float2> tmpl;     // polar template [NR][256]
    std::vector<float2> tw;       // e^(-2 pi i e / 256), e = 0..255
    unsigned sbj_batch = 1;       // the reference's subject batch size
};

// Validates cfg exactly as every entry point does (recording the error on
// failure) and fills the host tables.  Returns 0 or an error code.
int host_geometry(const AlignConfig* cfg, HostGeometry& out);

// The reference's subject batch size for cfg (its sbj_num / ref_num).
unsigned reference_batch(const AlignConfig* cfg);

// Images of side dim per 2D linear texture on device dev.
unsigned texture_images(int dev, unsigned dim);

// Records an error for gpuisac_last_error and prints it.
void record_error(int code, const char* msg);

// The reference's shift grid (x outer, y inner, float accumulation).
std::vector<float2> shift_grid_of(float rx, float ry, float step);

// The pre-alignment session (prealign.cu): reset_shifts on it (-1 when none
// is open, else 0 or an error code) and its release by gpu_clear.
int prealign_reset_shifts(float shift_range, float shift_step);
void prealign_clear();

// Copies n host images of img_elems floats (one pointer per image) into the
// device stack dst on `stream` and waits for the copies (host_upload.cu):
// pageable images through pinned staging filled by several host threads, a
// contiguous pinned stack directly.  A NULL image pointer returns
// cudaErrorInvalidValue with its index in *bad.
cudaError_t upload_host_images(const float* const* imgs, unsigned n, size_t img_elems, float* dst,
                               cudaStream_t stream, unsigned* bad);
// Frees the pinned staging area (gpu_clear).
void release_upload_staging();

// The multigroup session (multigroup.cu), likewise.
int multigroup_reset_shifts(float shift_range, float shift_step);
void multigroup_clear();

// The work spaces of the group assignment (assign.cu) and of the averaging
// step (averages.cu), released by gpu_clear.
void assign_clear();
void averages_clear();

} // namespace gpuisac
