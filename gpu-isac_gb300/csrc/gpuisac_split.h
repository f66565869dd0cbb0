// gpuisac_split.h -- host side of the tensor-core (BF16 hi/lo split)
// contraction: tile plan, work descriptors and launchers (ccf_split.cu).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

#include "gpuisac_kernels.h"

namespace gpuisac {

// shifts per shift block: one block fills at most 98 of the MMA's 128 lanes,
// and its Z block (256 x 49 float2, 100 KB) is double-buffered in the FFT
// kernel's shared memory
constexpr unsigned kSplitMaxBlock = 49;

// Tile plan of one (ring count, shift count, reference count).
struct SplitPlan {
    unsigned n_blocks = 0;   // shift blocks per particle
    unsigned block = 0;      // shifts per block (the last may have fewer)
    unsigned zw = 0;         // row length of a Z block: block rounded up to odd
    unsigned kg = 0;         // K groups of 8 rings stored
    unsigned rga = 0;        // row groups of a subject tile (2 rows per shift)
    unsigned rblock = 0;     // references per reference tile
    unsigned n_rtiles = 0;   // reference tiles
    unsigned n_cols = 0;     // MMA N: 2 x rblock rounded up to 16
    unsigned rgb = 0;        // row groups of a reference tile (n_cols / 8)
    unsigned n_stages = 0;   // operand stages of the MMA kernel
    unsigned rounds = 1;     // shifts per FFT group and block (1: a group per shift)
    unsigned fft_groups = 0; // 16-thread FFT groups of the FFT kernel
    size_t sop_slot = 0;     // bytes of one subject tile's slot (hi + lo)
    size_t rop_slot = 0;     // bytes of one reference tile's slot (hi + lo)
};

struct SplitMmaWork {
    const unsigned char* sop; // subject operand tiles [n_part x n_blocks][kSlots][sop_slot]
    const unsigned char* rop; // reference operand tiles [n_rtiles][kSlots][rop_slot]
    float2* z;                // ring sums [n_part][n_ref][n_blocks][128 slots][zw][a|b] of (sum u, sum v)
    unsigned n_part, n_blocks, block, n_shift;
    unsigned n_ref, rblock, n_rtiles;
    unsigned kg, rga, rgb, n_cols, n_stages, zw;
    size_t sop_slot, rop_slot;
    unsigned n_items;         // n_part x n_blocks x n_rtiles
    unsigned test_stall, wait_iters; // failure-path tests only (CcfWork)
};

struct SplitFftWork {
    const float2* z;
    unsigned n_part, n_ref, n_shift, n_blocks, block, zw;
    unsigned p_first, p_total; // output columns: particle p of the chunk -> p_first + p of a [n_ref][p_total] array
    const float2* shifts_f;
    const float2* base;        // base shifts by global particle index, or null
    float* d_out;
    float4* peak_out;
    unsigned rule;
    unsigned test_stall, wait_iters; // failure-path tests only (CcfWork)
};

// false when the shape does not fit the kernels' shared memory
bool split_plan(unsigned ring_num, unsigned n_shift, unsigned n_ref, SplitPlan& p);
size_t split_sop_bytes(const SplitPlan& p, unsigned n_part);
size_t split_rop_bytes(const SplitPlan& p);
size_t split_z_bytes(const SplitPlan& p, unsigned n_part, unsigned n_ref);
OperandLayout split_sbj_layout(const SplitPlan& p, unsigned char* base);
OperandLayout split_ref_layout(const SplitPlan& p, unsigned char* base);

// contraction of n_part particles whose operands are in sop against all
// n_ref references (rop) into the pair spectra z (split_z_bytes(p, n_part,
// n_ref) bytes): ccf_mma_kernel
cudaError_t launch_ccf_mma(const SplitPlan& p, const unsigned char* sop, const unsigned char* rop, float2* z,
                           unsigned n_part, unsigned n_ref, unsigned n_shift, unsigned* err, cudaStream_t stream);

// inverse FFT + peak search of those pair spectra (zfft_peak_kernel); results
// to column p_first + i of d_out / peak_out [n_ref][p_total]
cudaError_t launch_zfft_peak(const SplitPlan& p, const float2* z, unsigned n_part, unsigned p_first,
                             unsigned p_total, unsigned n_ref, unsigned n_shift, const float2* twiddle,
                             const float2* shifts_f, const float2* base, float* d_out, float4* peak_out,
                             unsigned* err, cudaStream_t stream, unsigned rule = kPeakMref);

} // namespace gpuisac
