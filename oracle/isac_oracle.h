/*
 * isac_oracle.h -- CPU restatement of GPU-ISAC's multi-reference 2D alignment.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product path links, loads or calls
 * this library: it is the checker the CUDA path is compared against (tests/,
 * __graft_entry__.smoke()) and the timed CPU baseline of bench.py.
 *
 * It restates the arithmetic of the reference's GPU path (the only
 * implementation of this path that ships with the reference; its CPU
 * counterpart lives in the un-vendored EMAN2 C++ library):
 *
 *   polar template            cuda/gpu_aln_common.cu:39-62
 *   shift grid                cuda/gpu_aln_common.cu:64-86
 *   texture-unit sampling     cuda/gpu_aln_noref.cu:1258-1286, 2314-2339
 *   per-image normalisation   cuda/gpu_aln_noref.cu:1289-1352
 *   ring R2C FFT (cuFFT)      cuda/gpu_aln_noref.cu:2121-2125
 *   ring-weighted CCF         cuda/gpu_aln_noref.cu:1483-1537
 *   C2R of every table entry  cuda/gpu_aln_noref.cu:2453-2461
 *   peak search + parabola    cuda/gpu_aln_noref.cu:1667-1794
 *   host scatter (d, peaks)   cuda/gpu_aln_noref.cu:516-541
 *   batch / texture grouping  cuda/gpu_aln_noref.cu:429-440, 1831-1854
 *
 * Two precisions are built from one source (isac_oracle_core.h):
 *   orc_f64_*  -- every value after the sample positions is FP64; the error
 *                 reference for peak values;
 *   orc_f32_*  -- the same steps in FP32, the type the reference computes in;
 *                 used as the timed CPU baseline.
 * Sample positions and texture filter weights are computed exactly as the
 * reference and the texture unit do in both modes (they decide *which* pixels
 * are read, not rounding noise).
 */
#ifndef ISAC_ORACLE_H
#define ISAC_ORACLE_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Same fields and meaning as the reference's AlignConfig (cuda/gpu_aln_common.h:62-76),
 * minus the aln_type string, which only selects this path. */
typedef struct {
    unsigned sbj_num;
    unsigned ref_num;
    unsigned img_dim;
    unsigned ring_num;
    unsigned ring_len;
    float    shift_step;
    float    shift_rng_x;
    float    shift_rng_y;
} orc_cfg;

/* How the reference groups images into 2D textures.  Bilinear taps that fall
 * below/above an image read the neighbouring image of the same texture; the
 * first/last image of a texture clamps.  sbj_batch is the reference's subject
 * batch size (noref.cu:433-440), tex_limit its images-per-texture
 * (maxTexture2DLinear[1] / img_dim, noref.cu:1831), ref_batch the reference
 * batch (min(ref_num,100), noref.cu:431). */
typedef struct {
    unsigned sbj_batch;
    unsigned tex_limit;
    unsigned ref_batch;
} orc_layout;

/* polar template: out[(ring*ring_len + j)*2 + {0,1}] = (x, y) offsets */
void orc_polar_template(unsigned ring_num, unsigned ring_len, float *out);

/* shift grid, x outer / y inner; returns the number of shifts (<= cap) or -1 */
int orc_shift_array(float rng_x, float rng_y, float step, float *out_xy, int cap);

/* Texture-unit fixed-point filter weight of one coordinate: splits the
 * texel-space coordinate t into the integer texel index i = floor(t - 0.5)
 * (after the 8-bit rounding) and the weight a in [0,1) in 1/256 steps. */
void orc_tex_split(float t, int *i, float *a);

/* Bilinear tap weights (units of 1/256, summing to 256) of the texture unit
 * at texel-space point (x, y): w = {(ix,iy), (ix+1,iy), (ix,iy+1), (ix+1,iy+1)}. */
void orc_tex_weights(float x, float y, int *ix, int *iy, int w[4]);

/* Reference subject batch size for this config (the cuFFT int32 guard of
 * noref.cu:238; the device-memory half of that check is assumed to pass). */
unsigned orc_reference_sbj_batch(const orc_cfg *cfg);

#define ORC_DECLARE(P, REAL)                                                     \
/* polar resample + normalise one image of the stack; out [ring_num][ring_len] */\
int orc_##P##_polar(const orc_cfg *cfg, const orc_layout *lay,                   \
                    const float *stack, unsigned n_imgs, unsigned img,           \
                    int is_ref, float shift_x, float shift_y,                    \
                    const float *base_shift, REAL *out);                          \
/* ring spectra of one image; out [ring_num][ring_len/2+1][2] */                 \
int orc_##P##_spectra(const orc_cfg *cfg, const orc_layout *lay,                 \
                      const float *stack, unsigned n_imgs, unsigned img,         \
                      int is_ref, float shift_x, float shift_y,                  \
                      const float *base_shift, REAL *out);                        \
/* CCF of one (particle, ref) pair for every shift and mirror;                  \
 * out [2][n_shift][ring_len]  (mirror-major, like one ccf-table row) */         \
int orc_##P##_pair_ccf(const orc_cfg *cfg, const orc_layout *lay,                \
                       const float *sbj, const float *ref, unsigned p,           \
                       unsigned q, const float *base_shifts, REAL *out);         \
/* full multi_ref_align: peak_list [ref][sbj][4], d [ref][d_pitch] */           \
int orc_##P##_multi_ref_align(const orc_cfg *cfg, const orc_layout *lay,         \
                              const float *sbj, const float *ref,                \
                              const float *base_shifts, float *peak_list,        \
                              REAL *d, unsigned d_pitch, int n_threads);

ORC_DECLARE(f64, double)
ORC_DECLARE(f32, float)

/* peak search over one table row segment set: ccf [2*n_shift][ring_len]
 * (FP64 input), first strict max + 7-point parabola; writes
 * out4 = (angle, shift_idx, 0, mirror) and *peak */
void orc_f64_peak_search(const double *ccf, unsigned n_shift, unsigned ring_len,
                         float *out4, double *peak, unsigned *tau);

/* The multigroup alignment's class averages of transformed particles
 * (cu_transform_batch + cu_average_batch); see isac_oracle.c. */
int orc_multigroup_averages(const float *stack, unsigned n, unsigned dim, unsigned tex, const float *params,
                            const int *mirror, const unsigned *cid_idx, unsigned n_class, float *avg_out);

#ifdef __cplusplus
}
#endif
#endif
