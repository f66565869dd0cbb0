/*
 * gpu_aln_pack.h -- C-ABI of the GB300 multi-reference alignment library
 * (libgpu_aln_pack.so, a drop-in for the reference's gpu_aln_pack.so).
 *
 * Every declaration below names the reference interface it replaces
 * (paths inside the GPU-ISAC repository).  Types are plain C: no CUDA or
 * PyTorch types cross this boundary.  Callers bind it with ctypes exactly as
 * bin/sp_isac2_gpu.py:121-187 and bin/sp_isac_applications.py:86-157 do.
 */
#ifndef GPU_ALN_PACK_H
#define GPU_ALN_PACK_H

#include <stdbool.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Replaces struct AlignConfig, cuda/gpu_aln_common.h:62-76 (40 bytes on LP64;
 * the pointer is stored, not copied, so the struct must outlive the calls).
 * Python mirror: bin/sp_isac2_gpu.py:139-152. */
typedef struct AlignConfig {
    unsigned int sbj_num;
    unsigned int ref_num;
    unsigned int img_dim;
    unsigned int ring_num;
    unsigned int ring_len;
    float shift_step;
    float shift_rng_x;
    float shift_rng_y;
    const char *aln_type; /* "mref_aln" for the multi-reference path */
} AlignConfig;

/* Replaces struct AlignParam, cuda/gpu_aln_common.h:78-85 (24 bytes).
 * Python mirror: bin/sp_isac2_gpu.py:154-160.  The multi-reference path reads
 * shift_x / shift_y as each particle's base shift. */
typedef struct AlignParam {
    int sbj_id;
    int ref_id;
    float shift_x;
    float shift_y;
    float angle;
    bool mirror;
} AlignParam;

/* ---- multi-reference alignment (the hot path) ---- */

/* Replaces multi_ref_align_init, cuda/gpu_aln_noref.h:61-64 /
 * cuda/gpu_aln_noref.cu:311-324.  Selects the device, builds the polar
 * template and shift grid, and returns a zero-filled, host-writable
 * AlignParam[sbj_num] owned by the library (freed by gpu_clear).
 * Returns NULL on error (see gpuisac_last_error). */
AlignParam *multi_ref_align_init(const AlignConfig *aln_cfg, unsigned int cuda_device_id);

/* Replaces multi_ref_align, cuda/gpu_aln_noref.h:66-73 /
 * cuda/gpu_aln_noref.cu:326-554.  sbj_data: sbj_num pointers to img_dim^2
 * float images (row-major); ref_data: ref_num pointers.  Writes
 * isac_peak_list[(q*sbj_num + p)*4 + {0..3}] = (angle, shift_x, shift_y,
 * mirror) and isac_d[q*isac_d_pitch + p] = the peak correlation, for every
 * reference q and particle p.  cuda_mem_request: fraction of free device
 * memory the call may use for its work space. */
void multi_ref_align(const float **sbj_data, const float **ref_data, float *isac_peak_list, float *isac_d,
                     unsigned int isac_d_pitch, float cuda_mem_request);

/* Replaces gpu_clear, cuda/gpu_aln_noref.h:57 / cuda/gpu_aln_noref.cu:139-180:
 * ends the open sessions and frees the library's device and pinned memory,
 * including the work spaces of this library's additions (group assignment,
 * averaging step, host staging). */
void gpu_clear(void);

/* Replaces reset_shifts, cuda/gpu_aln_noref.cu:117-137: rebuilds the shift
 * grid with range (shift_range, shift_range) for the open multi-reference
 * and/or pre-alignment session; the number of shifts must not change. */
void reset_shifts(float shift_range, float shift_step);

/* Replaces print_gpu_info, cuda/gpu_aln_common.h:124 / gpu_aln_common.cu:180-218. */
void print_gpu_info(unsigned int device_idx);

/* Replaces get_texture_limit, cuda/gpu_aln_common.h:133 / gpu_aln_common.cu:233-237:
 * images of side img_dim that fit the height of one 2D linear texture. */
int get_texture_limit(unsigned int img_dim);

/* ---- pre-alignment: every particle against one reference (the running
 * global average), shifts accumulating in the returned AlignParam array;
 * same call sequence as bin/sp_isac_applications.py:1455-1660 ---- */

/* Replaces pre_align_init, cuda/gpu_aln_noref.h:77-81 (noref.cu:565-609):
 * opens a session with cfg->sbj_num subject slots (the GPU batch) and
 * returns host memory AlignParam[num_particles], all zero, ref_id 0, which
 * the caller reads after each run (freed by gpu_clear).  NULL on error. */
AlignParam *pre_align_init(unsigned int num_particles, const AlignConfig *aln_cfg, unsigned int cuda_device_id);
/* Replaces pre_align_size_check, cuda/gpu_aln_noref.h:83-89: whether a batch
 * of cfg->sbj_num subjects fits in request x the free device memory. */
bool pre_align_size_check(unsigned int num_particles, const AlignConfig *cfg, unsigned int cuda_device_id,
                          float request, bool verbose);
/* Replaces pre_align_fetch, cuda/gpu_aln_noref.h:91-95: "sbj_batch" copies
 * img_num <= cfg->sbj_num subject images into slots 0.. (later slots keep
 * what an earlier fetch put there), "ref_batch" the one reference. */
void pre_align_fetch(const float **img_data, unsigned int img_num, const char *batch_type);
/* Replaces pre_align_run, cuda/gpu_aln_noref.h:97 (noref.cu:742-769): aligns
 * the fetched subjects, slot i = particle start_idx + i, against the
 * reference over the current shift grid around each particle's accumulated
 * shift; updates AlignParam[start_idx .. stop_idx): shift += best shift,
 * clamped to +-(img_dim - ring_num - 2), angle, mirror. */
void pre_align_run(int start_idx, int stop_idx);

/* ---- the multigroup alignment of the stability test (aln_type
 * "multigroup_aln"), as bin/sp_isac_applications.py:4552-4650 drives it:
 * init with every particle's class (sorted runs 0 .. ref_num-1) and the
 * initial class averages; the caller may write AlignParam shift_x/y; each
 * ref_free_alignment_2D aligns every particle to its class average over the
 * shift grid around its accumulated shift (the pre-alignment's peak and update
 * rules), then replaces the averages by the averages of the particles
 * transformed by their new parameters; _filter_references low-passes the
 * averages (hyperbolic tangent); gpu_clear ends the session. ---- */

/* Replaces ref_free_alignment_2D_init, cuda/gpu_aln_noref.h:101-107. */
AlignParam *ref_free_alignment_2D_init(const AlignConfig *aln_cfg, const float **sbj_data_list,
                                       const float **ref_data_list, const int *sbj_cid_list,
                                       unsigned int cuda_device_id);
/* Replaces ref_free_alignment_2D_size_check, cuda/gpu_aln_noref.h:109-114. */
bool ref_free_alignment_2D_size_check(const AlignConfig *cfg, unsigned int cuda_device_id, float request,
                                      bool verbose);
/* Replaces ref_free_alignment_2D, cuda/gpu_aln_noref.h:116. */
void ref_free_alignment_2D(void);
/* Replaces ref_free_alignment_2D_filter_references, cuda/gpu_aln_noref.h:118. */
void ref_free_alignment_2D_filter_references(float cutoff_freq, float falloff);
/* No counterpart in the reference (its extract_gpu_averages,
 * cuda/gpu_aln_noref.cu:50-81, is compiled out).  Copies the current class
 * averages of the multigroup session, [ref_num][img_dim][img_dim], into the
 * host array out.  Returns 0 or an error code. */
int gpuisac_ref_free_averages(float *out);

/* Replaces the caller-side "normalize.mask" processing of every image before
 * each alignment call (bin/sp_isac2_gpu.py:925-931; the processor itself is
 * EMAN2's, not part of the reference tree): for each of the n_img device
 * images [img_dim][img_dim] in imgs, in place, the mean (and, unless
 * no_sigma, the population standard deviation) of the pixels where the
 * device mask [img_dim][img_dim] exceeds 0.5, then x <- (x - mean) / sigma
 * (x <- x - mean with no_sigma, or when the masked pixels have no spread).
 * References take no_sigma = 1, particles no_sigma = 0, as the caller does.
 * Asynchronous on stream.  Returns 0 or an error code. */
int gpuisac_normalize_mask(float *imgs, unsigned int n_img, unsigned int img_dim, const float *mask, int no_sigma,
                           void *stream);

/* Replaces the averaging step that follows the group assignment in every
 * ISAC main iteration (bin/sp_isac2_gpu.py:1153-1234, the peak conversion
 * before it at :1015-1022; the image operations are EMAN2's, not part of the
 * reference tree).  Device arrays:
 *   imgs [n_img][img_dim][img_dim] the particles as they were aligned;
 *   peaks [n_class][peak_pitch][4] the alignment's (angle, sx, sy, mirror) per
 *     (reference, particle), as gpuisac_multi_ref_align_device writes them
 *     (peak_pitch 0 = n_img; 16-byte aligned);
 *   belongsto [n_img] each particle's group (gpuisac_assign_groups_device).
 * Particle i of group r takes the caller's conversion of peaks[r][i]
 * (sx' = -sx cos a - sy sin a, sy' = sx sin a - sy cos a, as float); its image
 * rot_shift2D'd by (a, sx', sy', mirror) -- quadratic interpolation,
 * "background" mode, the x-mirror after -- is added to the group's sum.  Each
 * group's mean shift (sx' negated for mirrored particles, summed in FP64,
 * rounded to float, divided by the member count) re-centres its members:
 * params[i] = (a, sx' -/+ mean x, sy' - mean y, mirror), the values the caller
 * stores with set_params2D.  averages[r] = sum times float(1 / members),
 * filt_tanl(fl, ff) when fl > 0 (0 <= ff <= 0.5, fl <= 0.5 in cycles per
 * pixel), then fshift by minus the mean shift when center.  members [n_class]
 * and shifts [n_class][2] (the mean shifts) are optional outputs, as is params.
 * img_dim 2..256.  Blocks until done.  Returns 0; 2 for bad arguments, a
 * belongsto entry outside [0, n_class) or a group without members (the
 * caller's division by the member count fails there; its average is zero); 1
 * for a CUDA error. */
int gpuisac_class_averages(const float *imgs, unsigned int n_img, unsigned int img_dim, const float *peaks,
                           unsigned long long peak_pitch, const int *belongsto, unsigned int n_class, float fl,
                           float ff, int center, float *averages, float *params, int *members, float *shifts,
                           void *stream);

/* ---- additions of this library (no counterpart in the reference, which
 * prints and exits on any CUDA error, cuda/gpu_aln_common.cu:104-118) ---- */

/* Last error of the calling process: returns its code (0 = none) and copies
 * the message into buf (NUL-terminated, truncated to n bytes). */
int gpuisac_last_error(char *buf, size_t n);
/* Clears the recorded error. */
void gpuisac_clear_error(void);
/* Library version, e.g. "gpuisac-gb300 0.1.0". */
const char *gpuisac_version(void);

/* Device-resident form of multi_ref_align for callers that keep images in
 * GPU memory (all pointers are device pointers on the current device):
 * sbj [sbj_num][img_dim][img_dim], ref [ref_num][img_dim][img_dim],
 * base_shift [sbj_num][2] or NULL, d_out [ref_num][sbj_num],
 * peak_out [ref_num][sbj_num][4].  stream: a cudaStream_t or NULL.
 * Blocks until the results are written.  Returns 0 or an error code. */
int gpuisac_multi_ref_align_device(const AlignConfig *cfg, const float *sbj, const float *ref,
                                   const float *base_shift, float *d_out, float *peak_out, void *stream);

/* No counterpart in the reference (its contraction, cu_ccf_mult_mref at
 * cuda/gpu_aln_noref.cu:1483-1537, is FP32 on the CUDA cores).  Arithmetic of
 * the ring-summed contraction used by multi_ref_align and
 * gpuisac_multi_ref_align_device:
 *   GPUISAC_CONTRACTION_FP32    FP32 fused multiply-adds on the CUDA cores,
 *                               the drop-in default;
 *   GPUISAC_CONTRACTION_BF16X3  every FP32 operand split into a BF16 high part
 *                               and the BF16 rounding of the remainder, the
 *                               three products hi*hi + hi*lo + lo*hi
 *                               accumulated in FP32 on the tensor cores
 *                               (tcgen05), peak values within 1e-4 relative of
 *                               the FP32 form.
 * The environment variable GPUISAC_CONTRACTION=bf16x3 selects the second at
 * load time.  gpuisac_set_contraction returns the previous mode, or -1 for an
 * unknown one. */
/* No counterpart in the reference (whose CUDA errors exit the process).  For
 * failure-path tests only: while wait_iters > 0, the kernels that stage their
 * inputs with asynchronous bulk copies (the tensor-memory CCF kernels, both
 * kernels of the tensor-core contraction and the averaging step's sum kernel)
 * issue no copies and give up each bounded wait after wait_iters tries of at
 * most 20 us, so that the call comes back with error code 1 ("timed out") and
 * the context stays usable; 0 restores normal operation. */
void gpuisac_test_stall_ccf(unsigned int wait_iters);
/* No counterpart in the reference (whose cudaMalloc failures exit the
 * process): failure-path tests only -- the next n device allocations of the
 * alignment's work space fail as if the device were out of memory, so that
 * the call returns error code 5 (E_NOMEM, "injected") with nothing left
 * allocated half-way; 0 cancels what is pending. */
void gpuisac_test_fail_alloc(unsigned int n);

#define GPUISAC_CONTRACTION_FP32 0
#define GPUISAC_CONTRACTION_BF16X3 1
int gpuisac_set_contraction(int mode);
int gpuisac_get_contraction(void);
/* No counterpart in the reference.  The tensor-core contraction's tile plan
 * for a shape, for measurement: fields[0..9] = shift blocks, shifts per
 * block, Z row length, K groups of 8 rings, subject row groups, references
 * per tile, reference tiles, MMA N, operand stages, FFT groups (as many as
 * n_fields holds).  Returns 0, or 4 when the shape has no plan. */
int gpuisac_split_plan(unsigned int ring_num, unsigned int n_shift, unsigned int n_ref, unsigned int *fields,
                       unsigned int n_fields);

/* No counterpart in the reference.  gpuisac_multi_ref_align_device without
 * any device memory allocation, for callers that cannot call cudaMalloc:
 * their GPU memory belongs to another allocator, or they must not pay the
 * implicit synchronisation cudaMalloc / cudaFree can cause.  The work space is
 * one 32 MiB array built into the library, held on every GPU that loads it
 * until the process exits; a workload whose reference spectra plus one
 * particle's spectra (ref_num + n_shift) * ring_num * 1 KiB exceed it is
 * rejected with error 2.  The first call on a device looks up the array's
 * device address (once per device); make that first call before any stream
 * capture.  Every call shares the array, so calls that overlapped on the GPU
 * would race: the entry point serialises its callers and returns only after
 * its work on `stream` has finished.  Returns 0 or an error code. */
int gpuisac_multi_ref_align_device_noalloc(const AlignConfig *cfg, const float *sbj, const float *ref,
                                           const float *base_shift, float *d_out, float *peak_out,
                                           void *stream);

/* One independent alignment group of gpuisac_multi_ref_align_groups_device. */
typedef struct GpuisacGroup {
    unsigned int sbj_offset;       /* first particle of the group in the subject stack */
    unsigned int sbj_num;          /* its particles */
    unsigned int ref_offset;       /* first reference of the group in the reference stack */
    unsigned int ref_num;          /* its references */
    unsigned long long out_offset; /* element offset of its [ref_num][sbj_num] block in d_out
                                      (and of its [ref_num][sbj_num][4] block in peak_out) */
} GpuisacGroup;

/* No single counterpart in the reference, which aligns one group per
 * multi_ref_align_init / multi_ref_align / gpu_clear cycle
 * (bin/sp_isac2_gpu.py:937-1032).  Aligns n_groups independent groups --
 * each group's particles against its own references -- in one pass over
 * device stacks: cfg gives the shared geometry (img_dim, ring_num, ring_len,
 * shift grid) and, in sbj_num / ref_num, the stack sizes.  Each group's
 * results equal those of a separate alignment of that group.  The launches
 * (one texture fill, then a spectra and a CCF launch per wave of particles)
 * read their work from device tables; the sequence is recorded in a CUDA
 * graph once per number of waves and tile shape and replayed by every later
 * call of that shape, whatever its groups.  Blocks until done.
 * Returns 0 or an error code. */
int gpuisac_multi_ref_align_groups_device(const AlignConfig *cfg, const GpuisacGroup *groups,
                                          unsigned int n_groups, const float *sbj, const float *ref,
                                          const float *base_shift, float *d_out, float *peak_out,
                                          void *stream);

/* No counterpart in the reference (its only checks are cudaGetLastError
 * after each launch).  In a library built with -DGPUISAC_CHECKED
 * (gpu-isac_gb300/build.py --checked), every guarded global access of the spectra, contraction, FFT
 * and peak kernels tests its index against the extent the kernel was given
 * and skips (and records) an access outside it.  Returns the number of
 * accesses skipped since the last call (and clears the records), the first
 * one's (site << 48 | index) in *first; -1 in a normal build. */
int gpuisac_checked_failures(unsigned long long *first);

/* What the last gpuisac_multi_ref_align_groups_device call of the process
 * did: host milliseconds from entry to its tables and texture objects being
 * uploaded (plan_ms), milliseconds recording and instantiating a new launch
 * graph (record_ms; 0 when a recorded one was replayed), waves of particles,
 * kernel launches in the graph, and whether a graph was recorded. */
typedef struct GpuisacGroupStats {
    double plan_ms;
    double record_ms;
    unsigned int waves;
    unsigned int graph_launches;
    unsigned int graphs_recorded;
} GpuisacGroupStats;
int gpuisac_groups_stats(GpuisacGroupStats *out);

/* No counterpart in the reference.  The exhaustive shift x angle x mirror
 * search of selected particles against k references each: particle
 * part_idx[i] (i < n_sel; NULL selects particles 0..sbj_num-1 and n_sel must
 * be sbj_num) against references proposals[i*k .. i*k+k-1] (device arrays of
 * reference indices < ref_num).  Writes d_out[i*k + j] and
 * peak_out[(i*k + j)*4 ..]; each entry equals the one a full
 * gpuisac_multi_ref_align_device of the same stacks gives for that
 * (reference, particle).  Used with proposed reference lists, and with every
 * reference for particles that fall back to the full search.  Blocks until
 * done.  Returns 0 or an error code. */
int gpuisac_align_proposals_device(const AlignConfig *cfg, const float *sbj, const float *ref,
                                   const float *base_shift, const unsigned int *part_idx, unsigned int n_sel,
                                   const unsigned int *proposals, unsigned int k, float *d_out, float *peak_out,
                                   void *stream);

/* No counterpart in the reference.  A trained proposal network, as the
 * learned search reads it (device arrays, row-major FP32). */
typedef struct GpuisacProposalNet {
    unsigned int nk;     /* harmonics per ring: ring_num * nk network inputs */
    unsigned int hidden; /* hidden width */
    unsigned int emb;    /* embedding width */
    const float *mu;     /* [ring_num*nk] feature standardisation */
    const float *inv_sd; /* [ring_num*nk] */
    const float *W1;     /* [hidden][ring_num*nk] */
    const float *b1;     /* [hidden] */
    const float *W2;     /* [emb][hidden] */
    const float *b2;     /* [emb] */
} GpuisacProposalNet;

/* No counterpart in the reference.  Best reference and alignment of every
 * particle by the learned search: the particle's ring spectra at every shift
 * of cfg's grid feed the network, each reference is scored by the best
 * cosine similarity over shifts between the particle's embedding and
 * ref_emb[ref] ([ref_num][emb], unit rows), the top k references are searched
 * exhaustively (shift x angle x mirror, as the full search does), and a
 * particle whose best proposed peak beats the runner-up proposal by less
 * than gap_margin is searched against every reference.  Outputs per particle
 * p: best_ref[p], best_peak[p], best_param[p*4 ..] (angle, sx, sy, mirror,
 * as the full search reports them); optional best_gap[p] (best minus
 * runner-up proposed peak, +inf for k = 1) and fallback[p] (1 if searched
 * against every reference).  *pairs (optional, host) receives the number of
 * particle x reference alignments run.  A result equals the full search's
 * entry for the reference it names; ties go to the smaller reference index.
 * Blocks until done.  Returns 0 or an error code. */
int gpuisac_learned_align_device(const AlignConfig *cfg, const float *sbj, const float *ref, const float *base_shift,
                                 const GpuisacProposalNet *net, const float *ref_emb, unsigned int k,
                                 float gap_margin, int *best_ref, float *best_peak, float *best_param,
                                 float *best_gap, unsigned int *fallback, unsigned long long *pairs, void *stream);

/* No counterpart in the reference.  Autotuner of the CCF launch's tile shape
 * (kernel variant, contraction warps, particles per work item): times every
 * candidate on the first n_sample particles (0: 2048) of the device stacks
 * through gpuisac_multi_ref_align_device and keeps the fastest for cfg's ring
 * count and shift count for the rest of the process; every candidate gives
 * bit-identical results.  report (optional) receives one line: each
 * candidate's time and the choice.  Blocks until done.  Returns 0 or an error
 * code. */
int gpuisac_autotune_ccf(const AlignConfig *cfg, const float *sbj, const float *ref, unsigned int n_sample,
                         char *report, size_t report_len, void *stream);
/* No counterpart in the reference.  The tile shape the CCF launches of this
 * ring count and shift count use, as text ("ws8/ppc8"). */
int gpuisac_ccf_tile_name(unsigned int ring_num, unsigned int n_shift, char *buf, size_t len);

/* ---- learned reference proposal (no counterpart in the reference): kernels
 * of a small embedding network, all on caller-owned row-major FP32 device
 * arrays, asynchronous on `stream`; each returns 0, or 2 for bad arguments,
 * 1 for a launch error ---- */

/* feat[i][r*nk + k] = log(1 + |F_r[k]|), k < nk, rows scaled to unit L2 norm,
 * then standardised per column ((v - mu) * inv_sd) when mu and inv_sd are
 * given, from spectra rows [n][ring_num][128][2] made by
 * gpuisac_spectra_device (subject basis): rotation- and mirror-invariant
 * ring features. */
int gpuisac_nn_features(const float *spectra, unsigned int n, unsigned int ring_num, unsigned int nk,
                        const float *mu, const float *inv_sd, float *feat, void *stream);
/* per-column mean and 1/sqrt(variance + eps) of X [rows][cols]. */
int gpuisac_nn_col_stats(const float *X, long rows, int cols, float eps, float *mean, float *inv_sd, void *stream);
/* X[i][j] = (X[i][j] - mu[j]) * inv_sd[j]. */
int gpuisac_nn_affine_cols(float *X, long rows, int cols, const float *mu, const float *inv_sd, void *stream);
/* out[i][j] = max over s < group of G[i*group + s][j]. */
int gpuisac_nn_group_max(const float *G, long n, int group, int cols, float *out, void *stream);
/* C = alpha * op(A) op(B) + beta * C; A(m,k) at A[m*sam + k*sak], B(k,n) at
 * B[k*sbk + n*sbn], C row pitch ldc. */
int gpuisac_nn_gemm(int M, int N, int K, float alpha, const float *A, long sam, long sak, const float *B, long sbk,
                    long sbn, float beta, float *C, long ldc, void *stream);
/* C = alpha * A B^T (+ bias[n] when given, then ReLU if relu != 0) on the
 * tensor cores: A [M][K] (pitch lda) and B [N][K] (pitch ldb) FP32, rounded
 * to BF16 as they are staged, FP32 accumulation, C [M][N] FP32 (pitch ldc).
 * K, lda, ldb multiples of 4 and A, B 16-byte aligned (else 2); err: device
 * word set non-zero if a kernel gave up waiting for its own tensor-core work. */
int gpuisac_nn_gemm_bf16(int M, int N, int K, float alpha, const float *A, long lda, const float *B, long ldb,
                         const float *bias, int relu, float *C, long ldc, unsigned int *err, void *stream);
/* Y[i][j] += b[j], then ReLU if relu != 0. */
int gpuisac_nn_bias_act(float *Y, const float *b, long rows, int cols, int relu, void *stream);
/* dY[i] = 0 where Y[i] <= 0. */
int gpuisac_nn_relu_backward(float *dY, const float *Y, long n, void *stream);
/* db[j] = sum_i dY[i][j], added to db when accumulate != 0. */
int gpuisac_nn_colsum(const float *dY, long rows, int cols, float *db, int accumulate, void *stream);
/* E[i] = X[i] / |X[i]|, norm[i] = |X[i]|. */
int gpuisac_nn_l2norm(const float *X, long rows, int cols, float *E, float *norm, void *stream);
/* gradient of the row normalisation: dX = (dE - E (E . dE)) / norm. */
int gpuisac_nn_l2norm_backward(const float *E, const float *dE, const float *norm, long rows, int cols, float *dX,
                               void *stream);
/* loss[i] = -log softmax(S[i])[labels[i]]; if dS is given,
 * dS = (softmax - onehot) / rows (gradient of the mean loss). */
int gpuisac_nn_softmax_xent(const float *S, const int *labels, long rows, int cols, float *loss, float *dS,
                            void *stream);
/* AdamW step (bias-corrected, step >= 1) on n parameters. */
int gpuisac_nn_adam(float *p, const float *g, float *m, float *v, long n, float lr, float b1, float b2, float eps,
                    float wd, int step, void *stream);
/* idx[i][0..k-1] = columns of the k largest S[i][.], best first (cols <= 1024, k <= 64). */
int gpuisac_nn_topk(const float *S, long rows, int cols, int k, unsigned int *idx, void *stream);

/* Replaces EMAN2's Util::assign_groups (util_sparx.cpp, not vendored), which
 * bin/sp_isac2_gpu.py:1119 calls on the alignment's peak matrix right after
 * the alignment: the equal-size assignment of nima particles to nref groups
 * taking (reference, particle) pairs in descending peak order (equal peaks:
 * smaller index ref*nima + particle first), maxasi = nima / nref per group, the
 * group that closes last also taking the nima % nref particles left over.
 * d: device array d[ref * d_pitch + particle] (d_pitch 0 = nima; the layout
 * gpuisac_multi_ref_align_device writes), finite values; 1 <= nref <= nima,
 * nref * nima < 2^32.  Outputs (device, either may be NULL but not both):
 * belongsto[nima] = each particle's group; id_list_long[nima + 1] = the list
 * Util::assign_groups returns (each group's maxasi members in descending pair
 * order, group after group, the leftovers in descending order of their pair
 * with the last group, then that group's index).  rounds (host, optional)
 * receives the number of parallel proposal rounds.  Blocks until done.
 * Returns 0, 2 (bad arguments, a NaN peak) or 1 (CUDA error). */
int gpuisac_assign_groups_device(const float *d, unsigned long long d_pitch, unsigned int nref, unsigned int nima,
                                 int *belongsto, int *id_list_long, unsigned int *rounds, void *stream);
/* The same on host arrays, in Util::assign_groups' shape: d[nref * nima]
 * (host), id_list_long[nima + 1] (host) receives the list.  Copies d to the
 * current device and the list back.  Returns 0 or an error code. */
int gpuisac_assign_groups(const float *d, unsigned int nref, unsigned int nima, int *id_list_long);

/* Ring spectra of a device image stack at every shift of cfg's grid, as the
 * CCF kernel consumes them: out [n_img][n_shift][ring_num][128][2] (float),
 * slot 0 = (F[0], F[128]); is_ref selects the reference layout (ring weight
 * folded in, no shift).  base_shift may be NULL.  For tests and diagnostics. */
int gpuisac_spectra_device(const AlignConfig *cfg, const float *imgs, unsigned int n_img, int is_ref,
                           const float *base_shift, float *out, void *stream);

/* Same, with an explicit image grouping: images are read as the reference's
 * textures read them, in batches of `batch` images split into textures of
 * `tex` images.  For tests. */
int gpuisac_spectra_device_layout(const AlignConfig *cfg, const float *imgs, unsigned int n_img, int is_ref,
                                  const float *base_shift, unsigned int batch, unsigned int tex, float *out,
                                  void *stream);

/* The CCF / inverse FFT / peak-search stage alone, on spectra made by
 * gpuisac_spectra_device: sbj_spectra holds n_part particles (global indices
 * p_global0..), ref_spectra cfg->ref_num references; writes their columns of
 * d_out [ref_num][sbj_num] and peak_out [ref_num][sbj_num][4].  Asynchronous
 * on `stream`.  Returns 0 or an error code. */
int gpuisac_ccf_peak_device(const AlignConfig *cfg, const float *sbj_spectra, const float *ref_spectra,
                            const float *base_shift, unsigned int n_part, unsigned int p_global0, float *d_out,
                            float *peak_out, void *stream);

/* Number of shifts in cfg's grid (the reference's generate_shift_array). */
int gpuisac_shift_count(const AlignConfig *cfg);

/* Kernels this library has launched since it was loaded. */
unsigned long long gpuisac_launch_count(void);

/* Turns CUDA-event timing of each pipeline kernel on (1) or off (0) and
 * resets the totals. */
void gpuisac_profile(int on);

/* Launches and summed device time (ms) of one pipeline kernel
 * ("polar_spectra" or "ccf_peak") since gpuisac_profile(1). */
int gpuisac_kernel_time(const char *kernel, unsigned long long *launches, double *total_ms);

#ifdef __cplusplus
}
#endif
#endif
