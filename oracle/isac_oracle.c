/*
 * isac_oracle.c -- CPU restatement of GPU-ISAC's multi-reference alignment.
 * TEST INFRASTRUCTURE ONLY (see isac_oracle.h).  Built with -ffp-contract=off
 * so that x86-64 and aarch64 hosts round identically.
 */
#include "isac_oracle.h"

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Reference: generate_polar_sampling_points, cuda/gpu_aln_common.cu:39-62.
 * The angle is formed in double from a float quotient and then stored as
 * float; the offsets are float products (host libm cosf/sinf). */
void orc_polar_template(unsigned ring_num, unsigned ring_len, float *out)
{
    for (unsigned i = 0; i < ring_num; i++) {
        for (unsigned j = 0; j < ring_len; j++) {
            unsigned idx = i * ring_len + j;
            float angle = (float)((double)((float)j / (float)ring_len) * 3.14159265358979 * 2);
            float cx = cosf(angle) * (float)(i + 1);
            float sy = sinf(angle) * (float)(i + 1);
            out[idx * 2 + 0] = cx * (float)ring_num / (float)ring_num;
            out[idx * 2 + 1] = sy * (float)ring_num / (float)ring_num;
        }
    }
}

/* Reference: generate_shift_array, cuda/gpu_aln_common.cu:64-86 (float
 * accumulation, x outer, y inner). */
int orc_shift_array(float rng_x, float rng_y, float step, float *out_xy, int cap)
{
    int n = 0;
    if (!(step > 0.0f))
        return -1;
    for (float sx = -rng_x; sx <= rng_x; sx += step) {
        for (float sy = -rng_y; sy <= rng_y; sy += step) {
            if (n >= cap)
                return -1;
            out_xy[2 * n + 0] = sx;
            out_xy[2 * n + 1] = sy;
            n++;
        }
    }
    return n;
}

/* Texture unit, linear filter, unnormalised coordinates
 * (cuda/gpu_aln_noref.cu:2333-2336): the texel-space coordinate t is moved by
 * -0.5 and converted to fixed point with 8 fractional bits, rounding to
 * nearest with ties upward; the integer part selects the left texel, the
 * fraction is the weight of the right one.  The rounding rule is pinned
 * against the texture unit by tests/test_gpu_texture.py. */
void orc_tex_split(float t, int *i, float *a)
{
    float tb = t - 0.5f;
    double q = floor((double)tb * 256.0 + 0.5);
    double fi = floor(q / 256.0);
    *i = (int)fi;
    *a = (float)((q - fi * 256.0) / 256.0);
}

/* Texture unit bilinear weights of one sample point, in units of 1/256:
 * the two 8-bit fractions A (x) and B (y) give w11 = round(A*B/256) (ties
 * upward) and the other three taps take what is left of each fraction, so
 * the four weights always sum to 256.  Pinned against the hardware by
 * tests/test_gpu_texture.py. */
void orc_tex_weights(float x, float y, int *ix, int *iy, int w[4])
{
    float ax, ay;
    orc_tex_split(x, ix, &ax);
    orc_tex_split(y, iy, &ay);
    int A = (int)(ax * 256.0f), B = (int)(ay * 256.0f);
    int w11 = (A * B + 128) >> 8;
    w[0] = 256 - A - B + w11; /* (ix,   iy)   */
    w[1] = A - w11;           /* (ix+1, iy)   */
    w[2] = B - w11;           /* (ix,   iy+1) */
    w[3] = w11;               /* (ix+1, iy+1) */
}

/* Reference: multi_ref_align batch sizing, cuda/gpu_aln_noref.cu:429-440 with
 * the cuFFT int32 guard of multi_ref_align_size_check (:238). */
unsigned orc_reference_sbj_batch(const orc_cfg *cfg)
{
    unsigned ref_b = cfg->ref_num < 100 ? cfg->ref_num : 100;
    size_t shift_num = (size_t)((2 * (cfg->shift_rng_x / cfg->shift_step) + 1) *
                                (2 * (cfg->shift_rng_y / cfg->shift_step) + 1));
    unsigned bs = 0;
    if (cfg->sbj_num == 0)
        return 0;
    for (int i = (int)log2((double)cfg->sbj_num); i >= 0; i--) {
        unsigned split = (unsigned)pow(2.0, i);
        unsigned cand = bs + split < cfg->sbj_num ? bs + split : cfg->sbj_num;
        size_t entries = (size_t)cand * (size_t)ref_b * (shift_num * 2) * (size_t)(cfg->ring_len + 2);
        if (entries <= (((size_t)1) << 31) - 1)
            bs = cand;
    }
    return bs;
}

/* One texel of the stacked image textures.  Images are fetched batch by batch
 * into textures sized for the first batch (noref.cu:1831-1854, 2001-2052):
 * rows past an image read the next image of the same texture, the ends of a
 * texture clamp, and slots a short final batch does not overwrite still hold
 * the previous batch's image. */
typedef struct {
    const float *stack;
    unsigned n_imgs;   /* images in the whole stack */
    unsigned dim;
    unsigned batch;    /* images per batch */
    unsigned tex;      /* images per texture */
} orc_texture_stack;

static float texel(const orc_texture_stack *ts, unsigned img, long row, long col)
{
    unsigned D = ts->dim;
    unsigned bstart = (img / ts->batch) * ts->batch;
    unsigned blen = ts->n_imgs - bstart < ts->batch ? ts->n_imgs - bstart : ts->batch;
    unsigned local = img - bstart;
    unsigned tex_idx = local / ts->tex;
    unsigned n_tex_alloc = (ts->batch + ts->tex - 1) / ts->tex;
    unsigned alloc_imgs = (tex_idx != n_tex_alloc - 1) ? ts->tex : ts->batch - tex_idx * ts->tex;
    long H = (long)alloc_imgs * D;
    if (row < 0) row = 0;
    if (row > H - 1) row = H - 1;
    if (col < 0) col = 0;
    if (col > (long)D - 1) col = (long)D - 1;
    unsigned slot = (unsigned)(row / D);
    unsigned yy = (unsigned)(row % D);
    unsigned g = bstart + tex_idx * ts->tex + slot;
    if (g >= bstart + blen)
        g -= ts->batch; /* stale slot from the previous batch */
    return ts->stack[(size_t)g * D * D + (size_t)yy * D + (size_t)col];
}

/* position of an image inside its texture (the kernel's block index) */
static unsigned tex_local_index(const orc_texture_stack *ts, unsigned img)
{
    unsigned local = img % ts->batch;
    return local % ts->tex;
}

/* Reference: centre of the polar grid, cuda/gpu_aln_noref.cu:1262-1269.
 * D/2 + shift is unsigned arithmetic, the base shift a float add, +0.5 a
 * double add, the result a float. */
static float centre_coord(unsigned dim, int shift_int, const float *base)
{
    unsigned u = dim / 2u + (unsigned)shift_int;
    if (base) {
        float f = (float)u + *base;
        return (float)((double)f + 0.5);
    }
    return (float)((double)u + 0.5);
}

static int is_pow2(unsigned n) { return n >= 2 && (n & (n - 1)) == 0; }

static int check_cfg(const orc_cfg *cfg)
{
    if (!cfg || cfg->img_dim == 0 || cfg->ring_num == 0 || !is_pow2(cfg->ring_len))
        return -1;
    if (cfg->ring_num > cfg->ring_len)
        return -1;
    return 0;
}

/* Reference: cu_aln_param_wizard, cuda/gpu_aln_noref.cu:1716-1793.  Scan order
 * h = mirror*S + shift, tau = 0..L-1; first strict maximum starting from
 * -3.40282e38; 7-point parabola over (tau+i) mod L with the reference's
 * unsigned wrap; angle = 360 - a (+180 when mirrored), folded below 360. */
void orc_f64_peak_search(const double *ccf, unsigned n_shift, unsigned L,
                         float *out4, double *peak, unsigned *tau_out)
{
    double best = (double)(float)-3.40282e+038;
    unsigned best_h = 0, best_t = 0;
    for (unsigned h = 0; h < 2 * n_shift; h++) {
        const double *row = ccf + (size_t)h * L;
        for (unsigned t = 0; t < L; t++) {
            if (row[t] > best) {
                best = row[t];
                best_h = h;
                best_t = t;
            }
        }
    }
    unsigned mirror = best_h >= n_shift;
    unsigned sidx = mirror ? best_h - n_shift : best_h;
    const double *row = ccf + (size_t)best_h * L;
    double x[7];
    for (int i = -3; i <= 3; i++)
        x[i + 3] = row[(unsigned)(best_t + (unsigned)i) % L];
    double c2 = 49. * x[0] + 6. * x[1] - 21. * x[2] - 32. * x[3] - 27. * x[4] - 6. * x[5] + 31. * x[6];
    double c3 = 5. * x[0] - 3. * x[2] - 4. * x[3] - 3. * x[4] + 5. * x[6];
    double step = 360.0 / (double)L;
    double angle = step * (double)best_t;
    if (c3 != 0.0)
        angle = angle + step * (c2 / (2.0 * c3) - 4);
    angle = 360.0 - angle;
    if (mirror)
        angle += 180.0;
    if (angle >= 360.0)
        angle -= 360.0;
    out4[0] = (float)angle;
    out4[1] = (float)sidx;
    out4[2] = 0.0f;
    out4[3] = mirror ? 1.0f : 0.0f;
    if (peak) *peak = best;
    if (tau_out) *tau_out = best_t;
}

/* Same search with the reference's own float/double mixing (noref.cu:1777-1793),
 * for the FP32 pipeline. */
static void orc_f32_peak_search(const float *ccf, unsigned n_shift, unsigned L,
                                float *out4, float *peak)
{
    float best = -3.40282e+038f;
    unsigned best_h = 0, best_t = 0;
    for (unsigned h = 0; h < 2 * n_shift; h++) {
        const float *row = ccf + (size_t)h * L;
        for (unsigned t = 0; t < L; t++) {
            if (row[t] > best) {
                best = row[t];
                best_h = h;
                best_t = t;
            }
        }
    }
    unsigned mirror = best_h >= n_shift;
    unsigned sidx = mirror ? best_h - n_shift : best_h;
    const float *row = ccf + (size_t)best_h * L;
    float x[7];
    for (int i = -3; i <= 3; i++)
        x[i + 3] = row[(unsigned)(best_t + (unsigned)i) % L];
    float c2 = (float)(49. * x[0] + 6. * x[1] - 21. * x[2] - 32. * x[3] - 27. * x[4] - 6. * x[5] + 31. * x[6]);
    float c3 = (float)(5. * x[0] - 3. * x[2] - 4. * x[3] - 3. * x[4] + 5. * x[6]);
    float step = (float)(360.0 / (double)(float)L);
    float angle = step * (float)best_t;
    if (c3 != 0.0)
        angle = (float)((double)angle + (double)step * ((double)c2 / (2.0 * (double)c3) - 4));
    angle = (float)(360.0 - (double)angle);
    if (mirror)
        angle = (float)((double)angle + 180.0);
    if (angle >= 360.0)
        angle = (float)((double)angle - 360.0);
    out4[0] = angle;
    out4[1] = (float)sidx;
    out4[2] = 0.0f;
    out4[3] = mirror ? 1.0f : 0.0f;
    *peak = best;
}

/* ---- precision-generic part ---- */
#define P f64
#define REAL double
#include "isac_oracle_core.h"
#undef P
#undef REAL

#define P f32
#define REAL float
#include "isac_oracle_core.h"
#undef P
#undef REAL

/* Reference: cu_transform_batch (cuda/gpu_aln_noref.cu:1539-1590) followed by
 * cu_average_batch (:1592-1622), as ref_free_alignment_2D runs them
 * (:964-996): every particle of the stack (one batch of n images in textures
 * of tex images) is resampled through the texture at
 *   x' = (mirror ? D - x : x) - D/2,  y' = y - D/2,
 *   (xr, yr) = (x' cos a - y' sin a, x' sin a + y' cos a) + D/2,
 *   sample at (xr + shift_x + 0.5, slot*D + yr + shift_y + 0.5)
 * (each step rounded to float, the +0.5 added in double; a = DEG2RAD * angle
 * in float, its cosine and sine computed in double and rounded to float), and
 * class k's average is the float sum of its members' pixels in member order
 * divided by the member count.  params[i] = (angle, shift_x, shift_y) and
 * mirror[i]; cid_idx[n_class + 1] holds the class ranges.  Coordinates beyond
 * +-1e6 are clamped (they read the clamped edge either way). */
int orc_multigroup_averages(const float *stack, unsigned n, unsigned dim, unsigned tex, const float *params,
                            const int *mirror, const unsigned *cid_idx, unsigned n_class, float *avg_out)
{
    if (!stack || !params || !mirror || !cid_idx || !avg_out || n == 0 || dim == 0 || tex == 0)
        return -1;
    orc_texture_stack ts;
    ts.stack = stack;
    ts.n_imgs = n;
    ts.dim = dim;
    ts.batch = n;
    ts.tex = tex;
    const float ctr = (float)(dim / 2u);
    const float deg2rad = 3.141592653589793f / 180.0f;
    for (unsigned k = 0; k < n_class; k++) {
        const unsigned i0 = cid_idx[k], i1 = cid_idx[k + 1];
        if (i1 <= i0 || i1 > n)
            return -1;
        for (unsigned y = 0; y < dim; y++)
            for (unsigned x = 0; x < dim; x++) {
                float sum = 0.0f;
                for (unsigned i = i0; i < i1; i++) {
                    const float rad = deg2rad * params[3 * i + 0];
                    const float c = (float)cos((double)rad), s = (float)sin((double)rad);
                    const float sxp = mirror[i] ? (float)(dim - x) : (float)x;
                    const float x0 = sxp - ctr, y0 = (float)y - ctr;
                    const float p0 = x0 * c, p1 = y0 * s, p2 = x0 * s, p3 = y0 * c;
                    float xr = p0 - p1, yr = p2 + p3;
                    xr = xr + ctr;
                    yr = yr + ctr;
                    float xs = (float)((double)(xr + params[3 * i + 1]) + 0.5);
                    float ys = (float)((double)(yr + params[3 * i + 2]) + 0.5);
                    xs = xs < -1.0e6f ? -1.0e6f : (xs > 1.0e6f ? 1.0e6f : xs);
                    ys = ys < -1.0e6f ? -1.0e6f : (ys > 1.0e6f ? 1.0e6f : ys);
                    const float yt = (float)(tex_local_index(&ts, i) * dim) + ys;
                    int ix, iy, w[4];
                    orc_tex_weights(xs, yt, &ix, &iy, w);
                    const float t00 = texel(&ts, i, iy, ix), t10 = texel(&ts, i, iy, ix + 1);
                    const float t01 = texel(&ts, i, iy + 1, ix), t11 = texel(&ts, i, iy + 1, ix + 1);
                    const float v = ((float)w[0] * t00 + (float)w[1] * t10 + (float)w[2] * t01 +
                                     (float)w[3] * t11) * (1.0f / 256.0f);
                    sum = sum + v;
                }
                avg_out[((size_t)k * dim + y) * dim + x] = sum / (float)(i1 - i0);
            }
    }
    return 0;
}
