/*
 * isac_oracle_core.h -- precision-generic body of the oracle; included by
 * isac_oracle.c once with REAL=double (orc_f64_*) and once with REAL=float
 * (orc_f32_*).  TEST INFRASTRUCTURE ONLY.
 */
#define ORC_CAT2(a, b, c) a##_##b##_##c
#define ORC_CAT(a, b, c) ORC_CAT2(a, b, c)
#define FN(name) ORC_CAT(orc, P, name)

/* iterative radix-2 complex FFT; sign -1 forward (cuFFT R2C/C2C forward),
 * +1 unnormalised inverse (cuFFT C2R); twiddles e^{-2 pi i k / n} in tw */
static void FN(fft)(REAL *re, REAL *im, unsigned n, int sign, const REAL *tw_re, const REAL *tw_im)
{
    for (unsigned i = 1, j = 0; i < n; i++) {
        unsigned bit = n >> 1;
        for (; j & bit; bit >>= 1)
            j ^= bit;
        j ^= bit;
        if (i < j) {
            REAL t = re[i]; re[i] = re[j]; re[j] = t;
            t = im[i]; im[i] = im[j]; im[j] = t;
        }
    }
    for (unsigned len = 2; len <= n; len <<= 1) {
        unsigned stride = n / len;
        for (unsigned i = 0; i < n; i += len) {
            for (unsigned k = 0; k < len / 2; k++) {
                REAL wr = tw_re[k * stride];
                REAL wi = sign < 0 ? tw_im[k * stride] : -tw_im[k * stride];
                REAL ur = re[i + k], ui = im[i + k];
                REAL xr = re[i + k + len / 2], xi = im[i + k + len / 2];
                REAL vr = xr * wr - xi * wi, vi = xr * wi + xi * wr;
                re[i + k] = ur + vr; im[i + k] = ui + vi;
                re[i + k + len / 2] = ur - vr; im[i + k + len / 2] = ui - vi;
            }
        }
    }
}

typedef struct {
    unsigned L;
    REAL *tw_re, *tw_im; /* L/2 entries */
    float *tmpl;         /* polar template */
    float *shifts;       /* n_shift (x, y) pairs */
    int n_shift;
} FN(ctx);

static void FN(ctx_free)(FN(ctx) *c)
{
    free(c->tw_re); free(c->tw_im); free(c->tmpl); free(c->shifts);
    memset(c, 0, sizeof(*c));
}

static int FN(ctx_init)(FN(ctx) *c, const orc_cfg *cfg)
{
    memset(c, 0, sizeof(*c));
    if (check_cfg(cfg))
        return -1;
    unsigned L = cfg->ring_len;
    c->L = L;
    c->tw_re = (REAL *)malloc(sizeof(REAL) * (L / 2));
    c->tw_im = (REAL *)malloc(sizeof(REAL) * (L / 2));
    c->tmpl = (float *)malloc(sizeof(float) * 2 * cfg->ring_num * L);
    int cap = 1 << 20;
    c->shifts = (float *)malloc(sizeof(float) * 2 * cap);
    if (!c->tw_re || !c->tw_im || !c->tmpl || !c->shifts) {
        FN(ctx_free)(c);
        return -1;
    }
    for (unsigned k = 0; k < L / 2; k++) {
        double a = -2.0 * M_PI * (double)k / (double)L;
        c->tw_re[k] = (REAL)cos(a);
        c->tw_im[k] = (REAL)sin(a);
    }
    orc_polar_template(cfg->ring_num, L, c->tmpl);
    c->n_shift = orc_shift_array(cfg->shift_rng_x, cfg->shift_rng_y, cfg->shift_step, c->shifts, cap);
    if (c->n_shift <= 0) {
        FN(ctx_free)(c);
        return -1;
    }
    return 0;
}

/* Reference: cu_resample_to_polar, cuda/gpu_aln_noref.cu:1221-1354 (sampling
 * :1258-1286, normalisation :1289-1352). */
static int FN(polar_ctx)(const FN(ctx) *c, const orc_cfg *cfg, const orc_layout *lay,
                         const float *stack, unsigned n_imgs, unsigned img, int is_ref,
                         float shift_x, float shift_y, const float *base, REAL *out)
{
    unsigned D = cfg->img_dim, L = c->L, NR = cfg->ring_num;
    orc_texture_stack ts;
    ts.stack = stack;
    ts.n_imgs = n_imgs;
    ts.dim = D;
    ts.batch = is_ref ? lay->ref_batch : lay->sbj_batch;
    ts.tex = lay->tex_limit;
    if (ts.batch == 0 || ts.tex == 0 || img >= n_imgs)
        return -1;
    if (is_ref && ts.batch > ts.tex)
        return -1; /* the reference asserts on this (noref.cu:1837-1840) */
    if (ts.batch > n_imgs)
        ts.batch = n_imgs;

    /* kernel parameters are int: the float grid shift is truncated */
    int sxi = (int)shift_x, syi = (int)shift_y;
    float cnt_x = centre_coord(D, sxi, base ? &base[0] : NULL);
    float cnt_y = centre_coord(D, syi, base ? &base[1] : NULL);
    unsigned li = tex_local_index(&ts, img);
    float yoff = (float)(li * D);

    for (unsigned r = 0; r < NR; r++) {
        for (unsigned j = 0; j < L; j++) {
            float ox = c->tmpl[(r * L + j) * 2 + 0];
            float oy = c->tmpl[(r * L + j) * 2 + 1];
            float x = cnt_x + ox;
            float y = (yoff + cnt_y) + oy;
            int ix, iy, w[4];
            orc_tex_weights(x, y, &ix, &iy, w);
            REAL t00 = texel(&ts, img, iy, ix), t10 = texel(&ts, img, iy, ix + 1);
            REAL t01 = texel(&ts, img, iy + 1, ix), t11 = texel(&ts, img, iy + 1, ix + 1);
            out[(size_t)r * L + j] = ((REAL)w[0] * t00 + (REAL)w[1] * t10 + (REAL)w[2] * t01 +
                                      (REAL)w[3] * t11) * (REAL)(1.0 / 256.0);
        }
    }

    /* ring sums, radius-weighted mean and deviation (same operation order) */
    REAL avg = 0, std = 0, nn = 0;
    for (unsigned r = 0; r < NR; r++) {
        REAL s = 0, q = 0;
        for (unsigned j = 0; j < L; j++) {
            REAL v = out[(size_t)r * L + j];
            s += v;
            q += v * v;
        }
        avg += s * (REAL)(r + 1);
        std += q * (REAL)(r + 1);
        nn += (REAL)(r + 1);
    }
    const REAL two_pi = (REAL)2 * (REAL)3.141592653589793f;
    nn *= two_pi;
    avg *= two_pi;
    std *= two_pi;
    avg /= (REAL)L;
    std /= (REAL)L;
    avg /= nn;
    std /= nn;
    std = (REAL)sqrt(fabs((double)(std - avg * avg)));
    for (size_t i = 0; i < (size_t)NR * L; i++)
        out[i] = (REAL)((out[i] - avg) / ((double)std + 0.0000001));
    return 0;
}

int FN(polar)(const orc_cfg *cfg, const orc_layout *lay, const float *stack, unsigned n_imgs,
              unsigned img, int is_ref, float shift_x, float shift_y, const float *base_shift,
              REAL *out)
{
    FN(ctx) c;
    if (FN(ctx_init)(&c, cfg))
        return -1;
    int rc = FN(polar_ctx)(&c, cfg, lay, stack, n_imgs, img, is_ref, shift_x, shift_y, base_shift, out);
    FN(ctx_free)(&c);
    return rc;
}

/* Reference: per-ring unnormalised R2C FFT, cuda/gpu_aln_noref.cu:2121-2125;
 * out [ring][k=0..L/2][re,im] */
static int FN(spectra_ctx)(const FN(ctx) *c, const orc_cfg *cfg, const orc_layout *lay,
                           const float *stack, unsigned n_imgs, unsigned img, int is_ref,
                           float shift_x, float shift_y, const float *base, REAL *out,
                           REAL *scratch /* NR*L + 2L */)
{
    unsigned L = c->L, NR = cfg->ring_num, K = L / 2 + 1;
    REAL *pol = scratch, *re = scratch + (size_t)NR * L, *im = re + L;
    if (FN(polar_ctx)(c, cfg, lay, stack, n_imgs, img, is_ref, shift_x, shift_y, base, pol))
        return -1;
    for (unsigned r = 0; r < NR; r++) {
        for (unsigned j = 0; j < L; j++) {
            re[j] = pol[(size_t)r * L + j];
            im[j] = 0;
        }
        FN(fft)(re, im, L, -1, c->tw_re, c->tw_im);
        for (unsigned k = 0; k < K; k++) {
            out[((size_t)r * K + k) * 2 + 0] = re[k];
            out[((size_t)r * K + k) * 2 + 1] = (k == 0 || k == L / 2) ? (REAL)0 : im[k];
        }
    }
    return 0;
}

int FN(spectra)(const orc_cfg *cfg, const orc_layout *lay, const float *stack, unsigned n_imgs,
                unsigned img, int is_ref, float shift_x, float shift_y, const float *base_shift,
                REAL *out)
{
    FN(ctx) c;
    if (FN(ctx_init)(&c, cfg))
        return -1;
    REAL *scratch = (REAL *)malloc(sizeof(REAL) * ((size_t)cfg->ring_num * c.L + 2 * c.L));
    int rc = scratch ? FN(spectra_ctx)(&c, cfg, lay, stack, n_imgs, img, is_ref, shift_x, shift_y,
                                       base_shift, out, scratch)
                     : -1;
    free(scratch);
    FN(ctx_free)(&c);
    return rc;
}

/* Reference: cu_ccf_mult_mref (cuda/gpu_aln_noref.cu:1512-1528) followed by
 * the table-wide C2R (:2453-2461).  O = sum_r (r+1) R conj(S) and
 * M = sum_r (r+1) conj(R S) are inverted together as one complex transform of
 * O + iM (both are Hermitian-extended spectra of real signals; the imaginary
 * parts of the DC and Nyquist bins are ignored as C2R does).
 * out_o / out_m: c[tau] for the normal and mirrored subject. */
static void FN(ccf_pair)(const FN(ctx) *c, unsigned NR, const REAL *refsp, const REAL *sbjsp,
                         REAL *out_o, REAL *out_m, REAL *re, REAL *im)
{
    unsigned L = c->L, K = L / 2 + 1;
    for (unsigned k = 0; k < K; k++) {
        REAL o_r = 0, o_i = 0, m_r = 0, m_i = 0;
        for (unsigned r = 0; r < NR; r++) {
            REAL rr = refsp[((size_t)r * K + k) * 2], ri = refsp[((size_t)r * K + k) * 2 + 1];
            REAL sr = sbjsp[((size_t)r * K + k) * 2], si = sbjsp[((size_t)r * K + k) * 2 + 1];
            REAL rr_sr = rr * sr, ri_si = ri * si, rr_si = rr * si, ri_sr = ri * sr;
            REAL w = (REAL)(r + 1);
            o_r += (rr_sr + ri_si) * w;
            o_i += (-rr_si + ri_sr) * w;
            m_r += (rr_sr - ri_si) * w;
            m_i += (-rr_si - ri_sr) * w;
        }
        if (k == 0 || k == L / 2) {
            re[k] = o_r;
            im[k] = m_r;
        } else {
            re[k] = o_r - m_i;
            im[k] = o_i + m_r;
            re[L - k] = o_r + m_i;
            im[L - k] = m_r - o_i;
        }
    }
    FN(fft)(re, im, L, +1, c->tw_re, c->tw_im);
    for (unsigned t = 0; t < L; t++) {
        out_o[t] = re[t];
        out_m[t] = im[t];
    }
}

int FN(pair_ccf)(const orc_cfg *cfg, const orc_layout *lay, const float *sbj, const float *ref,
                 unsigned p, unsigned q, const float *base_shifts, REAL *out)
{
    FN(ctx) c;
    if (FN(ctx_init)(&c, cfg))
        return -1;
    unsigned L = c.L, NR = cfg->ring_num, K = L / 2 + 1, S = (unsigned)c.n_shift;
    size_t sp = (size_t)NR * K * 2;
    REAL *refsp = (REAL *)malloc(sizeof(REAL) * sp);
    REAL *sbjsp = (REAL *)malloc(sizeof(REAL) * sp);
    REAL *scratch = (REAL *)malloc(sizeof(REAL) * ((size_t)NR * L + 2 * L));
    int rc = -1;
    if (!refsp || !sbjsp || !scratch)
        goto done;
    if (FN(spectra_ctx)(&c, cfg, lay, ref, cfg->ref_num, q, 1, 0.0f, 0.0f, NULL, refsp, scratch))
        goto done;
    for (unsigned s = 0; s < S; s++) {
        if (FN(spectra_ctx)(&c, cfg, lay, sbj, cfg->sbj_num, p, 0, c.shifts[2 * s], c.shifts[2 * s + 1],
                            base_shifts ? &base_shifts[2 * p] : NULL, sbjsp, scratch))
            goto done;
        REAL *re = scratch, *im = scratch + L;
        FN(ccf_pair)(&c, NR, refsp, sbjsp, out + (size_t)s * L, out + ((size_t)S + s) * L, re, im);
    }
    rc = 0;
done:
    free(refsp); free(sbjsp); free(scratch);
    FN(ctx_free)(&c);
    return rc;
}

/* Reference: multi_ref_align, cuda/gpu_aln_noref.cu:326-554.  Every particle
 * against every reference over the full grid; d[q*d_pitch + p] = raw peak,
 * peak_list[(q*P + p)*4 ..] = (angle, base_x + sx, base_y + sy, mirror). */
int FN(multi_ref_align)(const orc_cfg *cfg, const orc_layout *lay, const float *sbj,
                        const float *ref, const float *base_shifts, float *peak_list, REAL *d,
                        unsigned d_pitch, int n_threads)
{
    FN(ctx) c;
    if (FN(ctx_init)(&c, cfg))
        return -1;
    unsigned L = c.L, NR = cfg->ring_num, K = L / 2 + 1, S = (unsigned)c.n_shift;
    unsigned P = cfg->sbj_num, R = cfg->ref_num;
    size_t sp = (size_t)NR * K * 2;
    int rc = 0;
    REAL *refsp = (REAL *)malloc(sizeof(REAL) * sp * (R ? R : 1));
    if (!refsp) {
        FN(ctx_free)(&c);
        return -1;
    }
    {
        REAL *scratch = (REAL *)malloc(sizeof(REAL) * ((size_t)NR * L + 2 * L));
        for (unsigned q = 0; q < R && rc == 0; q++)
            if (!scratch || FN(spectra_ctx)(&c, cfg, lay, ref, R, q, 1, 0.0f, 0.0f, NULL, refsp + sp * q, scratch))
                rc = -1;
        free(scratch);
    }
#ifdef _OPENMP
    if (n_threads > 0)
        omp_set_num_threads(n_threads);
#else
    (void)n_threads;
#endif
    if (rc == 0) {
#pragma omp parallel
        {
            REAL *sbjsp = (REAL *)malloc(sizeof(REAL) * sp * S);
            REAL *scratch = (REAL *)malloc(sizeof(REAL) * ((size_t)NR * L + 2 * L));
            REAL *ccf = (REAL *)malloc(sizeof(REAL) * 2 * (size_t)S * L);
            int ok = sbjsp && scratch && ccf;
            if (!ok) {
#pragma omp atomic write
                rc = -1;
            }
#pragma omp for schedule(dynamic, 1)
            for (long pl = 0; pl < (long)P; pl++) {
                unsigned p = (unsigned)pl;
                if (!ok)
                    continue;
                const float *base = base_shifts ? &base_shifts[2 * p] : NULL;
                int bad = 0;
                for (unsigned s = 0; s < S && !bad; s++)
                    bad = FN(spectra_ctx)(&c, cfg, lay, sbj, P, p, 0, c.shifts[2 * s], c.shifts[2 * s + 1],
                                          base, sbjsp + sp * s, scratch);
                if (bad) {
#pragma omp atomic write
                    rc = -1;
                    continue;
                }
                for (unsigned q = 0; q < R; q++) {
                    for (unsigned s = 0; s < S; s++)
                        FN(ccf_pair)(&c, NR, refsp + sp * q, sbjsp + sp * s, ccf + (size_t)s * L,
                                     ccf + ((size_t)S + s) * L, scratch, scratch + L);
                    float out4[4];
                    REAL peak;
#if defined(ORC_IS_F32)
                    orc_f32_peak_search(ccf, S, L, out4, &peak);
#else
                    {
                        double pk;
                        if (sizeof(REAL) == sizeof(double)) {
                            orc_f64_peak_search((const double *)(const void *)ccf, S, L, out4, &pk, NULL);
                            peak = (REAL)pk;
                        } else {
                            orc_f32_peak_search((const float *)(const void *)ccf, S, L, out4, (float *)(void *)&peak);
                        }
                    }
#endif
                    unsigned sidx = (unsigned)out4[1];
                    float bx = base ? base[0] : 0.0f, by = base ? base[1] : 0.0f;
                    float *pl4 = peak_list + ((size_t)q * P + p) * 4;
                    pl4[0] = out4[0];
                    pl4[1] = bx + c.shifts[2 * sidx];
                    pl4[2] = by + c.shifts[2 * sidx + 1];
                    pl4[3] = out4[3];
                    d[(size_t)q * d_pitch + p] = peak;
                }
            }
            free(sbjsp); free(scratch); free(ccf);
        }
    }
    free(refsp);
    FN(ctx_free)(&c);
    return rc;
}

#undef FN
#undef ORC_CAT
#undef ORC_CAT2
