/*
 * FP64 CPU oracle for the generalized Lomb-Scargle (GLS) path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker that the CUDA path is
 * compared against; the product library never links, loads or calls it.  Only
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference arm
 * use it.
 *
 * What it restates (paths relative to the cuvarbase source tree):
 *   - oracle_gls_flmean: cuvarbase/lombscargle.py:337-400 (mhdirect_sums, H=1),
 *     :403-447 (add_regularization), :497-536 (mhgls_from_sums) and
 *     :539-576 (lomb_scargle_direct_sums).  Phase = 2*pi*((t*f) mod 1) in FP64
 *     exactly as lombscargle.py:370 does.
 *   - oracle_gls_flmean_blocks: the same sums on blocks of contiguous bins,
 *     exp(2 pi i f t) advanced by exp(2 pi i df t) between bins and re-seeded
 *     every 64 bins (for N ~ 1e6 curves); terms of eight points are summed
 *     pairwise before they are accumulated.
 *   - oracle_gls_tau: the closed-form "tau" evaluations of
 *     cuvarbase/kernels/lomb.cu:36-83 (lspow_flmean), :85-123 (lspow0) and the
 *     mode switch :126-141 (mode 0 standard, 1 floating mean, 2 window), with
 *     the direct sums of lomb.cu:144-165 (lomb_dirsum), all in FP64.
 *   - oracle_nfft_direct: cuvarbase/tests/test_nfft.py:31-34 (direct_sums),
 *     out[k] = sum_j y_j exp(+2 pi i f_k t_j).
 *   - oracle_grid_ref: cuvarbase/kernels/cunfft.cu:84-163 (precompute_psi +
 *     fast_gaussian_grid) as restated by cuvarbase/tests/test_nfft.py:57-87
 *     (precomp_psi, gpu_grid_scalar), in FP64.
 *
 * Build: oracle/Makefile (gcc -O2 -fopenmp -shared).  Portable C99, no
 * architecture-specific code, so it gives the same answers on x86_64 and
 * aarch64 hosts.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORACLE_PI 3.14159265358979323846264338327950288

int oracle_version(void) { return 1; }

int oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* Python's floored modulo, (a % 1.0), as used at lombscargle.py:370. */
static inline double pymod1(double a) { return a - floor(a); }

/* Sums of one frequency: W=sum w, C,S,C2,S2 (w-weighted), yc,ys (yw-weighted). */
typedef struct { double W, C, S, C2, S2, yc, ys; } sums_t;

static void direct_sums_one(const double *t, const double *yw, const double *w,
                            int64_t n, double f, sums_t *o) {
    double W = 0, C = 0, S = 0, C2 = 0, S2 = 0, yc = 0, ys = 0;
    for (int64_t j = 0; j < n; ++j) {
        double ph = 2.0 * ORACLE_PI * pymod1(t[j] * f);
        double c = cos(ph), s = sin(ph);
        double c2 = cos(2.0 * ph), s2 = sin(2.0 * ph);
        W += w[j];
        C += w[j] * c;  S += w[j] * s;
        C2 += w[j] * c2; S2 += w[j] * s2;
        yc += yw[j] * c; ys += yw[j] * s;
    }
    o->W = W; o->C = C; o->S = S; o->C2 = C2; o->S2 = S2; o->yc = yc; o->ys = ys;
}

/*
 * Floating-mean GLS power, H=1, restating mhdirect_sums -> add_regularization
 * -> mhgls_from_sums.  amp_prior <= 0 means no prior; otherwise the diagonal
 * regulariser is D = amp_prior**-2 (lombscargle.py:436-443).
 * Writes NAN where the 2x2 system is singular (np.linalg.solve would raise).
 */
int oracle_gls_flmean(const double *t, const double *yw, const double *w,
                      int64_t n, const double *freqs, int64_t nfreq,
                      double YY, double amp_prior, double *P, int nthreads) {
    /* ybar = sum(yw) (lombscargle.py:384): Python's builtin sum over the
       float32 yw array accumulates sequentially in float32. */
    float ybar32 = 0.0f;
    for (int64_t j = 0; j < n; ++j) ybar32 += (float)yw[j];
    const double ybar = (double)ybar32;
    const double D = amp_prior > 0 ? 1.0 / (amp_prior * amp_prior) : 0.0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 64)
#endif
    for (int64_t i = 0; i < nfreq; ++i) {
        sums_t s;
        direct_sums_one(t, yw, w, n, freqs[i], &s);
        double C = s.C, S = s.S;
        double YC = s.yc - ybar * C, YS = s.ys - ybar * S;
        double CC = 0.5 * (s.C2 + s.W) - C * C + D;          /* cc[1][1] - C*C */
        double SS = 0.5 * (s.W - s.C2) - S * S + D;          /* ss[1][1] - S*S */
        double CS = 0.5 * s.S2 - C * S;  /* cs[1][1]: s[0] = sum w sin(0) = 0 */
        double det = CC * SS - CS * CS;
        if (det == 0.0) { P[i] = NAN; continue; }
        double cn = (SS * YC - CS * YS) / det;
        double sn = (CC * YS - CS * YC) / det;
        double XX = cn * cn * CC + 2.0 * cn * sn * CS + sn * sn * SS;
        double YX = 2.0 * (cn * YC + sn * YS);
        P[i] = (YX - XX) / YY;
    }
    return 0;
}

/*
 * The same floating-mean GLS power on blocks of contiguous bins,
 * f = f_start[b] + k df (k < block_len), for curves too long for one
 * sin/cos per (point, bin): exp(2 pi i f t) advances by exp(2 pi i df t) from
 * bin to bin (FP64 complex products) and is re-seeded directly, with the
 * phase reduced as (t f) mod 1 like lombscargle.py:370, every 64 bins.  Sums
 * and the 2x2 solve are those of oracle_gls_flmean.  P has nblocks*block_len
 * entries, block-major.
 */
#define ORACLE_SEED 64
int oracle_gls_flmean_blocks(const double *t, const double *yw, const double *w,
                             int64_t n, const double *f_start, int64_t nblocks,
                             double df, int64_t block_len, double YY, double *P,
                             int nthreads) {
    float ybar32 = 0.0f;
    for (int64_t j = 0; j < n; ++j) ybar32 += (float)yw[j];
    const double ybar = (double)ybar32;
    double W = 0.0;
    for (int64_t j = 0; j < n; ++j) W += w[j];
    int rc = 0;
    /* the per-bin step exp(2 pi i df t_j) of every point, once */
    double *stp = (double *)malloc((size_t)(2 * (n > 0 ? n : 1)) * sizeof(double));
    if (!stp) return -1;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(static)
#endif
    for (int64_t j = 0; j < n; ++j) {
        const double pd = 2.0 * ORACLE_PI * pymod1(t[j] * df);
        stp[2 * j] = cos(pd);
        stp[2 * j + 1] = sin(pd);
    }
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1)
#endif
    for (int64_t bi = 0; bi < nblocks * ((block_len + ORACLE_SEED - 1) / ORACLE_SEED); ++bi) {
        const int64_t nseg = (block_len + ORACLE_SEED - 1) / ORACLE_SEED;
        const int64_t b = bi / nseg, k0 = (bi % nseg) * ORACLE_SEED;
        const int64_t len = (block_len - k0 < ORACLE_SEED) ? block_len - k0 : ORACLE_SEED;
        double acc[6][ORACLE_SEED];  /* C, S, C2, S2, yc, ys */
        for (int a = 0; a < 6; ++a)
            for (int k = 0; k < ORACLE_SEED; ++k) acc[a][k] = 0.0;
        const double f0 = f_start[b] + (double)k0 * df;
        /* eight points advance in lock-step (independent recurrences); their
           terms are summed pairwise before they reach the bin accumulators */
        for (int64_t j = 0; j < n; j += 8) {
            double zr[8], zi[8], sr[8], si[8], wj[8], yj[8];
            for (int q = 0; q < 8; ++q) {
                const int64_t jj = j + q;
                if (jj < n) {
                    const double ph = 2.0 * ORACLE_PI * pymod1(t[jj] * f0);
                    zr[q] = cos(ph); zi[q] = sin(ph);
                    sr[q] = stp[2 * jj]; si[q] = stp[2 * jj + 1];
                    wj[q] = w[jj]; yj[q] = yw[jj];
                } else {
                    zr[q] = 1.0; zi[q] = 0.0; sr[q] = 1.0; si[q] = 0.0;
                    wj[q] = 0.0; yj[q] = 0.0;
                }
            }
            for (int64_t k = 0; k < len; ++k) {
                double v[6][8];
                for (int q = 0; q < 8; ++q) {
                    const double c = zr[q], s = zi[q];
                    v[0][q] = wj[q] * c;
                    v[1][q] = wj[q] * s;
                    v[2][q] = wj[q] * (c * c - s * s);
                    v[3][q] = wj[q] * (2.0 * c * s);
                    v[4][q] = yj[q] * c;
                    v[5][q] = yj[q] * s;
                    zr[q] = c * sr[q] - s * si[q];
                    zi[q] = c * si[q] + s * sr[q];
                }
                for (int a = 0; a < 6; ++a)
                    acc[a][k] += ((v[a][0] + v[a][1]) + (v[a][2] + v[a][3])) +
                                 ((v[a][4] + v[a][5]) + (v[a][6] + v[a][7]));
            }
        }
        for (int64_t k = 0; k < len; ++k) {
            const double C = acc[0][k], S = acc[1][k];
            const double YC = acc[4][k] - ybar * C, YS = acc[5][k] - ybar * S;
            const double CC = 0.5 * (acc[2][k] + W) - C * C;
            const double SS = 0.5 * (W - acc[2][k]) - S * S;
            const double CS = 0.5 * acc[3][k] - C * S;
            const double det = CC * SS - CS * CS;
            double val = NAN;
            if (det != 0.0) {
                const double cn = (SS * YC - CS * YS) / det;
                const double sn = (CC * YS - CS * YC) / det;
                const double XX = cn * cn * CC + 2.0 * cn * sn * CS + sn * sn * SS;
                const double YX = 2.0 * (cn * YC + sn * YS);
                val = (YX - XX) / YY;
            }
            P[b * block_len + k0 + k] = val;
        }
    }
    free(stp);
    return rc;
}

/* lomb.cu:36-83, FP64. reg may be NULL. */
static double lspow_flmean64(double C, double S, double C2, double S2,
                             double YCh, double YSh, double YY, double Y,
                             const double *reg) {
    double r0 = 0, r1 = 0, r2 = 0;
    if (reg) { r0 = reg[0]; r1 = reg[1]; r2 = reg[2]; }
    double tan2wt = (S2 - 2 * S * C) / (C2 - (C * C - S * S));
    double C2wInv2 = 1.0 + tan2wt * tan2wt;
    double C2w = 1.0 / sqrt(C2wInv2);
    double S2w = tan2wt * C2w;
    double Cw = sqrt(0.5 * (1.0 + C2w));
    double Sw = sqrt(0.5 * (1.0 - C2w));
    if (S2w < 0.0) Sw = -Sw;
    double Cshft = C * Cw + S * Sw;
    double Sshft = S * Cw - C * Sw;
    double CC = 0.5 * (1.0 + C2 * C2w + S2 * S2w);
    double SS = 0.5 * (1.0 - C2 * C2w - S2 * S2w);
    CC -= Cshft * Cshft;
    SS -= Sshft * Sshft;
    double xreg = r2 / (1.0 + r2);
    CC += Cshft * Cshft * xreg + r0;
    SS += Sshft * Sshft * xreg + r1;
    double YC = (YCh + Y * C * xreg) * Cw + (YSh + Y * S * xreg) * Sw;
    double YS = (YSh + Y * S * xreg) * Cw - (YCh + Y * C * xreg) * Sw;
    double P = ((YC * YC) / CC + (YS * YS) / SS) / YY;
    if (isnan(P) || isinf(P) || P < 0.0) P = -1.0;
    return P;
}

/* lomb.cu:85-123, FP64. */
static double lspow0_64(double C, double S, double C2, double S2, double YCh,
                        double YSh, double YY, double Y, const double *reg) {
    double tan2wt = S2 / C2;
    double r0 = 0, r1 = 0;
    if (reg) { r0 = reg[0]; r1 = reg[1]; }
    double C2wInv2 = 1.0 + tan2wt * tan2wt;
    double C2w = 1.0 / sqrt(C2wInv2);
    double S2w = tan2wt * C2w;
    double Cw = sqrt(0.5 * (1.0 + C2w));
    double Sw = sqrt(0.5 * (1.0 - C2w));
    if (S2w < 0) Sw = -Sw;
    double YC = (YCh + Y * C) * Cw + (YSh + Y * S) * Sw;
    double YS = (YSh + Y * S) * Cw - (YCh + Y * C) * Sw;
    double CC = 0.5 * (1.0 + C2 * C2w + S2 * S2w) + r0;
    double SS = 0.5 * (1.0 - C2 * C2w - S2 * S2w) + r1;
    double P = ((YC * YC) / CC + (YS * YS) / SS) / (YY + Y * Y);
    if (isnan(P) || isinf(P) || P < 0.0) P = -1.0;
    return P;
}

/*
 * Closed-form ("tau") GLS in FP64 for modes 0 (standard), 1 (floating mean)
 * and 2 (window), from direct sums (lomb.cu:126-165).  Y is the weighted mean
 * of y (LombScargleMemory.ybar); reg = (r0, r1, r2) or NULL.
 */
int oracle_gls_tau(const double *t, const double *yw, const double *w,
                   int64_t n, const double *freqs, int64_t nfreq, double YY,
                   double Y, const double *reg, int mode, double *P,
                   int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 64)
#endif
    for (int64_t i = 0; i < nfreq; ++i) {
        sums_t s;
        direct_sums_one(t, yw, w, n, freqs[i], &s);
        double p;
        switch (mode) {
        case 0: p = lspow0_64(s.C, s.S, s.C2, s.S2, s.yc, s.ys, YY, Y, reg); break;
        case 1: p = lspow_flmean64(s.C, s.S, s.C2, s.S2, s.yc, s.ys, YY, Y, reg); break;
        case 2: p = lspow0_64(s.C, s.S, s.C2, s.S2, s.C, s.S, 0.0, 1.0, NULL); break;
        default: p = -1.0;
        }
        P[i] = p;
    }
    return 0;
}

/*
 * Adjoint NFFT by direct summation (tests/test_nfft.py:31-34):
 * out[2k] + i out[2k+1] = sum_j y_j exp(+2 pi i f_k t_j), phase reduced in FP64.
 */
int oracle_nfft_direct(const double *t, const double *y, int64_t n,
                       const double *freqs, int64_t nfreq, double *out,
                       int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 64)
#endif
    for (int64_t i = 0; i < nfreq; ++i) {
        double re = 0, im = 0;
        for (int64_t j = 0; j < n; ++j) {
            double ph = 2.0 * ORACLE_PI * pymod1(t[j] * freqs[i]);
            re += y[j] * cos(ph);
            im += y[j] * sin(ph);
        }
        out[2 * i] = re;
        out[2 * i + 1] = im;
    }
    return 0;
}

/*
 * Reference-convention Gaussian gridding (cunfft.cu:84-163 and the scalar
 * restatement tests/test_nfft.py:57-87), FP64:
 *   x   = (t - tmin) / (spp * (tmax - tmin))        (scaled position)
 *   u   = floor(ng * x - m)
 *   grid[(u + k) mod ng] += y * exp(-(ng*x - u - k)^2 / b) / sqrt(pi b),
 *   k = 0 .. 2m,  b = 2 sigma m / ((2 sigma - 1) pi).
 * The scalar restatement writes the same weights as q1 * q2**k * q3[k].
 */
int oracle_grid_ref(const double *t, const double *y, int64_t n, int64_t ng,
                    int m, double sigma, double tmin, double tmax, double spp,
                    double *grid) {
    const double b = (2.0 * sigma * m) / ((2.0 * sigma - 1.0) * ORACLE_PI);
    const double norm = 1.0 / sqrt(ORACLE_PI * b);
    for (int64_t l = 0; l < ng; ++l) grid[l] = 0.0;
    for (int64_t j = 0; j < n; ++j) {
        double x = (t[j] - tmin) / (spp * (tmax - tmin));
        double gx = (double)ng * x;
        int64_t u = (int64_t)floor(gx - m);
        for (int k = 0; k <= 2 * m; ++k) {
            double d = gx - (double)(u + k);
            int64_t l = (u + k) % ng;
            if (l < 0) l += ng;
            grid[l] += y[j] * exp(-d * d / b) * norm;
        }
    }
    return 0;
}
