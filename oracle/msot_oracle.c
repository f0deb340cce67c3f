/*
 * msot_oracle.c -- CPU restatement (FP64, OpenMP, portable C) of the four
 * model-based operator MEX functions of juestellab/mb-rec-msot.
 *
 * TEST INFRASTRUCTURE ONLY ("the oracle"): used by tests/ as the checker,
 * by __graft_entry__.smoke() and by bench.py's CPU baseline leg.  The
 * product (the CUDA library) never links or calls it.
 *
 * Each function restates the arithmetic of one reference file with the same
 * accumulation order per output element, so with floating-point contraction
 * disabled (-ffp-contract=off) it reproduces the reference MEX bit for bit on
 * any host (the reference itself needs x86 AVX intrinsics and does not build
 * on aarch64):
 *   orc_forward_das    <- forwardDelayAndSumMex.cpp:72-103
 *   orc_transpose_das  <- transposeDelayAndSumMex.cpp:67-97
 *   orc_forward_sir    <- forwardMex.cpp:100-161
 *   orc_transpose_sir  <- transposeMex.cpp:97-158 (file lines 259-320 of the
 *                         concatenated listing; loop over pixels outermost)
 * Notation: tri weight  f = 1 - |t - tau| / r  on taps t = ceil(tau-r) ..
 * floor(tau+r); arrays are column-major as in MATLAB: image W x P, sinogram
 * W x T x D, travel times P x D, SIR S x NS, start/end 2 x NS (1-based).
 *
 * Unlike the reference, every entry point range-checks its inputs first
 * (finite travel times; all DAS taps inside [0, T); SIR indices in range) and
 * returns -2 rather than reading or writing out of bounds.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static int das_taps_ok(const double *tt, long n, double r, int T) {
    for (long i = 0; i < n; ++i) {
        double t = tt[i];
        if (!isfinite(t)) return 0;
        if ((long)ceil(t - r) < 0 || (long)floor(t + r) >= T) return 0;
    }
    return 1;
}

static int sir_ok(const int32_t *idx, long n, const int32_t *se, int S, int NS, const double *tt) {
    for (long i = 0; i < n; ++i) {
        if (idx[i] < 1 || idx[i] > NS) return 0;
        if (!isfinite(tt[i])) return 0;
    }
    for (int s = 0; s < NS; ++s)
        if (se[2 * s] < 1 || se[2 * s + 1] > S) return 0;
    return 1;
}

void orc_set_threads(int n) {
#ifdef _OPENMP
    omp_set_num_threads(n > 0 ? n : 1);
#else
    (void)n;
#endif
}

int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* Scatter: one detector column per thread, pixels in order, taps in order. */
int orc_forward_das(const double *image, int W, int P, const double *tt, int D, int T,
                    double r, double *out) {
    if (!das_taps_ok(tt, (long)P * D, r, T)) return -2;
    memset(out, 0, sizeof(double) * (size_t)W * T * D);
#pragma omp parallel for schedule(static)
    for (int d = 0; d < D; ++d) {
        double *col = out + (size_t)d * W * T;
        const double *tau_d = tt + (size_t)d * P;
        for (int p = 0; p < P; ++p) {
            const double tau = tau_d[p];
            const int t0 = (int)ceil(tau - r), t1 = (int)floor(tau + r);
            const double *xp = image + (size_t)p * W;
            for (int t = t0; t <= t1; ++t) {
                const double f = 1.0 - fabs((double)t - tau) / r;
                double *yt = col + (size_t)t * W;
                for (int w = 0; w < W; ++w) yt[w] += f * xp[w];
            }
        }
    }
    return 0;
}

/* Gather: one pixel per thread, detectors in order, taps in order. */
int orc_transpose_das(const double *sig, int W, int T, int D, const double *tt, int P,
                      double r, double *out) {
    if (!das_taps_ok(tt, (long)P * D, r, T)) return -2;
    memset(out, 0, sizeof(double) * (size_t)W * P);
#pragma omp parallel for schedule(static)
    for (int p = 0; p < P; ++p) {
        double *xp = out + (size_t)p * W;
        for (int d = 0; d < D; ++d) {
            const double tau = tt[(size_t)d * P + p];
            const int t0 = (int)ceil(tau - r), t1 = (int)floor(tau + r);
            const double *col = sig + (size_t)d * W * T;
            for (int t = t0; t <= t1; ++t) {
                const double f = 1.0 - fabs((double)t - tau) / r;
                const double *yt = col + (size_t)t * W;
                for (int w = 0; w < W; ++w) xp[w] = xp[w] + f * yt[w];
            }
        }
    }
    return 0;
}

/* SIR scatter: for every (pixel, detector) the SIR column s = idx-1 is
 * convolved with the tri interpolation; samples outside [0, T) are dropped. */
int orc_forward_sir(const double *image, int W, int P, const int32_t *sir_idx, const double *tt,
                    int D, const double *sir, int S, int NS, int T, const int32_t *start_end,
                    double r, double *out) {
    if (!sir_ok(sir_idx, (long)P * D, start_end, S, NS, tt)) return -2;
    memset(out, 0, sizeof(double) * (size_t)W * T * D);
    const int half = S / 2;
#pragma omp parallel for schedule(static)
    for (int d = 0; d < D; ++d) {
        double *col = out + (size_t)d * W * T;
        for (int p = 0; p < P; ++p) {
            const size_t pd = (size_t)d * P + p;
            const int s = sir_idx[pd] - 1;
            const double tau = tt[pd];
            const int t0 = (int)ceil(tau - r), t1 = (int)floor(tau + r);
            const double *xp = image + (size_t)p * W;
            const double *h = sir + (size_t)s * S;
            for (int k = start_end[2 * s] - 1; k <= start_end[2 * s + 1] - 1; ++k) {
                const double hk = h[k];
                for (int t = t0; t <= t1; ++t) {
                    const int j = t + k - half;
                    if (j < 0 || j >= T) continue;
                    const double f = 1.0 - fabs((double)t - tau) / r;
                    const double g = f * hk;
                    double *yj = col + (size_t)j * W;
                    for (int w = 0; w < W; ++w) yj[w] += g * xp[w];
                }
            }
        }
    }
    return 0;
}

/* SIR gather: exact adjoint of orc_forward_sir. */
int orc_transpose_sir(const double *sig, int W, int T, int D, const int32_t *sir_idx,
                      const double *tt, int P, const double *sir, int S, int NS,
                      const int32_t *start_end, double r, double *out) {
    if (!sir_ok(sir_idx, (long)P * D, start_end, S, NS, tt)) return -2;
    memset(out, 0, sizeof(double) * (size_t)W * P);
    const int half = S / 2;
#pragma omp parallel for schedule(static)
    for (int p = 0; p < P; ++p) {
        double *xp = out + (size_t)p * W;
        for (int d = 0; d < D; ++d) {
            const size_t pd = (size_t)d * P + p;
            const int s = sir_idx[pd] - 1;
            const double tau = tt[pd];
            const int t0 = (int)ceil(tau - r), t1 = (int)floor(tau + r);
            const double *col = sig + (size_t)d * W * T;
            const double *h = sir + (size_t)s * S;
            for (int k = start_end[2 * s] - 1; k <= start_end[2 * s + 1] - 1; ++k) {
                const double hk = h[k];
                for (int t = t0; t <= t1; ++t) {
                    const int j = t + k - half;
                    if (j < 0 || j >= T) continue;
                    const double f = 1.0 - fabs((double)t - tau) / r;
                    const double g = f * hk;
                    const double *yj = col + (size_t)j * W;
                    for (int w = 0; w < W; ++w) xp[w] = xp[w] + g * yj[w];
                }
            }
        }
    }
    return 0;
}
