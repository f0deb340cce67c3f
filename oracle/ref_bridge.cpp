/*
 * ref_bridge.cpp -- plain C entry points around the reference's own four
 * operator MEX functions, compiled unmodified from
 *   reconstruction_model_based/models/forwardDelayAndSumMex.cpp:15
 *   reconstruction_model_based/models/transposeDelayAndSumMex.cpp:15
 *   reconstruction_model_based/models/forwardMex.cpp:16
 *   reconstruction_model_based/models/transposeMex.cpp:16
 * against the project's MEX stand-in header (mex_shim/mex.h).  Each source is
 * compiled with -DmexFunction=ref_<name>_mex so the four can share one .so.
 *
 * TEST INFRASTRUCTURE ONLY: this library is the FP64 oracle and the timed
 * CPU reference arm.  The product never links it.
 *
 * Because the reference does no bounds checking (forwardDelayAndSumMex.cpp:80
 * writes out of range when ceil(tau-r) < 0 or floor(tau+r) >= T), every entry
 * point validates the travel-time table first and returns -2 instead of
 * corrupting memory.  A MEX class error (mexErrMsgIdAndTxt) returns -1.
 */
#include "mex.h"
#include <cmath>
#include <omp.h>

void ref_forwardDelayAndSumMex_mex(int, mxArray *[], int, const mxArray *[]);
void ref_transposeDelayAndSumMex_mex(int, mxArray *[], int, const mxArray *[]);
void ref_forwardMex_mex(int, mxArray *[], int, const mxArray *[]);
void ref_transposeMex_mex(int, mxArray *[], int, const mxArray *[]);

static bool taps_in_range(const double *tt, long n, double r, int T) {
    for (long i = 0; i < n; ++i) {
        double t = tt[i];
        if (!std::isfinite(t)) return false;
        if ((long)std::ceil(t - r) < 0 || (long)std::floor(t + r) >= T) return false;
    }
    return true;
}

typedef void (*mexfn)(int, mxArray *[], int, const mxArray *[]);

static int call_mex(mexfn f, int nrhs, const mxArray **prhs, double *out, size_t nout) {
    mxArray *plhs[1] = {nullptr};
    try {
        f(1, plhs, nrhs, prhs);
    } catch (const mex_shim_error &) {
        if (plhs[0]) mxDestroyArray(plhs[0]);
        return -1;
    }
    std::memcpy(out, mxGetDoubles(plhs[0]), nout * sizeof(double));
    mxDestroyArray(plhs[0]);
    return 0;
}

extern "C" {

void ref_set_threads(int n) { omp_set_num_threads(n > 0 ? n : 1); }
int ref_max_threads(void) { return omp_get_max_threads(); }

/* image W x P, travelTimes P x D, out W x T x D (all column-major). */
int ref_forward_das(const double *image, int W, int P, const double *tt, int D, int T,
                    double radius, double *out) {
    if (!taps_in_range(tt, (long)P * D, radius, T)) return -2;
    mwSize di[2] = {(mwSize)W, (mwSize)P}, dt[2] = {(mwSize)P, (mwSize)D}, d1[2] = {1, 1};
    int32_t T32 = T;
    mxArray a0 = mx_wrap(mxDOUBLE_CLASS, (void *)image, 2, di);
    mxArray a1 = mx_wrap(mxDOUBLE_CLASS, (void *)tt, 2, dt);
    mxArray a2 = mx_wrap(mxINT32_CLASS, &T32, 2, d1);
    mxArray a3 = mx_wrap(mxDOUBLE_CLASS, &radius, 2, d1);
    const mxArray *prhs[4] = {&a0, &a1, &a2, &a3};
    return call_mex(ref_forwardDelayAndSumMex_mex, 4, prhs, out, (size_t)W * T * D);
}

/* sigMat W x T x D, travelTimes P x D, out W x P. */
int ref_transpose_das(const double *sig, int W, int T, int D, const double *tt, int P,
                      double radius, double *out) {
    if (!taps_in_range(tt, (long)P * D, radius, T)) return -2;
    mwSize ds[3] = {(mwSize)W, (mwSize)T, (mwSize)D}, dt[2] = {(mwSize)P, (mwSize)D}, d1[2] = {1, 1};
    mxArray a0 = mx_wrap(mxDOUBLE_CLASS, (void *)sig, 3, ds);
    mxArray a1 = mx_wrap(mxDOUBLE_CLASS, (void *)tt, 2, dt);
    mxArray a2 = mx_wrap(mxDOUBLE_CLASS, &radius, 2, d1);
    const mxArray *prhs[3] = {&a0, &a1, &a2};
    return call_mex(ref_transposeDelayAndSumMex_mex, 3, prhs, out, (size_t)W * P);
}

static bool sir_args_ok(const int32_t *idx, long n, const int32_t *se, int S, int NS) {
    for (long i = 0; i < n; ++i)
        if (idx[i] < 1 || idx[i] > NS) return false;
    for (int s = 0; s < NS; ++s)
        if (se[2 * s] < 1 || se[2 * s + 1] > S) return false;
    return true;
}

/* image W x P, sirIdx P x D (1-based), tt P x D, sir S x NS, startEnd 2 x NS (1-based). */
int ref_forward_sir(const double *image, int W, int P, const int32_t *sir_idx, const double *tt,
                    int D, const double *sir, int S, int NS, int T, const int32_t *start_end,
                    double radius, double *out) {
    if (!sir_args_ok(sir_idx, (long)P * D, start_end, S, NS)) return -2;
    for (long i = 0; i < (long)P * D; ++i)
        if (!std::isfinite(tt[i])) return -2;
    mwSize di[2] = {(mwSize)W, (mwSize)P}, dt[2] = {(mwSize)P, (mwSize)D};
    mwSize dsr[2] = {(mwSize)S, (mwSize)NS}, dse[2] = {2, (mwSize)NS}, d1[2] = {1, 1};
    int32_t T32 = T;
    mxArray a0 = mx_wrap(mxDOUBLE_CLASS, (void *)image, 2, di);
    mxArray a1 = mx_wrap(mxINT32_CLASS, (void *)sir_idx, 2, dt);
    mxArray a2 = mx_wrap(mxDOUBLE_CLASS, (void *)tt, 2, dt);
    mxArray a3 = mx_wrap(mxDOUBLE_CLASS, (void *)sir, 2, dsr);
    mxArray a4 = mx_wrap(mxINT32_CLASS, &T32, 2, d1);
    mxArray a5 = mx_wrap(mxINT32_CLASS, (void *)start_end, 2, dse);
    mxArray a6 = mx_wrap(mxDOUBLE_CLASS, &radius, 2, d1);
    const mxArray *prhs[7] = {&a0, &a1, &a2, &a3, &a4, &a5, &a6};
    return call_mex(ref_forwardMex_mex, 7, prhs, out, (size_t)W * T * D);
}

/* sigMat W x T x D, out W x P. */
int ref_transpose_sir(const double *sig, int W, int T, int D, const int32_t *sir_idx,
                      const double *tt, int P, const double *sir, int S, int NS,
                      const int32_t *start_end, double radius, double *out) {
    if (!sir_args_ok(sir_idx, (long)P * D, start_end, S, NS)) return -2;
    for (long i = 0; i < (long)P * D; ++i)
        if (!std::isfinite(tt[i])) return -2;
    mwSize ds[3] = {(mwSize)W, (mwSize)T, (mwSize)D}, dt[2] = {(mwSize)P, (mwSize)D};
    mwSize dsr[2] = {(mwSize)S, (mwSize)NS}, dse[2] = {2, (mwSize)NS}, d1[2] = {1, 1};
    mxArray a0 = mx_wrap(mxDOUBLE_CLASS, (void *)sig, 3, ds);
    mxArray a1 = mx_wrap(mxINT32_CLASS, (void *)sir_idx, 2, dt);
    mxArray a2 = mx_wrap(mxDOUBLE_CLASS, (void *)tt, 2, dt);
    mxArray a3 = mx_wrap(mxDOUBLE_CLASS, (void *)sir, 2, dsr);
    mxArray a4 = mx_wrap(mxINT32_CLASS, (void *)start_end, 2, dse);
    mxArray a5 = mx_wrap(mxDOUBLE_CLASS, &radius, 2, d1);
    const mxArray *prhs[6] = {&a0, &a1, &a2, &a3, &a4, &a5};
    return call_mex(ref_transposeMex_mex, 6, prhs, out, (size_t)W * P);
}

}  // extern "C"
