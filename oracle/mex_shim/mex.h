/*
 * mex.h -- a minimal stand-in for MATLAB's MEX C API (interleaved-complex,
 * `mex -R2018a` flavour), written for this project.
 *
 * Test infrastructure, not product: it lets the reference's four operator
 * MEX sources (reconstruction_model_based/models/{forward,transpose}Mex.cpp,
 * {forward,transpose}DelayAndSumMex.cpp) compile unmodified with g++ when
 * MATLAB is absent, so that they can act as the FP64 oracle, and it lets the
 * project's own GPU MEX gateways be compile-checked.  Only the calls those
 * sources use are provided.  Arrays are column-major, real, double or int32.
 *
 * Errors: mexErrMsgIdAndTxt() throws mex_shim_error (a C++ exception); the
 * bridge functions that call a mexFunction catch it and return an error code.
 */
#ifndef MSOT_MEX_SHIM_H
#define MSOT_MEX_SHIM_H

#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cstdarg>
#include <string>
#include <stdexcept>

typedef size_t mwSize;
typedef size_t mwIndex;

typedef enum { mxUNKNOWN_CLASS = 0, mxDOUBLE_CLASS = 6, mxINT32_CLASS = 12 } mxClassID;
typedef enum { mxREAL = 0, mxCOMPLEX = 1 } mxComplexity;

struct mxArray {
    mxClassID cls;
    mwSize ndim;
    mwSize dims[8];
    void *data;
    bool owns;
};

struct mex_shim_error : public std::runtime_error {
    std::string id;
    mex_shim_error(const char *i, const char *m) : std::runtime_error(m), id(i) {}
};

inline mwSize mx_numel_(const mxArray *a) {
    mwSize n = 1;
    for (mwSize k = 0; k < a->ndim; ++k) n *= a->dims[k];
    return n;
}
inline size_t mx_elsize_(mxClassID c) { return c == mxDOUBLE_CLASS ? 8 : 4; }

/* Wrap caller-owned memory as an mxArray (no copy). */
inline mxArray mx_wrap(mxClassID cls, void *data, mwSize ndim, const mwSize *dims) {
    mxArray a;
    a.cls = cls;
    a.ndim = ndim < 2 ? 2 : ndim;
    a.dims[0] = 1; a.dims[1] = 1;
    for (mwSize k = 0; k < ndim && k < 8; ++k) a.dims[k] = dims[k];
    a.data = data;
    a.owns = false;
    return a;
}

inline mxArray *mxCreateNumericArray(mwSize ndim, const mwSize *dims, mxClassID cls, mxComplexity) {
    mxArray *a = new mxArray;
    *a = mx_wrap(cls, nullptr, ndim, dims);
    a->data = std::calloc(mx_numel_(a) ? mx_numel_(a) : 1, mx_elsize_(cls));
    a->owns = true;
    return a;
}
inline mxArray *mxCreateDoubleMatrix(mwSize m, mwSize n, mxComplexity c) {
    mwSize d[2] = {m, n};
    return mxCreateNumericArray(2, d, mxDOUBLE_CLASS, c);
}
inline void mxDestroyArray(mxArray *a) {
    if (!a) return;
    if (a->owns) std::free(a->data);
    delete a;
}

inline bool mxIsDouble(const mxArray *a) { return a->cls == mxDOUBLE_CLASS; }
inline bool mxIsInt32(const mxArray *a) { return a->cls == mxINT32_CLASS; }
inline bool mxIsComplex(const mxArray *) { return false; }
inline double *mxGetDoubles(const mxArray *a) { return a->cls == mxDOUBLE_CLASS ? (double *)a->data : nullptr; }
inline int32_t *mxGetInt32s(const mxArray *a) { return a->cls == mxINT32_CLASS ? (int32_t *)a->data : nullptr; }
inline mwSize mxGetM(const mxArray *a) { return a->dims[0]; }
inline mwSize mxGetN(const mxArray *a) {
    mwSize n = 1;
    for (mwSize k = 1; k < a->ndim; ++k) n *= a->dims[k];
    return n;
}
inline mwSize mxGetNumberOfDimensions(const mxArray *a) { return a->ndim; }
inline const mwSize *mxGetDimensions(const mxArray *a) { return a->dims; }
inline double mxGetScalar(const mxArray *a) {
    if (a->cls == mxDOUBLE_CLASS) return ((const double *)a->data)[0];
    if (a->cls == mxINT32_CLASS) return (double)((const int32_t *)a->data)[0];
    return 0.0;
}

[[noreturn]] inline void mexErrMsgIdAndTxt(const char *id, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    throw mex_shim_error(id, buf);
}
inline int mexPrintf(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    int n = std::vprintf(fmt, ap);
    va_end(ap);
    return n;
}

#endif
