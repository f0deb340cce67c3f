/*
 * mex.h -- a minimal stand-in for MATLAB's MEX C API (interleaved-complex,
 * `mex -R2018a` flavour), written for this project.  Besides the numeric
 * arrays of the four operator MEX sources it has what the project's model
 * and solver gateways use: 1 x 1 structs (standing in for the reference's
 * model object, whose properties mxGetProperty reads), uint64 handles,
 * character arrays, complex doubles, function handles (func2str through
 * mexCallMATLAB) and mexLock / mexUnlock.
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
#include <utility>
#include <vector>

typedef size_t mwSize;
typedef size_t mwIndex;

typedef enum {
    mxUNKNOWN_CLASS = 0,
    mxSTRUCT_CLASS = 2,
    mxLOGICAL_CLASS = 3,
    mxCHAR_CLASS = 4,
    mxDOUBLE_CLASS = 6,
    mxINT32_CLASS = 12,
    mxUINT64_CLASS = 15,
    mxFUNCTION_CLASS = 16
} mxClassID;
typedef enum { mxREAL = 0, mxCOMPLEX = 1 } mxComplexity;
typedef struct {
    double real, imag;
} mxComplexDouble;
typedef bool mxLogical;
typedef char mxChar_;

/* Struct arrays are 1 x 1 here (field name -> value); character arrays and
 * function handles hold their text (for a function handle, what func2str
 * returns). */
struct mxArray {
    mxClassID cls;
    mwSize ndim;
    mwSize dims[8];
    void *data;
    bool owns;
    bool complex_ = false;
    std::vector<std::pair<std::string, mxArray *>> fields;
    std::string text;
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
inline size_t mx_elsize_(const mxArray *a) {
    switch (a->cls) {
        case mxDOUBLE_CLASS: return a->complex_ ? 16 : 8;
        case mxUINT64_CLASS: return 8;
        case mxLOGICAL_CLASS: return 1;
        default: return 4;
    }
}

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

inline mxArray *mxCreateNumericArray(mwSize ndim, const mwSize *dims, mxClassID cls,
                                     mxComplexity cx) {
    mxArray *a = new mxArray;
    *a = mx_wrap(cls, nullptr, ndim, dims);
    a->complex_ = cx == mxCOMPLEX;
    a->data = std::calloc(mx_numel_(a) ? mx_numel_(a) : 1, mx_elsize_(a));
    a->owns = true;
    return a;
}
inline mxArray *mxCreateNumericMatrix(mwSize m, mwSize n, mxClassID cls, mxComplexity c) {
    mwSize d[2] = {m, n};
    return mxCreateNumericArray(2, d, cls, c);
}
inline mxArray *mxCreateDoubleMatrix(mwSize m, mwSize n, mxComplexity c) {
    return mxCreateNumericMatrix(m, n, mxDOUBLE_CLASS, c);
}
inline mxArray *mxCreateDoubleScalar(double v) {
    mxArray *a = mxCreateDoubleMatrix(1, 1, mxREAL);
    *(double *)a->data = v;
    return a;
}
inline mxArray *mxCreateString(const char *str) {
    mxArray *a = new mxArray;
    const mwSize d[2] = {1, (mwSize)std::strlen(str)};
    *a = mx_wrap(mxCHAR_CLASS, nullptr, 2, d);
    a->text = str;
    return a;
}
inline mxArray *mxCreateStructMatrix(mwSize m, mwSize n, int nfields, const char **names) {
    mxArray *a = new mxArray;
    const mwSize d[2] = {m, n};
    *a = mx_wrap(mxSTRUCT_CLASS, nullptr, 2, d);
    for (int k = 0; k < nfields; ++k) a->fields.push_back({names[k], nullptr});
    return a;
}
inline void mxDestroyArray(mxArray *a) {
    if (!a) return;
    if (a->owns) std::free(a->data);
    for (auto &f : a->fields) mxDestroyArray(f.second);
    delete a;
}
/* Test helper (not in MATLAB's API): a function handle whose func2str text is `text`. */
inline mxArray *mx_shim_function_handle(const char *text) {
    mxArray *a = new mxArray;
    const mwSize d[2] = {1, 1};
    *a = mx_wrap(mxFUNCTION_CLASS, nullptr, 2, d);
    a->text = text;
    return a;
}

inline bool mxIsStruct(const mxArray *a) { return a && a->cls == mxSTRUCT_CLASS; }
inline bool mxIsChar(const mxArray *a) { return a && a->cls == mxCHAR_CLASS; }
inline bool mxIsUint64(const mxArray *a) { return a && a->cls == mxUINT64_CLASS; }
inline bool mxIsLogical(const mxArray *a) { return a && a->cls == mxLOGICAL_CLASS; }
inline bool mxIsClass(const mxArray *a, const char *name) {
    if (!a) return false;
    if (std::strcmp(name, "function_handle") == 0) return a->cls == mxFUNCTION_CLASS;
    if (std::strcmp(name, "double") == 0) return a->cls == mxDOUBLE_CLASS;
    if (std::strcmp(name, "struct") == 0) return a->cls == mxSTRUCT_CLASS;
    return false;
}
inline mwSize mxGetNumberOfElements(const mxArray *a) {
    return a->cls == mxCHAR_CLASS ? a->text.size() : mx_numel_(a);
}
inline bool mxIsEmpty(const mxArray *a) { return mxGetNumberOfElements(a) == 0; }
inline mxArray *mxGetField(const mxArray *a, mwIndex, const char *name) {
    if (!a || a->cls != mxSTRUCT_CLASS) return nullptr;
    for (auto &f : a->fields)
        if (f.first == name) return f.second;
    return nullptr;
}
/* MATLAB returns a copy of an object's property; for the 1 x 1 structs that
 * stand in for objects here the field itself is returned (not to be freed). */
inline mxArray *mxGetProperty(const mxArray *a, mwIndex i, const char *name) {
    return mxGetField(a, i, name);
}
inline void mxSetField(mxArray *a, mwIndex, const char *name, mxArray *v) {
    for (auto &f : a->fields)
        if (f.first == name) {
            mxDestroyArray(f.second);
            f.second = v;
            return;
        }
    a->fields.push_back({name, v});
}
inline char *mxArrayToString(const mxArray *a) {
    if (!a || a->cls != mxCHAR_CLASS) return nullptr;
    char *s = (char *)std::malloc(a->text.size() + 1);
    std::memcpy(s, a->text.c_str(), a->text.size() + 1);
    return s;
}
inline void mxFree(void *p) { std::free(p); }
inline uint64_t *mxGetUint64s(const mxArray *a) {
    return a->cls == mxUINT64_CLASS ? (uint64_t *)a->data : nullptr;
}
inline mxComplexDouble *mxGetComplexDoubles(const mxArray *a) {
    return (a->cls == mxDOUBLE_CLASS && a->complex_) ? (mxComplexDouble *)a->data : nullptr;
}

inline bool mxIsDouble(const mxArray *a) { return a->cls == mxDOUBLE_CLASS; }
inline bool mxIsInt32(const mxArray *a) { return a->cls == mxINT32_CLASS; }
inline bool mxIsComplex(const mxArray *a) { return a->complex_; }
inline double *mxGetDoubles(const mxArray *a) {
    return (a->cls == mxDOUBLE_CLASS && !a->complex_) ? (double *)a->data : nullptr;
}
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
    if (mx_numel_(a) == 0 || !a->data) return 0.0;
    if (a->cls == mxDOUBLE_CLASS) return ((const double *)a->data)[0];
    if (a->cls == mxINT32_CLASS) return (double)((const int32_t *)a->data)[0];
    if (a->cls == mxUINT64_CLASS) return (double)((const uint64_t *)a->data)[0];
    if (a->cls == mxLOGICAL_CLASS) return ((const bool *)a->data)[0] ? 1.0 : 0.0;
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
/* MEX-file locking: a counter here (MATLAB keeps a locked MEX file loaded) */
inline int &mex_shim_lock_count() {
    static int n = 0;
    return n;
}
inline void mexLock(void) { ++mex_shim_lock_count(); }
inline void mexUnlock(void) { --mex_shim_lock_count(); }
inline bool mexIsLocked(void) { return mex_shim_lock_count() > 0; }
inline int mexAtExit(void (*)(void)) { return 0; }
/* Only func2str of a function handle is provided. */
inline int mexCallMATLAB(int nlhs, mxArray *plhs[], int nrhs, mxArray *prhs[], const char *name) {
    if (std::strcmp(name, "func2str") == 0 && nlhs >= 1 && nrhs == 1 && prhs[0] &&
        prhs[0]->cls == mxFUNCTION_CLASS) {
        plhs[0] = mxCreateString(prhs[0]->text.c_str());
        return 0;
    }
    return 1;
}
inline int mexPrintf(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    int n = std::vprintf(fmt, ap);
    va_end(ap);
    return n;
}

#endif
