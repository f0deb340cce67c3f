/*
 * msot_mex_model.h -- helpers shared by the model and solver MEX gateways:
 * members of the reference's model object, the plan behind a `model`
 * argument, and the kind of a regulariser argument.
 *
 * The reference's model is a MATLAB object (MSOTmodel.m:1-11) whose
 * properties Data, Discretization and Probe are structs / objects; the
 * gateways read them with mxGetField (structs) or mxGetProperty (objects,
 * which returns a copy the gateway frees).  The GPU model that the solver
 * gateways take is the uint64 handle msot_model_mex('create', ...) returns,
 * or a struct / object holding it in a field gpuPlan.
 */
#ifndef MSOT_MEX_MODEL_H
#define MSOT_MEX_MODEL_H

#include <cstdint>
#include <cstring>
#include <string>

#include "mex.h"
#include "msot_gpu.h"

/* One member of a struct or object (an object's property is a copy). */
struct msot_mex_member {
    const mxArray *a = nullptr;
    mxArray *owned = nullptr;
    msot_mex_member(const mxArray *obj, const char *name) {
        if (!obj) return;
        if (mxIsStruct(obj)) {
            a = mxGetField(obj, 0, name);
        } else {
            owned = mxGetProperty(obj, 0, name);
            a = owned;
        }
    }
    ~msot_mex_member() {
        if (owned) mxDestroyArray(owned);
    }
    msot_mex_member(const msot_mex_member &) = delete;
    msot_mex_member &operator=(const msot_mex_member &) = delete;
};

static inline std::string msot_mex_id(const char *who, const char *what) {
    return std::string(who) + ":" + what;
}

/* The live plan behind `model` (a uint64 handle, or a struct / object with a
 * uint64 gpuPlan); raises <who>:model otherwise. */
static inline msot_plan_t msot_mex_plan(const mxArray *model, const char *who) {
    uint64_t h = 0;
    bool found = false;
    if (model && mxIsUint64(model) && mxGetNumberOfElements(model) == 1) {
        h = mxGetUint64s(model)[0];
        found = true;
    } else if (model) {
        msot_mex_member m(model, "gpuPlan");
        if (m.a && mxIsUint64(m.a) && mxGetNumberOfElements(m.a) == 1) {
            h = mxGetUint64s(m.a)[0];
            found = true;
        }
    }
    msot_plan_t p = (msot_plan_t)(uintptr_t)h;
    if (!found || !msot_plan_valid(p))
        mexErrMsgIdAndTxt(msot_mex_id(who, "model").c_str(),
                          "model must be a live GPU model: the uint64 handle of "
                          "msot_model_mex('create', ...), or a struct with it in gpuPlan.");
    return p;
}

/* Real double array with the given element count. */
static inline const double *msot_mex_doubles(const mxArray *a, size_t n, const char *who,
                                             const char *name) {
    if (!a || !mxIsDouble(a) || mxIsComplex(a) || (size_t)mxGetNumberOfElements(a) != n)
        mexErrMsgIdAndTxt(msot_mex_id(who, "input").c_str(),
                          "%s must be a real double array of %zu elements.", name, n);
    return mxGetDoubles(a);
}

/* A scalar, or `dflt` for a missing or empty ([]) argument. */
static inline double msot_mex_scalar_or(int nrhs, const mxArray *prhs[], int i, double dflt) {
    if (i >= nrhs || !prhs[i] || mxIsEmpty(prhs[i])) return dflt;
    return mxGetScalar(prhs[i]);
}

enum msot_reg_kind { MSOT_REG_NONE, MSOT_REG_IDENTITY, MSOT_REG_LAPLACIAN, MSOT_REG_OTHER };

/* Kind of a regulariser argument of rec_nn_with_L2_reg: [] or missing; the
 * identity (a function handle whose func2str is "@(v)v", or 'identity');
 * laplacian_per_wavelength (a handle whose text calls it, as the reference's
 * overview script writes, or the name); anything else. */
static inline msot_reg_kind msot_mex_reg_kind(int nrhs, const mxArray *prhs[], int i) {
    if (i >= nrhs || !prhs[i] || mxIsEmpty(prhs[i])) return MSOT_REG_NONE;
    std::string txt;
    if (mxIsChar(prhs[i])) {
        char *s = mxArrayToString(prhs[i]);
        txt = s ? s : "";
        mxFree(s);
    } else if (mxIsClass(prhs[i], "function_handle")) {
        mxArray *in = const_cast<mxArray *>(prhs[i]);
        mxArray *out = nullptr;
        if (mexCallMATLAB(1, &out, 1, &in, "func2str") != 0 || !out) return MSOT_REG_OTHER;
        char *s = mxArrayToString(out);
        txt = s ? s : "";
        mxFree(s);
        mxDestroyArray(out);
    } else {
        return MSOT_REG_OTHER;
    }
    std::string t;
    for (char c : txt)
        if (c != ' ' && c != '\t') t += c;
    if (t == "identity") return MSOT_REG_IDENTITY;
    if (t.find("laplacian_per_wavelength") != std::string::npos) return MSOT_REG_LAPLACIAN;
    if (t.size() >= 5 && t[0] == '@' && t[1] == '(') {
        const size_t close = t.find(')');
        if (close != std::string::npos && close > 2 && t.substr(2, close - 2) == t.substr(close + 1))
            return MSOT_REG_IDENTITY;
    }
    return MSOT_REG_OTHER;
}

/* err (zeros) and t (per-iteration time, the mean over the solve) outputs
 * of the reference's solvers: calculate_objective_per_iter is false there,
 * so err stays zeros(nIter, 1) (nnls_L2_less.m:32-33). */
static inline void msot_mex_iter_outputs(int nlhs, mxArray *plhs[], int first, int num_iter,
                                         double seconds) {
    const mwSize n = (mwSize)(num_iter > 0 ? num_iter : 0);
    if (nlhs > first) plhs[first] = mxCreateDoubleMatrix(n, 1, mxREAL);
    if (nlhs > first + 1) {
        plhs[first + 1] = mxCreateDoubleMatrix(n, 1, mxREAL);
        double *t = mxGetDoubles(plhs[first + 1]);
        for (mwSize k = 0; k < n; ++k) t[k] = seconds / (double)n;
    }
}

/* The reconstruction stack Nz x Nx x W (Nz x Nx for one wavelength), as
 * reshape(rec_img, N(2), N(1), []) returns it. */
static inline mxArray *msot_mex_image_stack(int nx, int nz, int W) {
    const mwSize d3[3] = {(mwSize)nz, (mwSize)nx, (mwSize)W};
    return mxCreateNumericArray(W > 1 ? 3 : 2, d3, mxDOUBLE_CLASS, mxREAL);
}

/* Wavelengths W of a T x D x W stack (raises <who>:input if the element
 * count is not a multiple of T * D or exceeds max_batch). */
static inline int msot_mex_wavelengths(const mxArray *data, msot_plan_t plan, const char *who,
                                       int *nx, int *nz, int *D, int *T) {
    int mb = 0;
    msot_plan_shape(plan, nx, nz, D, T, &mb);
    const size_t per = (size_t)(*D) * (size_t)(*T);
    const size_t n = data ? (size_t)mxGetNumberOfElements(data) : 0;
    if (!data || !mxIsDouble(data) || mxIsComplex(data) || n == 0 || n % per)
        mexErrMsgIdAndTxt(msot_mex_id(who, "input").c_str(),
                          "data_filt must be a real double T x D x W array with T = %d and "
                          "D = %d.",
                          *T, *D);
    const int W = (int)(n / per);
    if (W > mb)
        mexErrMsgIdAndTxt(msot_mex_id(who, "input").c_str(),
                          "%d wavelengths exceed the GPU model's maxBatch %d.", W, mb);
    return W;
}

#endif
