/*
 * mex_gateway_driver.cpp -- test driver for the model and solver MEX
 * gateways (msot_model_mex, rec_nn_with_L2_reg, rec_nn_with_L1_eye_reg,
 * rec_nn_with_TV_reg), each compiled with -Dmexfunction=gw_<name> against
 * the project's MEX stand-in header.  The functions below build the
 * mxArrays a MATLAB caller would pass -- a 1 x 1 struct standing in for the
 * reference's model object, function handles with their func2str text --
 * call the gateway, and copy the outputs into caller memory, so that a
 * Python test can drive the gateways through ctypes.  Each returns 0, or 1
 * with "<error id>|<message>" in msg when the gateway raised an error.
 */
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "mex.h"

void gw_msot_model_mex(int, mxArray *[], int, const mxArray *[]);
void gw_rec_nn_with_L2_reg(int, mxArray *[], int, const mxArray *[]);
void gw_rec_nn_with_L1_eye_reg(int, mxArray *[], int, const mxArray *[]);
void gw_rec_nn_with_TV_reg(int, mxArray *[], int, const mxArray *[]);

typedef void (*mexfn)(int, mxArray *[], int, const mxArray *[]);

namespace {

mxArray *doubles(const double *v, mwSize m, mwSize n) {
    mxArray *a = mxCreateDoubleMatrix(m, n, mxREAL);
    if (m * n) std::memcpy(mxGetDoubles(a), v, m * n * sizeof(double));
    return a;
}

mxArray *complexes(const double *interleaved, mwSize m, mwSize n) {
    mxArray *a = mxCreateDoubleMatrix(m, n, mxCOMPLEX);
    std::memcpy(mxGetComplexDoubles(a), interleaved, m * n * 2 * sizeof(double));
    return a;
}

mxArray *uint64_scalar(uint64_t h) {
    mxArray *a = mxCreateNumericMatrix(1, 1, mxUINT64_CLASS, mxREAL);
    mxGetUint64s(a)[0] = h;
    return a;
}

// a regulariser argument: NULL -> [], "fh:<text>" -> function handle with
// that func2str text, otherwise a character array
mxArray *reg_arg(const char *spec) {
    if (!spec) return mxCreateDoubleMatrix(0, 0, mxREAL);
    if (std::strncmp(spec, "fh:", 3) == 0) return mx_shim_function_handle(spec + 3);
    return mxCreateString(spec);
}

int call(mexfn f, int nlhs, mxArray *plhs[], std::vector<mxArray *> &in, char *msg, int msglen) {
    std::vector<const mxArray *> prhs(in.begin(), in.end());
    int rc = 0;
    try {
        f(nlhs, plhs, (int)prhs.size(), prhs.data());
    } catch (const mex_shim_error &e) {
        std::snprintf(msg, (size_t)msglen, "%s|%s", e.id.c_str(), e.what());
        rc = 1;
    }
    for (mxArray *a : in) mxDestroyArray(a);
    return rc;
}

}  // namespace

extern "C" {

/* msot_model_mex('create', model, norm, maxBatch) with model.Data /
 * Discretization / Probe filled from the arguments (pre_interleaved may be
 * NULL: no prefilter member; norm <= 0: []). */
int drv_create(int nx, int nz, int n_det, int n_t, double radius, const double *travel,
               const double *ir_hat_interleaved, int n_hat, int eir_length,
               const double *pre_interleaved, double norm, int max_batch, uint64_t *handle,
               char *msg, int msglen) {
    const char *top[] = {"Data", "Discretization", "Probe", "includeSir"};
    mxArray *model = mxCreateStructMatrix(1, 1, 4, top);
    mxArray *data = mxCreateStructMatrix(1, 1, 0, nullptr);
    mxSetField(data, 0, "absoluteTravelTimeIndices", doubles(travel, (mwSize)nx * nz, n_det));
    mxSetField(data, 0, "circularInterpolationRadiusInSamples", mxCreateDoubleScalar(radius));
    mxArray *nt = mxCreateNumericMatrix(1, 1, mxINT32_CLASS, mxREAL);
    mxGetInt32s(nt)[0] = n_t;
    mxSetField(data, 0, "numTimeSamplesPerTransducer", nt);
    if (ir_hat_interleaved)
        mxSetField(data, 0, "IRHat", complexes(ir_hat_interleaved, (mwSize)n_hat, 1));
    mxArray *disc = mxCreateStructMatrix(1, 1, 0, nullptr);
    const double grid[2] = {(double)nx, (double)nz};
    mxSetField(disc, 0, "sizeOfPixelGrid", doubles(grid, 1, 2));
    if (pre_interleaved) mxSetField(disc, 0, "prefilter", complexes(pre_interleaved, nz, nx));
    mxArray *probe = mxCreateStructMatrix(1, 1, 0, nullptr);
    mxSetField(probe, 0, "eirLength", mxCreateDoubleScalar(eir_length));
    mxSetField(model, 0, "Data", data);
    mxSetField(model, 0, "Discretization", disc);
    mxSetField(model, 0, "Probe", probe);
    mxSetField(model, 0, "includeSir", mxCreateDoubleScalar(0.0));
    std::vector<mxArray *> in = {mxCreateString("create"), model,
                                 norm > 0 ? mxCreateDoubleScalar(norm)
                                          : mxCreateDoubleMatrix(0, 0, mxREAL),
                                 mxCreateDoubleScalar(max_batch)};
    mxArray *out[1] = {nullptr};
    if (call(gw_msot_model_mex, 1, out, in, msg, msglen)) return 1;
    *handle = mxGetUint64s(out[0])[0];
    mxDestroyArray(out[0]);
    return 0;
}

/* msot_model_mex(command, h [, data]) for destroy / normalizationFactor /
 * applyForward / applyTranspose; out receives n_out doubles (may be NULL). */
int drv_model(const char *command, uint64_t h, const double *in_data, size_t n_in, double *out,
              size_t n_out, char *msg, int msglen) {
    std::vector<mxArray *> in = {mxCreateString(command), uint64_scalar(h)};
    if (in_data) in.push_back(doubles(in_data, (mwSize)n_in, 1));
    mxArray *o[1] = {nullptr};
    if (call(gw_msot_model_mex, 1, o, in, msg, msglen)) return 1;
    if (o[0]) {
        if (out) std::memcpy(out, mxGetDoubles(o[0]), n_out * sizeof(double));
        mxDestroyArray(o[0]);
    }
    return 0;
}

/* rec_nn_with_L2_reg(model, data, num_iter, lambdaL2, RegL2, RegL2T,
 * lambdaL2_2, RegL2_2, RegL2T_2); lambda < 0 passes []; outs receives
 * lCurveErrImg, lCurveErrReg, lCurveErrReg_2, numel(err), sum(t). */
int drv_l2(uint64_t h, const double *data, size_t n, int num_iter, double lambdaL2,
           const char *reg, double lambdaL2_2, const char *reg2, double *rec, size_t n_rec,
           double *outs, char *msg, int msglen) {
    std::vector<mxArray *> in = {
        uint64_scalar(h), doubles(data, (mwSize)n, 1), mxCreateDoubleScalar(num_iter),
        lambdaL2 < 0 ? mxCreateDoubleMatrix(0, 0, mxREAL) : mxCreateDoubleScalar(lambdaL2),
        reg_arg(reg), reg_arg(reg),
        lambdaL2_2 < 0 ? mxCreateDoubleMatrix(0, 0, mxREAL) : mxCreateDoubleScalar(lambdaL2_2),
        reg_arg(reg2), reg_arg(reg2)};
    mxArray *o[6] = {};
    if (call(gw_rec_nn_with_L2_reg, 6, o, in, msg, msglen)) return 1;
    std::memcpy(rec, mxGetDoubles(o[0]), n_rec * sizeof(double));
    outs[0] = mxGetScalar(o[1]);
    outs[1] = mxGetScalar(o[2]);
    outs[2] = mxGetScalar(o[3]);
    outs[3] = (double)mxGetNumberOfElements(o[4]);
    double ts = 0;
    for (mwSize k = 0; k < mxGetNumberOfElements(o[5]); ++k) ts += mxGetDoubles(o[5])[k];
    outs[4] = ts;
    for (mxArray *a : o) mxDestroyArray(a);
    return 0;
}

/* rec_nn_with_L1_eye_reg (which = 1) or rec_nn_with_TV_reg (which = 2);
 * outs receives lCurveErrImg, lCurveErrReg, numel(err). */
int drv_l1_tv(int which, uint64_t h, const double *data, size_t n, int num_iter, double reg,
              double *rec, size_t n_rec, double *outs, char *msg, int msglen) {
    std::vector<mxArray *> in = {uint64_scalar(h), doubles(data, (mwSize)n, 1),
                                 mxCreateDoubleScalar(num_iter), mxCreateDoubleScalar(reg)};
    mxArray *o[5] = {};
    if (call(which == 1 ? gw_rec_nn_with_L1_eye_reg : gw_rec_nn_with_TV_reg, 5, o, in, msg,
             msglen))
        return 1;
    std::memcpy(rec, mxGetDoubles(o[0]), n_rec * sizeof(double));
    outs[0] = mxGetScalar(o[1]);
    outs[1] = mxGetScalar(o[2]);
    outs[2] = (double)mxGetNumberOfElements(o[3]);
    for (mxArray *a : o) mxDestroyArray(a);
    return 0;
}

/* Calls that fail before any device work: the model gateway with an
 * unknown command (case 0) or a model struct lacking Data (case 1), a
 * solver with a double as the model (case 2) or a handle that is not a live
 * plan (case 3); msg receives the error. */
int drv_error_case(int which, char *msg, int msglen) {
    std::vector<mxArray *> in;
    mxArray *o[6] = {};
    mexfn f = gw_msot_model_mex;
    switch (which) {
        case 0:
            in = {mxCreateString("bogus")};
            break;
        case 1: {
            const char *names[] = {"Probe"};
            in = {mxCreateString("create"), mxCreateStructMatrix(1, 1, 1, names)};
            break;
        }
        case 2:
            f = gw_rec_nn_with_L2_reg;
            in = {mxCreateDoubleScalar(1.0), mxCreateDoubleScalar(0.0), mxCreateDoubleScalar(5)};
            break;
        default:
            f = gw_rec_nn_with_L1_eye_reg;
            in = {uint64_scalar(0x1234), mxCreateDoubleScalar(0.0), mxCreateDoubleScalar(5),
                  mxCreateDoubleScalar(1e-3)};
            break;
    }
    return call(f, 6, o, in, msg, msglen);
}

int drv_lock_count(void) { return mex_shim_lock_count(); }

}  // extern "C"
