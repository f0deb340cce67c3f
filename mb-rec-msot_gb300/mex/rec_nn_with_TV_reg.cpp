/*
 * rec_nn_with_TV_reg.cpp -- MEX gateway with the signature of the
 * reference's rec_nn_with_TV_reg (rec_nn_with_TV_reg.m:1):
 *   [rec_img, lCurveErrImg, lCurveErrReg, err, t] =
 *       rec_nn_with_TV_reg(model, data_filt, num_iter, regParam)
 * model: the GPU model of msot_model_mex('create', ...).  data_filt:
 * T x D x W double, one reference call (the wavelengths coupled).
 * lCurveErrReg = the ITV summed over the wavelengths (PhiForTVReg.m:2-9).
 * Square grids only, as rec_nn_with_TV_reg.m:21-24 errors otherwise.  err is
 * zeros(num_iter, 1) and t the mean time per outer iteration.
 *
 * Build (MATLAB): mex -R2018a rec_nn_with_TV_reg.cpp -I<repo>/include \
 *                     -L<repo>/mb-rec-msot_gb300/lib -lmsotgpu
 */
#include <chrono>

#include "msot_mex_model.h"

static const char *kWho = "rec_nn_with_TV_reg";

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]) {
    if (nrhs < 4)
        mexErrMsgIdAndTxt("rec_nn_with_TV_reg:nrhs",
                          "rec_nn_with_TV_reg(model, data_filt, num_iter, regParam) needs 4 "
                          "inputs.");
    msot_plan_t plan = msot_mex_plan(prhs[0], kWho);
    int nx, nz, D, T;
    const int W = msot_mex_wavelengths(prhs[1], plan, kWho, &nx, &nz, &D, &T);
    const int num_iter = (int)mxGetScalar(prhs[2]);
    const double reg = mxGetScalar(prhs[3]);
    if (num_iter < 0)
        mexErrMsgIdAndTxt("rec_nn_with_TV_reg:input", "num_iter must be >= 0.");
    plhs[0] = msot_mex_image_stack(nx, nz, W);
    double e_img = 0, e_reg = 0;
    const auto t0 = std::chrono::steady_clock::now();
    const int rc = msot_host_rec_nn_with_TV_reg(plan, mxGetDoubles(prhs[1]), W, num_iter, reg,
                                                mxGetDoubles(plhs[0]), &e_img, &e_reg);
    const double sec =
        std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (rc != MSOT_OK) mexErrMsgIdAndTxt("rec_nn_with_TV_reg:gpu", "%s", msot_last_error());
    if (nlhs > 1) plhs[1] = mxCreateDoubleScalar(e_img);
    if (nlhs > 2) plhs[2] = mxCreateDoubleScalar(e_reg);
    msot_mex_iter_outputs(nlhs, plhs, 3, num_iter, sec);
}
