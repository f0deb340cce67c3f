/*
 * rec_nn_with_L2_reg.cpp -- MEX gateway with the signature of the
 * reference's rec_nn_with_L2_reg (rec_nn_with_L2_reg.m:1):
 *   [rec_img, lCurveErrImg, lCurveErrReg, lCurveErrReg_2, err, t] =
 *       rec_nn_with_L2_reg(model, data_filt, num_iter_nn_outer, lambdaL2, RegL2,
 *                          RegL2T, lambdaL2_2, RegL2_2, RegL2T_2)
 * model: the GPU model of msot_model_mex('create', ...).  data_filt:
 * T x D x W double, one reference call (the wavelengths coupled).  The GPU
 * solver implements the regularisers of the reference's overview script:
 * RegL2 = RegL2T = @(x) x and RegL2_2 = RegL2T_2 = a handle calling
 * laplacian_per_wavelength; any other handle raises
 * rec_nn_with_L2_reg:regularizer.  As in
 * incorporate_l2_reg_into_model_functions.m:5-22 a term enters only with a
 * positive weight, and the Laplacian only together with lambdaL2 > 0.
 * lCurveErrReg / lCurveErrReg_2 are ||RegL2(rec)||^2 / ||RegL2_2(rec)||^2
 * when the handle is given, else 0 (rec_nn_with_L2_reg.m:52-62); err is
 * zeros(num_iter, 1) and t the mean time per outer iteration.
 *
 * Build (MATLAB): mex -R2018a rec_nn_with_L2_reg.cpp -I<repo>/include \
 *                     -L<repo>/mb-rec-msot_gb300/lib -lmsotgpu
 */
#include <chrono>

#include "msot_mex_model.h"

static const char *kWho = "rec_nn_with_L2_reg";

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]) {
    if (nrhs < 3)
        mexErrMsgIdAndTxt("rec_nn_with_L2_reg:nrhs",
                          "rec_nn_with_L2_reg(model, data_filt, num_iter_nn_outer, ...) needs at "
                          "least 3 inputs.");
    msot_plan_t plan = msot_mex_plan(prhs[0], kWho);
    int nx, nz, D, T;
    const int W = msot_mex_wavelengths(prhs[1], plan, kWho, &nx, &nz, &D, &T);
    const int num_iter = (int)mxGetScalar(prhs[2]);
    const double lambdaL2 = msot_mex_scalar_or(nrhs, prhs, 3, 0.0);
    const double lambdaL2_2 = msot_mex_scalar_or(nrhs, prhs, 6, 0.0);
    const msot_reg_kind r1 = msot_mex_reg_kind(nrhs, prhs, 4), r1t = msot_mex_reg_kind(nrhs, prhs, 5);
    const msot_reg_kind r2 = msot_mex_reg_kind(nrhs, prhs, 7), r2t = msot_mex_reg_kind(nrhs, prhs, 8);
    const bool add1 = lambdaL2 > 0.0, add2 = add1 && lambdaL2_2 > 0.0;
    if ((add1 && (r1 != MSOT_REG_IDENTITY || r1t != MSOT_REG_IDENTITY)) || r1 == MSOT_REG_OTHER)
        mexErrMsgIdAndTxt("rec_nn_with_L2_reg:regularizer",
                          "the GPU solver takes RegL2 = RegL2T = @(x) x.");
    if ((add2 && (r2 != MSOT_REG_LAPLACIAN || r2t != MSOT_REG_LAPLACIAN)) ||
        r2 == MSOT_REG_OTHER)
        mexErrMsgIdAndTxt("rec_nn_with_L2_reg:regularizer",
                          "the GPU solver takes RegL2_2 = RegL2T_2 = laplacian_per_wavelength.");
    if (num_iter < 0)
        mexErrMsgIdAndTxt("rec_nn_with_L2_reg:input", "num_iter_nn_outer must be >= 0.");
    plhs[0] = msot_mex_image_stack(nx, nz, W);
    double e_img = 0, e_reg = 0, e_reg2 = 0;
    const auto t0 = std::chrono::steady_clock::now();
    const int rc = msot_host_rec_nn_with_L2_reg(
        plan, mxGetDoubles(prhs[1]), W, num_iter, add1 ? lambdaL2 : 0.0, add2 ? lambdaL2_2 : 0.0,
        mxGetDoubles(plhs[0]), &e_img, r1 == MSOT_REG_IDENTITY ? &e_reg : nullptr,
        r2 == MSOT_REG_LAPLACIAN ? &e_reg2 : nullptr);
    const double sec =
        std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (rc != MSOT_OK) mexErrMsgIdAndTxt("rec_nn_with_L2_reg:gpu", "%s", msot_last_error());
    if (nlhs > 1) plhs[1] = mxCreateDoubleScalar(e_img);
    if (nlhs > 2) plhs[2] = mxCreateDoubleScalar(e_reg);
    if (nlhs > 3) plhs[3] = mxCreateDoubleScalar(e_reg2);
    msot_mex_iter_outputs(nlhs, plhs, 4, num_iter, sec);
}
