/*
 * transposeDelayAndSumMex.cpp -- MEX gateway with the contract of the
 * reference's transposeDelayAndSumMex (transposeDelayAndSumMex.cpp:15-61):
 *   image = transposeDelayAndSumMex(sigMat, travelTimes, radius)
 * sigMat: W x T x D double, travelTimes: P x D double -> W x P double.
 */
#include "mex.h"
#include "msot_gpu.h"
#include "msot_mex_inputs.h"

static const msot_mex_input kInputs[] = {
    {false, "sigMat"}, {false, "travelTimes"}, {false, "circularInterpolationRadiusInSamples"}};

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]) {
    msot_mex_check_inputs(nrhs, prhs, kInputs, 3);
    const int W = (int)mxGetM(prhs[0]);
    const int T = (int)mxGetDimensions(prhs[0])[1];
    const int P = (int)mxGetM(prhs[1]), D = (int)mxGetN(prhs[1]);
    plhs[0] = mxCreateDoubleMatrix(W, P, mxREAL);
    const int rc = msot_mex_transposeDelayAndSum(mxGetDoubles(prhs[0]), W, T, D,
                                                 mxGetDoubles(prhs[1]), P, mxGetScalar(prhs[2]),
                                                 mxGetDoubles(plhs[0]));
    if (rc != MSOT_OK) mexErrMsgIdAndTxt("forwardMex:gpu", "%s", msot_last_error());
}
