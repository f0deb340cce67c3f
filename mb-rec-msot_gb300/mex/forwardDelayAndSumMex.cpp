/*
 * forwardDelayAndSumMex.cpp -- MEX gateway with the contract of the
 * reference's forwardDelayAndSumMex (forwardDelayAndSumMex.cpp:15-65):
 *   sinogram = forwardDelayAndSumMex(image, travelTimes, int32(numTimesteps), radius)
 * image: W x P double, travelTimes: P x D double -> W x T x D double.
 * Build (MATLAB):  mex -R2018a forwardDelayAndSumMex.cpp -I<repo>/include \
 *                      -L<repo>/mb-rec-msot_gb300/lib -lmsotgpu
 * The arithmetic runs on the GPU (libmsotgpu.so, FP32).
 */
#include "mex.h"
#include "msot_gpu.h"
#include "msot_mex_inputs.h"

static const msot_mex_input kInputs[] = {
    {false, "image"}, {false, "travelTimes"}, {true, "numTimesteps"},
    {false, "circularInterpolationRadiusInSamples"}};

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]) {
    msot_mex_check_inputs(nrhs, prhs, kInputs, 4);
    const int W = (int)mxGetM(prhs[0]), P = (int)mxGetN(prhs[0]);
    const int D = (int)mxGetN(prhs[1]);
    const int T = (int)mxGetScalar(prhs[2]);
    const mwSize dims[3] = {(mwSize)W, (mwSize)T, (mwSize)D};
    plhs[0] = mxCreateNumericArray(3, dims, mxDOUBLE_CLASS, mxREAL);
    const int rc = msot_mex_forwardDelayAndSum(mxGetDoubles(prhs[0]), W, P, mxGetDoubles(prhs[1]),
                                               D, T, mxGetScalar(prhs[3]),
                                               mxGetDoubles(plhs[0]));
    if (rc != MSOT_OK) mexErrMsgIdAndTxt("forwardMex:gpu", "%s", msot_last_error());
}
