/*
 * transposeMex.cpp -- MEX gateway with the contract of the reference's
 * transposeMex (transposeMex.cpp:16-82), the SIR transpose:
 *   image = transposeMex(sigMat, sirIndices, travelTimes, sir, sirStartEnd, radius)
 */
#include "mex.h"
#include "msot_gpu.h"
#include "msot_mex_inputs.h"

static const msot_mex_input kInputs[] = {
    {false, "sigMat"}, {true, "sirIndices"}, {false, "travelTimes"}, {false, "sir"},
    {true, "sirTimestepsStartAndEnd"}, {false, "circularInterpolationRadiusInSamples"}};

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]) {
    msot_mex_check_inputs(nrhs, prhs, kInputs, 6);
    const int W = (int)mxGetM(prhs[0]);
    const int T = (int)mxGetDimensions(prhs[0])[1];
    const int P = (int)mxGetM(prhs[1]), D = (int)mxGetN(prhs[1]);
    const int S = (int)mxGetM(prhs[3]), NS = (int)mxGetN(prhs[3]);
    plhs[0] = mxCreateDoubleMatrix(W, P, mxREAL);
    const int rc = msot_mex_transpose(mxGetDoubles(prhs[0]), W, T, D, mxGetInt32s(prhs[1]),
                                      mxGetDoubles(prhs[2]), P, mxGetDoubles(prhs[3]), S, NS,
                                      mxGetInt32s(prhs[4]), mxGetScalar(prhs[5]),
                                      mxGetDoubles(plhs[0]));
    if (rc != MSOT_OK) mexErrMsgIdAndTxt("forwardMex:gpu", "%s", msot_last_error());
}
