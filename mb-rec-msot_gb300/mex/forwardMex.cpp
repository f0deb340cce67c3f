/*
 * forwardMex.cpp -- MEX gateway with the contract of the reference's
 * forwardMex (forwardMex.cpp:16-85), the SIR forward operator:
 *   sino = forwardMex(image, sirIndices, travelTimes, sir, int32(T), sirStartEnd, radius)
 */
#include "mex.h"
#include "msot_gpu.h"
#include "msot_mex_inputs.h"

static const msot_mex_input kInputs[] = {
    {false, "image"}, {true, "sirIndices"}, {false, "travelTimes"}, {false, "sir"},
    {true, "numTimesteps"}, {true, "sirTimestepsStartAndEnd"},
    {false, "circularInterpolationRadiusInSamples"}};

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]) {
    msot_mex_check_inputs(nrhs, prhs, kInputs, 7);
    const int W = (int)mxGetM(prhs[0]), P = (int)mxGetN(prhs[0]);
    const int D = (int)mxGetN(prhs[1]);
    const int S = (int)mxGetM(prhs[3]), NS = (int)mxGetN(prhs[3]);
    const int T = (int)mxGetScalar(prhs[4]);
    const mwSize dims[3] = {(mwSize)W, (mwSize)T, (mwSize)D};
    plhs[0] = mxCreateNumericArray(3, dims, mxDOUBLE_CLASS, mxREAL);
    const int rc = msot_mex_forward(mxGetDoubles(prhs[0]), W, P, mxGetInt32s(prhs[1]),
                                    mxGetDoubles(prhs[2]), D, mxGetDoubles(prhs[3]), S, NS, T,
                                    mxGetInt32s(prhs[5]), mxGetScalar(prhs[6]),
                                    mxGetDoubles(plhs[0]));
    if (rc != MSOT_OK) mexErrMsgIdAndTxt("forwardMex:gpu", "%s", msot_last_error());
}
