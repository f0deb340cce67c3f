/*
 * msot_mex_inputs.h -- input checks shared by the four MEX gateways.
 *
 * The reference's operator MEX files test their inputs in argument order and
 * stop at the first one of the wrong class, with one error ID per class and a
 * message naming the input (forwardMex.cpp:30-50, transposeMex.cpp:30-47,
 * forwardDelayAndSumMex.cpp:27-38, transposeDelayAndSumMex.cpp:26-34; all four
 * use the "forwardMex:" prefix).  A MATLAB caller that matches on those IDs or
 * messages sees the same errors from these gateways.  The reference reads its
 * inputs without checking their count; here fewer inputs than the contract
 * names raise forwardMex:nrhs, and extra inputs are ignored as there.
 */
#ifndef MSOT_MEX_INPUTS_H
#define MSOT_MEX_INPUTS_H

#include "mex.h"

struct msot_mex_input {
    bool int32;        /* int32 expected (else real double) */
    const char *name;  /* the reference's name for the input */
};

static inline void msot_mex_check_inputs(int nrhs, const mxArray *prhs[],
                                         const msot_mex_input *want, int n) {
    if (nrhs < n) mexErrMsgIdAndTxt("forwardMex:nrhs", "%d inputs required.", n);
    for (int i = 0; i < n; ++i) {
        if (want[i].int32) {
            if (!mxIsInt32(prhs[i]))
                mexErrMsgIdAndTxt("forwardMex:notInt32", "%s must be type int32.", want[i].name);
        } else if (!mxIsDouble(prhs[i]) || mxIsComplex(prhs[i])) {
            mexErrMsgIdAndTxt("forwardMex:notDouble", "%s must be type double.", want[i].name);
        }
    }
}

#endif
