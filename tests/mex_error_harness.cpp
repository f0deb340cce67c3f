/*
 * mex_error_harness.cpp -- test driver for the MEX gateways' input checks.
 *
 * Calls each of the four gateways (compiled with -DmexFunction=gw_<name>)
 * and, when built with -DWITH_REF, the reference's own mexFunction of the
 * same name (compiled into the oracle's reference library as
 * ref_<name>_mex), once per input with that one input of the wrong class,
 * and prints one line per call:
 *     <gw|ref> <name> <input index> <error id>|<message>
 * Only the class checks run: every call stops at the wrong input, before
 * any arithmetic or device work.  Built against the project's MEX stand-in
 * header, whose mexErrMsgIdAndTxt throws mex_shim_error.
 */
#include "mex.h"

#include <cstdint>
#include <cstdio>
#include <vector>

typedef void (*mexfn)(int, mxArray *[], int, const mxArray *[]);

void gw_forwardDelayAndSumMex(int, mxArray *[], int, const mxArray *[]);
void gw_transposeDelayAndSumMex(int, mxArray *[], int, const mxArray *[]);
void gw_forwardMex(int, mxArray *[], int, const mxArray *[]);
void gw_transposeMex(int, mxArray *[], int, const mxArray *[]);
#ifdef WITH_REF
void ref_forwardDelayAndSumMex_mex(int, mxArray *[], int, const mxArray *[]);
void ref_transposeDelayAndSumMex_mex(int, mxArray *[], int, const mxArray *[]);
void ref_forwardMex_mex(int, mxArray *[], int, const mxArray *[]);
void ref_transposeMex_mex(int, mxArray *[], int, const mxArray *[]);
#endif

struct Case {
    const char *name;
    const char *classes;  // 'd' double, 'i' int32, in argument order
    mexfn gw;
    mexfn ref;
};

static void run(const char *who, const Case &c, mexfn f, int wrong, int nrhs) {
    double dval[8] = {1, 1, 1, 1, 1, 1, 1, 1};
    int32_t ival[8] = {1, 1, 1, 1, 1, 1, 1, 1};
    const mwSize one[2] = {1, 1};
    std::vector<mxArray> arrs;
    const int n = (int)std::strlen(c.classes);
    for (int k = 0; k < n; ++k) {
        bool is_int = c.classes[k] == 'i';
        if (k == wrong) is_int = !is_int;
        arrs.push_back(is_int ? mx_wrap(mxINT32_CLASS, &ival[k], 2, one)
                              : mx_wrap(mxDOUBLE_CLASS, &dval[k], 2, one));
    }
    std::vector<const mxArray *> prhs;
    for (auto &a : arrs) prhs.push_back(&a);
    mxArray *plhs[1] = {nullptr};
    try {
        f(1, plhs, nrhs, prhs.data());
        std::printf("%s %s %d NONE|\n", who, c.name, wrong);
    } catch (const mex_shim_error &e) {
        std::printf("%s %s %d %s|%s\n", who, c.name, wrong, e.id.c_str(), e.what());
    }
    if (plhs[0]) mxDestroyArray(plhs[0]);
}

int main() {
#ifdef WITH_REF
#define REF(x) x
#else
#define REF(x) nullptr
#endif
    const Case cases[] = {
        {"forwardDelayAndSumMex", "ddid", gw_forwardDelayAndSumMex,
         REF(ref_forwardDelayAndSumMex_mex)},
        {"transposeDelayAndSumMex", "ddd", gw_transposeDelayAndSumMex,
         REF(ref_transposeDelayAndSumMex_mex)},
        {"forwardMex", "diddiid", gw_forwardMex, REF(ref_forwardMex_mex)},
        {"transposeMex", "diddid", gw_transposeMex, REF(ref_transposeMex_mex)},
    };
    for (const Case &c : cases) {
        const int n = (int)std::strlen(c.classes);
        for (int k = 0; k < n; ++k) {
            run("gw", c, c.gw, k, n);
            if (c.ref) run("ref", c, c.ref, k, n);
        }
        run("gw", c, c.gw, -1, n - 1);  // one input too few
    }
    return 0;
}
