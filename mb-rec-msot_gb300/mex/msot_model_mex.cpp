/*
 * msot_model_mex.cpp -- MEX gateway holding GPU models across calls: the
 * device-resident form of the reference's model object (MSOTmodel.m:18-48)
 * and its model.Funcs.applyForward / applyTranspose (MSOTmodel.m:285-286).
 *
 *   h = msot_model_mex('create', model, normalizationFactor, maxBatch)
 *       model: the reference's MSOTmodel (or a struct with its members):
 *         Data.absoluteTravelTimeIndices, circularInterpolationRadiusInSamples,
 *         numTimeSamplesPerTransducer, IRHat; Probe.eirLength;
 *         Discretization.sizeOfPixelGrid, prefilter; includeSir and, when
 *         true, Data.SPMR / SPMRIndices / SPMRTimestepIndexStartAndEnd.
 *       normalizationFactor: [] -> sigma_max estimated on the GPU (the
 *         reference runs svds, MSOTmodel.m:273-279); maxBatch: the largest
 *         wavelength stack per call (default 1).
 *       h: uint64 handle, valid until 'destroy'.  The MEX file stays locked
 *         (mexLock) while any handle is live.
 *   msot_model_mex('destroy', h)
 *   sig = msot_model_mex('applyForward', h, p0)     p0: Nz x Nx x W -> T x D x W
 *   img = msot_model_mex('applyTranspose', h, sig)  sig: T x D x W -> Nz x Nx x W
 *   s   = msot_model_mex('normalizationFactor', h)
 *
 * Build (MATLAB): mex -R2018a msot_model_mex.cpp -I<repo>/include \
 *                     -L<repo>/mb-rec-msot_gb300/lib -lmsotgpu
 */
#include <cstdint>
#include <set>
#include <string>
#include <vector>

#include "msot_mex_model.h"

static std::set<msot_plan_t> g_models;  // handles created here and not destroyed

static void destroy_all(void) {
    for (msot_plan_t p : g_models) msot_plan_destroy(p);
    g_models.clear();
}

static const char *kWho = "msot_model_mex";

static void fail(const char *what, const char *msg) {
    mexErrMsgIdAndTxt(msot_mex_id(kWho, what).c_str(), "%s", msg);
}

// interleaved complex copy of a double array (real arrays get zero imaginary parts)
static std::vector<double> complex_copy(const mxArray *a) {
    const size_t n = (size_t)mxGetNumberOfElements(a);
    std::vector<double> v(2 * n, 0.0);
    if (mxIsComplex(a)) {
        const mxComplexDouble *c = mxGetComplexDoubles(a);
        for (size_t i = 0; i < n; ++i) v[2 * i] = c[i].real, v[2 * i + 1] = c[i].imag;
    } else {
        const double *r = mxGetDoubles(a);
        for (size_t i = 0; i < n; ++i) v[2 * i] = r[i];
    }
    return v;
}

static void create(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]) {
    if (nrhs < 2) fail("nrhs", "msot_model_mex('create', model, [normalizationFactor], [maxBatch])");
    const mxArray *model = prhs[1];
    msot_mex_member data(model, "Data"), disc(model, "Discretization"), probe(model, "Probe");
    if (!data.a || !disc.a || !probe.a) fail("field", "model needs Data, Discretization and Probe.");
    msot_mex_member travel(data.a, "absoluteTravelTimeIndices");
    msot_mex_member radius(data.a, "circularInterpolationRadiusInSamples");
    msot_mex_member nt(data.a, "numTimeSamplesPerTransducer");
    msot_mex_member irhat(data.a, "IRHat");
    msot_mex_member grid(disc.a, "sizeOfPixelGrid");
    msot_mex_member pre(disc.a, "prefilter");
    msot_mex_member eirlen(probe.a, "eirLength");
    msot_mex_member sir_on(model, "includeSir");
    if (!travel.a || !mxIsDouble(travel.a) || mxIsComplex(travel.a))
        fail("field", "Data.absoluteTravelTimeIndices must be a real double P x D array.");
    if (!radius.a || !nt.a || !grid.a || mxGetNumberOfElements(grid.a) != 2 || !mxIsDouble(grid.a))
        fail("field", "model needs Data.circularInterpolationRadiusInSamples, "
                      "Data.numTimeSamplesPerTransducer and Discretization.sizeOfPixelGrid.");
    msot_model_fields f{};
    const double *g = mxGetDoubles(grid.a);
    f.nx = (int)g[0];
    f.nz = (int)g[1];
    f.n_t = (int)mxGetScalar(nt.a);
    f.radius = mxGetScalar(radius.a);
    const size_t P = (size_t)f.nx * f.nz;
    if (P == 0 || mxGetM(travel.a) != P)
        fail("field", "Data.absoluteTravelTimeIndices must have Nx * Nz rows.");
    f.n_det = (int)mxGetN(travel.a);
    f.travel = mxGetDoubles(travel.a);
    std::vector<double> ir_hat, prefilter;
    if (irhat.a && !mxIsEmpty(irhat.a)) {
        if (!mxIsDouble(irhat.a) || !eirlen.a)
            fail("field", "Data.IRHat must be double and Probe.eirLength given.");
        ir_hat = complex_copy(irhat.a);
        f.ir_hat = ir_hat.data();
        f.n_hat = (int)mxGetNumberOfElements(irhat.a);
        f.eir_length = (int)mxGetScalar(eirlen.a);
    }
    if (pre.a && !mxIsEmpty(pre.a)) {
        if (!mxIsDouble(pre.a) || (size_t)mxGetNumberOfElements(pre.a) != P)
            fail("field", "Discretization.prefilter must be a double Nz x Nx array.");
        prefilter = complex_copy(pre.a);
        f.prefilter = prefilter.data();
    }
    if (sir_on.a && mxGetScalar(sir_on.a) != 0.0) {
        msot_mex_member spmr(data.a, "SPMR"), idx(data.a, "SPMRIndices"),
            se(data.a, "SPMRTimestepIndexStartAndEnd");
        if (!spmr.a || !idx.a || !se.a || !mxIsDouble(spmr.a) || !mxIsInt32(idx.a) ||
            !mxIsInt32(se.a))
            fail("field", "includeSir needs Data.SPMR (double), SPMRIndices and "
                          "SPMRTimestepIndexStartAndEnd (int32).");
        f.sir_len = (int)mxGetM(spmr.a);
        f.n_sir = (int)mxGetN(spmr.a);
        f.sir = mxGetDoubles(spmr.a);
        f.sir_idx = mxGetInt32s(idx.a);
        f.sir_start_end = mxGetInt32s(se.a);
        if ((size_t)mxGetNumberOfElements(idx.a) != P * (size_t)f.n_det ||
            (size_t)mxGetNumberOfElements(se.a) != 2 * (size_t)f.n_sir)
            fail("field", "SPMRIndices must be P x D and SPMRTimestepIndexStartAndEnd 2 x NS.");
    }
    f.norm = msot_mex_scalar_or(nrhs, prhs, 2, 0.0);
    f.max_batch = (int)msot_mex_scalar_or(nrhs, prhs, 3, 1.0);
    msot_plan_t plan = nullptr;
    if (msot_plan_create_from_model(&f, &plan) != MSOT_OK) fail("gpu", msot_last_error());
    if (g_models.empty()) {
        mexLock();
        mexAtExit(destroy_all);
    }
    g_models.insert(plan);
    plhs[0] = mxCreateNumericMatrix(1, 1, mxUINT64_CLASS, mxREAL);
    mxGetUint64s(plhs[0])[0] = (uint64_t)(uintptr_t)plan;
    (void)nlhs;
}

static msot_plan_t own_handle(int nrhs, const mxArray *prhs[]) {
    if (nrhs < 2) fail("nrhs", "the command needs a model handle.");
    msot_plan_t p = msot_mex_plan(prhs[1], kWho);
    if (!g_models.count(p)) fail("model", "the handle was not created by this MEX file.");
    return p;
}

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]) {
    if (nrhs < 1 || !mxIsChar(prhs[0])) fail("command", "the first input must be a command name.");
    char *c = mxArrayToString(prhs[0]);
    const std::string cmd = c ? c : "";
    mxFree(c);
    if (cmd == "create") return create(nlhs, plhs, nrhs, prhs);
    if (cmd == "destroy") {
        msot_plan_t p = own_handle(nrhs, prhs);
        g_models.erase(p);
        msot_plan_destroy(p);
        if (g_models.empty()) mexUnlock();
        return;
    }
    if (cmd == "normalizationFactor") {
        plhs[0] = mxCreateDoubleScalar(msot_plan_norm(own_handle(nrhs, prhs)));
        return;
    }
    if (cmd == "applyForward" || cmd == "applyTranspose") {
        msot_plan_t p = own_handle(nrhs, prhs);
        if (nrhs < 3) fail("nrhs", "applyForward / applyTranspose need the data.");
        int nx = 0, nz = 0, D = 0, T = 0, mb = 0;
        msot_plan_shape(p, &nx, &nz, &D, &T, &mb);
        const bool tr = cmd == "applyTranspose";
        const size_t per = tr ? (size_t)D * T : (size_t)nx * nz;
        const size_t n = (size_t)mxGetNumberOfElements(prhs[2]);
        if (!mxIsDouble(prhs[2]) || mxIsComplex(prhs[2]) || n == 0 || n % per)
            fail("input", tr ? "applyTranspose takes a real double T x D x W array."
                             : "applyForward takes a real double Nz x Nx x W array.");
        const int W = (int)(n / per);
        if (W > mb) fail("input", "more wavelengths than the model's maxBatch.");
        if (tr) {
            plhs[0] = msot_mex_image_stack(nx, nz, W);
        } else {
            const mwSize d3[3] = {(mwSize)T, (mwSize)D, (mwSize)W};
            plhs[0] = mxCreateNumericArray(W > 1 ? 3 : 2, d3, mxDOUBLE_CLASS, mxREAL);
        }
        if (msot_host_apply(p, tr ? 1 : 0, mxGetDoubles(prhs[2]), W, mxGetDoubles(plhs[0])) !=
            MSOT_OK)
            fail("gpu", msot_last_error());
        return;
    }
    fail("command", "unknown command (create, destroy, applyForward, applyTranspose, "
                    "normalizationFactor).");
}
