// mex_api.cu -- host-buffer entry points with the contracts of the
// reference's four operator MEX functions (FP64 column-major in and out;
// forwardDelayAndSumMex.cpp:17-65, transposeDelayAndSumMex.cpp:17-61,
// forwardMex.cpp:18-85, transposeMex.cpp:18-82).  Each call builds a
// temporary plan from the given tables, moves the data to the GPU, runs the
// FP32 kernels and writes the FP64 result into caller memory, as the MEX
// boundary has no state that outlives a call.  Differences from the
// reference: inputs are range-checked (MSOT_ERANGE instead of out-of-bounds
// accesses) and the arithmetic is FP32.
#include <cmath>
#include <vector>

#include "common.cuh"

using namespace msot;

namespace {

// Grid shape used for the pixel patches when only P is known: any
// factorisation gives the same result; a near-square one keeps patches compact.
void factor_grid(int P, int &nx, int &nz) {
    nz = 1;
    for (int d = 1; (long)d * d <= P; ++d)
        if (P % d == 0) nz = d;
    nx = P / nz;
}

struct DevBuf {
    void *p = nullptr;
    ~DevBuf() {
        if (p) cudaFree(p);
    }
};

struct PlanGuard {
    msot_plan_t h = nullptr;
    ~PlanGuard() { msot_plan_destroy(h); }
};

int run_mex(bool forward, const double *in, int W, int P, int D, int T, const double *travel,
            double radius, const int32_t *sir_idx, const double *sir, int S, int NS,
            const int32_t *start_end, double *out) {
    if (!in || !travel || !out || W <= 0 || P <= 0 || D <= 0 || T <= 1) {
        set_error("mex: bad arguments");
        return MSOT_EINVAL;
    }
    msot_plan_desc d{};
    factor_grid(P, d.nx, d.nz);
    d.n_det = D;
    d.n_t = T;
    d.radius = radius;
    d.travel = travel;
    d.norm = 1.0;
    d.max_batch = W;
    if (sir) {
        d.sir_len = S;
        d.n_sir = NS;
        d.sir = sir;
        d.sir_start_end = start_end;
        d.sir_idx = sir_idx;
    }
    PlanGuard pg;
    int rc = msot_plan_create(&d, &pg.h);
    if (rc) return rc;
    const Plan &pl = pg.h->p;
    // the plan's grid is nx x nz with p = ix*nz + iz == the MEX pixel index
    const size_t NI = (size_t)W * P, NS_ = (size_t)W * D * T;
    DevBuf dimg, dsino;
    MSOT_CUDA_TRY(cudaMalloc(&dimg.p, NI * sizeof(float)));
    MSOT_CUDA_TRY(cudaMalloc(&dsino.p, NS_ * sizeof(float)));
    cudaStream_t st = 0;
    if (forward) {
        std::vector<float> h(NI);  // MATLAB W x P (w fastest) -> [W][P]
        for (int p = 0; p < P; ++p)
            for (int w = 0; w < W; ++w) h[(size_t)w * P + p] = (float)in[(size_t)p * W + w];
        MSOT_CUDA_TRY(cudaMemcpy(dimg.p, h.data(), NI * sizeof(float), cudaMemcpyHostToDevice));
        if ((rc = pl.S ? launch_permute(pl, (float *)dimg.p, pl.scr_img1, W, st)
                       : launch_to_pixmajor(pl, (float *)dimg.p, pl.scr_img1, W, st)))
            return rc;
        if ((rc = interp_forward(pl, pl.scr_img1, (float *)dsino.p, W, 1.f, st))) return rc;
        std::vector<float> o(NS_);
        MSOT_CUDA_TRY(cudaMemcpy(o.data(), dsino.p, NS_ * sizeof(float), cudaMemcpyDeviceToHost));
        // [W][D][T] -> MATLAB W x T x D
        for (int det = 0; det < D; ++det)
            for (int t = 0; t < T; ++t)
                for (int w = 0; w < W; ++w)
                    out[((size_t)det * T + t) * W + w] = o[((size_t)w * D + det) * T + t];
    } else {
        std::vector<float> h(NS_);  // MATLAB W x T x D -> [W][D][T]
        for (int det = 0; det < D; ++det)
            for (int t = 0; t < T; ++t)
                for (int w = 0; w < W; ++w)
                    h[((size_t)w * D + det) * T + t] = (float)in[((size_t)det * T + t) * W + w];
        MSOT_CUDA_TRY(
            cudaMemcpy(dsino.p, h.data(), NS_ * sizeof(float), cudaMemcpyHostToDevice));
        if ((rc = interp_adjoint(pl, (float *)dsino.p, (float *)dimg.p, W, 1.f, st))) return rc;
        std::vector<float> o(NI);
        MSOT_CUDA_TRY(cudaMemcpy(o.data(), dimg.p, NI * sizeof(float), cudaMemcpyDeviceToHost));
        for (int p = 0; p < P; ++p)
            for (int w = 0; w < W; ++w) out[(size_t)p * W + w] = o[(size_t)w * P + p];
    }
    return MSOT_OK;
}

}  // namespace

extern "C" {

int msot_mex_forwardDelayAndSum(const double *image, int W, int P, const double *travel, int D,
                                int T, double radius, double *out) {
    return run_mex(true, image, W, P, D, T, travel, radius, nullptr, nullptr, 0, 0, nullptr,
                   out);
}

int msot_mex_transposeDelayAndSum(const double *sig, int W, int T, int D, const double *travel,
                                  int P, double radius, double *out) {
    return run_mex(false, sig, W, P, D, T, travel, radius, nullptr, nullptr, 0, 0, nullptr,
                   out);
}

int msot_mex_forward(const double *image, int W, int P, const int32_t *sir_idx,
                     const double *travel, int D, const double *sir, int S, int NS, int T,
                     const int32_t *start_end, double radius, double *out) {
    if (!sir || !sir_idx || !start_end) {
        set_error("mex forward: missing SIR tables");
        return MSOT_EINVAL;
    }
    return run_mex(true, image, W, P, D, T, travel, radius, sir_idx, sir, S, NS, start_end,
                   out);
}

int msot_mex_transpose(const double *sig, int W, int T, int D, const int32_t *sir_idx,
                       const double *travel, int P, const double *sir, int S, int NS,
                       const int32_t *start_end, double radius, double *out) {
    if (!sir || !sir_idx || !start_end) {
        set_error("mex transpose: missing SIR tables");
        return MSOT_EINVAL;
    }
    return run_mex(false, sig, W, P, D, T, travel, radius, sir_idx, sir, S, NS, start_end, out);
}

}  // extern "C"
