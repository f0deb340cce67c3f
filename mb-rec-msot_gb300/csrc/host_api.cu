// host_api.cu -- host-buffer entry points of the MATLAB-level drop-in: a plan
// built from the fields of the reference's model object (MSOTmodel.m:18-48,
// Discretization.m:41-51), model.Funcs.applyForward / applyTranspose
// (MSOTmodel.m:285-286) and the three solvers (rec_nn_with_L2_reg.m:1,
// rec_nn_with_L1_eye_reg.m:1, rec_nn_with_TV_reg.m:1) on FP64 arrays in
// MATLAB's memory layout.  A multi-wavelength stack is one reference call:
// the solvers run coupled (shared scalars) and the l-curve values are sums
// over the stack, as the reference's norms over data_filt(:) are.  The MEX
// gateways in mex/ are thin wrappers over these functions.
#include <cmath>
#include <complex>
#include <vector>

#include "common.cuh"

using namespace msot;

namespace {

constexpr double kTwoPi = 6.283185307179586476925286766559;

struct DevMem {
    void *p = nullptr;
    ~DevMem() {
        if (p) cudaFree(p);
    }
};

struct PlanGuard {
    msot_plan_t h = nullptr;
    ~PlanGuard() {
        if (h) msot_plan_destroy(h);
    }
};

// ir[k] = Re (1/N) sum_f IRHat[f] e^{2 pi i f k / N}, k < L: the taps whose
// length-N transform the reference stores (MSOTmodel.m:338-346); the samples
// past L must vanish, else the transform is not of an L-tap IR
int taps_from_ir_hat(const double *hat, int N, int L, std::vector<double> &ir) {
    if (N < L || L < 1 || L % 2 == 0) {
        set_error("model: IRHat has %d entries for an eirLength of %d (odd, <= entries)", N, L);
        return MSOT_EINVAL;
    }
    std::vector<double> full(N);
    double peak = 0;
    for (int k = 0; k < N; ++k) {
        double acc = 0;
        for (int f = 0; f < N; ++f) {
            const double a = kTwoPi * (double)(((long long)f * k) % N) / N;
            acc += hat[2 * f] * std::cos(a) - hat[2 * f + 1] * std::sin(a);
        }
        full[k] = acc / N;
        peak = std::max(peak, std::fabs(full[k]));
    }
    for (int k = L; k < N; ++k)
        if (std::fabs(full[k]) > 1e-9 * peak) {
            set_error("model: IRHat is not the transform of an eirLength = %d tap IR", L);
            return MSOT_EINVAL;
        }
    ir.assign(full.begin(), full.begin() + L);
    return MSOT_OK;
}

// 1-D inverse DFT (real part) of n complex values
void idft_real(const std::vector<std::complex<double>> &in, std::vector<double> &out) {
    const int n = (int)in.size();
    out.assign(n, 0.0);
    for (int k = 0; k < n; ++k) {
        double acc = 0;
        for (int f = 0; f < n; ++f) {
            const double a = kTwoPi * (double)(((long long)f * k) % n) / n;
            acc += in[f].real() * std::cos(a) - in[f].imag() * std::sin(a);
        }
        out[k] = acc / n;
    }
}

// centred circular taps of one axis: kernel values at offsets -K .. K, K the
// largest offset whose value is above tol of the centre (at most kmax)
void centred_taps(const std::vector<double> &kern, double tol, int kmax,
                  std::vector<double> &taps) {
    const int n = (int)kern.size();
    int K = 0;
    for (int k = 1; k <= (n - 1) / 2; ++k)
        if (std::fabs(kern[k]) > tol * std::fabs(kern[0]) ||
            std::fabs(kern[n - k]) > tol * std::fabs(kern[0]))
            K = k;
    K = std::min(K, kmax);
    taps.resize(2 * K + 1);
    for (int k = -K; k <= K; ++k) taps[K + k] = kern[((k % n) + n) % n];
}

// The reference's prefilter (Discretization.m:47-51, shift_inv_proj.m:67-71)
// is the 2-D transform of a kernel that factors into one circular kernel per
// axis for the Gaussian pixel model: kernel(z, x) = kz(z) kx(x).  Row and
// column 0 of the kernel give the factors (kz scaled by 1 / kernel(0, 0)).
int taps_from_prefilter(const double *pre, int nz, int nx, std::vector<double> &tx,
                        std::vector<double> &tz) {
    // column 0 (x = 0): (1/nz) sum_fz e^{..} (1/nx) sum_fx P[fz, fx]
    std::vector<std::complex<double>> cz(nz), cx(nx);
    for (int fz = 0; fz < nz; ++fz) {
        std::complex<double> s = 0;
        for (int fx = 0; fx < nx; ++fx) {
            const size_t i = (size_t)fz + (size_t)nz * fx;  // column-major nz x nx
            s += std::complex<double>(pre[2 * i], pre[2 * i + 1]);
        }
        cz[fz] = s / (double)nx;
    }
    for (int fx = 0; fx < nx; ++fx) {
        std::complex<double> s = 0;
        for (int fz = 0; fz < nz; ++fz) {
            const size_t i = (size_t)fz + (size_t)nz * fx;
            s += std::complex<double>(pre[2 * i], pre[2 * i + 1]);
        }
        cx[fx] = s / (double)nz;
    }
    std::vector<double> kz, kx;
    idft_real(cz, kz);  // kernel(z, 0) = kz(z) kx(0)
    idft_real(cx, kx);  // kernel(0, x) = kz(0) kx(x)
    const double k00 = kz[0];
    if (!(std::fabs(k00) > 0) || !std::isfinite(k00)) {
        set_error("model: prefilter kernel has no centre value");
        return MSOT_EINVAL;
    }
    for (double &v : kz) v /= k00;  // kz(z) kx(0) / (kz(0) kx(0)) = kz(z) / kz(0)
    // kx(x) kz(0) stays: the product of the two factors is the kernel
    centred_taps(kx, 1e-13, 64, tx);
    centred_taps(kz, 1e-13, 64, tz);
    return MSOT_OK;
}

int device_copy_in(DevMem &d, const double *src, size_t n) {
    std::vector<float> h(n);
    for (size_t i = 0; i < n; ++i) h[i] = (float)src[i];
    MSOT_CUDA_TRY(cudaMalloc(&d.p, std::max<size_t>(1, n) * sizeof(float)));
    MSOT_CUDA_TRY(cudaMemcpy(d.p, h.data(), n * sizeof(float), cudaMemcpyHostToDevice));
    return MSOT_OK;
}

int device_copy_out(const DevMem &d, double *dst, size_t n) {
    std::vector<float> h(n);
    MSOT_CUDA_TRY(cudaMemcpy(h.data(), d.p, n * sizeof(float), cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < n; ++i) dst[i] = h[i];
    return MSOT_OK;
}

int check_host_call(msot_plan_t plan, const void *a, const void *b, int W, const char *who) {
    if (!msot_plan_valid(plan)) {
        set_error("%s: not a live plan handle", who);
        return MSOT_EINVAL;
    }
    if (!a || !b || W <= 0) {
        set_error("%s: null array or no wavelengths", who);
        return MSOT_EINVAL;
    }
    if (W > plan->p.max_batch) {
        set_error("%s: %d wavelengths exceed the plan's max_batch %d", who, W, plan->p.max_batch);
        return MSOT_EINVAL;
    }
    return check_plan_device(plan->p, who);
}

}  // namespace

extern "C" {

int msot_plan_create_from_model(const msot_model_fields *m, msot_plan_t *out) {
    if (!out || !m || !m->travel || m->nx <= 0 || m->nz <= 0 || m->n_det <= 0 || m->n_t <= 1) {
        set_error("model: bad grid / detector / sample counts or missing travel table");
        return MSOT_EINVAL;
    }
    *out = nullptr;
    std::vector<double> ir, tx, tz;
    int rc;
    if (m->ir_hat && (rc = taps_from_ir_hat(m->ir_hat, m->n_hat, m->eir_length, ir))) return rc;
    if (m->prefilter && (rc = taps_from_prefilter(m->prefilter, m->nz, m->nx, tx, tz))) return rc;
    msot_plan_desc d{};
    d.nx = m->nx;
    d.nz = m->nz;
    d.n_det = m->n_det;
    d.n_t = m->n_t;
    d.radius = m->radius;
    d.travel = m->travel;
    d.ir_len = (int)ir.size();
    d.ir = ir.empty() ? nullptr : ir.data();
    d.pre_len_x = (int)tx.size();
    d.pre_len_z = (int)tz.size();
    d.pre_x = tx.empty() ? nullptr : tx.data();
    d.pre_z = tz.empty() ? nullptr : tz.data();
    d.sir_len = m->sir_len;
    d.n_sir = m->n_sir;
    d.sir = m->sir;
    d.sir_start_end = m->sir_start_end;
    d.sir_idx = m->sir_idx;
    d.max_batch = m->max_batch > 0 ? m->max_batch : 1;
    double norm = m->norm;
    if (!(norm > 0)) {
        // the reference estimates sigma_max (svds) when no factor is given
        // (MSOTmodel.m:273-279); here by power iteration on an unnormalised plan
        d.norm = 1.0;
        PlanGuard g;
        if ((rc = msot_plan_create(&d, &g.h))) return rc;
        if ((rc = msot_estimate_norm(g.h, 100, 0, &norm, nullptr))) return rc;
    }
    d.norm = norm;
    return msot_plan_create(&d, out);
}

double msot_plan_norm(msot_plan_t plan) {
    return msot_plan_valid(plan) ? plan->p.norm : 0.0;
}

int msot_plan_shape(msot_plan_t plan, int *nx, int *nz, int *n_det, int *n_t, int *max_batch) {
    if (!msot_plan_valid(plan)) {
        set_error("plan_shape: not a live plan handle");
        return MSOT_EINVAL;
    }
    const Plan &pl = plan->p;
    if (nx) *nx = pl.nx;
    if (nz) *nz = pl.nz;
    if (n_det) *n_det = pl.D;
    if (n_t) *n_t = pl.T;
    if (max_batch) *max_batch = pl.max_batch;
    return MSOT_OK;
}

int msot_host_apply(msot_plan_t plan, int transpose, const double *in, int W, double *out) {
    int rc = check_host_call(plan, in, out, W, transpose ? "applyTranspose" : "applyForward");
    if (rc) return rc;
    const Plan &pl = plan->p;
    const size_t NI = (size_t)W * pl.P, NS = (size_t)W * pl.D * pl.T;
    DevMem a, b;
    // image Nz x Nx x W and sinogram T x D x W are [W][nx][nz] / [W][D][T]
    if ((rc = device_copy_in(a, in, transpose ? NS : NI))) return rc;
    MSOT_CUDA_TRY(cudaMalloc(&b.p, (transpose ? NI : NS) * sizeof(float)));
    rc = transpose ? msot_transpose(plan, (const float *)a.p, (float *)b.p, W, nullptr)
                   : msot_forward(plan, (const float *)a.p, (float *)b.p, W, nullptr);
    if (rc) return rc;
    return device_copy_out(b, out, transpose ? NI : NS);
}

int msot_host_rec_nn_with_L2_reg(msot_plan_t plan, const double *data, int W, int num_iter,
                                 double lambdaL2, double lambdaL2_2, double *rec,
                                 double *err_img, double *err_reg, double *err_reg2) {
    int rc = check_host_call(plan, data, rec, W, "rec_nn_with_L2_reg");
    if (rc) return rc;
    const Plan &pl = plan->p;
    const size_t NI = (size_t)W * pl.P, NS = (size_t)W * pl.D * pl.T;
    DevMem b, x;
    if ((rc = device_copy_in(b, data, NS))) return rc;
    MSOT_CUDA_TRY(cudaMalloc(&x.p, NI * sizeof(float)));
    std::vector<double> e1(W), e2(W), e3(W, 0.0);
    const bool two = lambdaL2 > 0 && lambdaL2_2 > 0;
    rc = two ? msot_rec_nn_with_L2_reg_2(plan, (const float *)b.p, (float *)x.p, W, num_iter,
                                         lambdaL2, lambdaL2_2, nullptr, 1, e1.data(), e2.data(),
                                         e3.data(), nullptr)
             : msot_rec_nn_with_L2_reg(plan, (const float *)b.p, (float *)x.p, W, num_iter,
                                       lambdaL2 > 0 ? lambdaL2 : 0.0, nullptr, 1, e1.data(),
                                       e2.data(), nullptr);
    if (rc) return rc;
    if (err_reg2 && !two) {
        // ||del2(rec)||^2 although the Laplacian did not enter the solve
        // (rec_nn_with_L2_reg.m:57-62 evaluates it whenever RegL2_2 is given)
        DevMem lap;
        MSOT_CUDA_TRY(cudaMalloc(&lap.p, NI * sizeof(float)));
        if ((rc = msot_laplacian_per_wavelength((const float *)x.p, (float *)lap.p, W, pl.nx,
                                                pl.nz, nullptr)))
            return rc;
        std::vector<double> h(NI);
        if ((rc = device_copy_out(lap, h.data(), NI))) return rc;
        double s = 0;
        for (double v : h) s += v * v;
        e3.assign(W, 0.0);
        e3[0] = s;
    }
    if ((rc = device_copy_out(x, rec, NI))) return rc;
    double s1 = 0, s3 = 0;
    for (int w = 0; w < W; ++w) s1 += e1[w], s3 += e3[w];
    if (err_img) *err_img = s1;
    if (err_reg) {
        // ||RegL2(rec)||^2 with RegL2 the identity, whatever lambdaL2
        // (rec_nn_with_L2_reg.m:52-56)
        double s2 = 0;
        for (size_t k = 0; k < NI; ++k) s2 += rec[k] * rec[k];
        *err_reg = s2;
    }
    if (err_reg2) *err_reg2 = s3;
    return MSOT_OK;
}

int msot_host_rec_nn_with_L1_eye_reg(msot_plan_t plan, const double *data, int W, int num_iter,
                                     double reg, double *rec, double *err_img,
                                     double *err_reg) {
    int rc = check_host_call(plan, data, rec, W, "rec_nn_with_L1_eye_reg");
    if (rc) return rc;
    const Plan &pl = plan->p;
    const size_t NI = (size_t)W * pl.P, NS = (size_t)W * pl.D * pl.T;
    DevMem b, x;
    if ((rc = device_copy_in(b, data, NS))) return rc;
    MSOT_CUDA_TRY(cudaMalloc(&x.p, NI * sizeof(float)));
    std::vector<double> e1(W), e2(W);
    if ((rc = msot_rec_nn_with_L1_eye_reg(plan, (const float *)b.p, (float *)x.p, W, num_iter,
                                          reg, nullptr, 1, e1.data(), e2.data(), nullptr)))
        return rc;
    if ((rc = device_copy_out(x, rec, NI))) return rc;
    double s1 = 0, s2 = 0;
    for (int w = 0; w < W; ++w) s1 += e1[w], s2 += e2[w];
    if (err_img) *err_img = s1;
    if (err_reg) *err_reg = s2;
    return MSOT_OK;
}

int msot_host_rec_nn_with_TV_reg(msot_plan_t plan, const double *data, int W, int num_iter,
                                 double reg, double *rec, double *err_img, double *err_reg) {
    int rc = check_host_call(plan, data, rec, W, "rec_nn_with_TV_reg");
    if (rc) return rc;
    const Plan &pl = plan->p;
    const size_t NI = (size_t)W * pl.P, NS = (size_t)W * pl.D * pl.T;
    DevMem b, x;
    if ((rc = device_copy_in(b, data, NS))) return rc;
    MSOT_CUDA_TRY(cudaMalloc(&x.p, NI * sizeof(float)));
    std::vector<double> e1(W), e2(W);
    if ((rc = msot_rec_nn_with_TV_reg(plan, (const float *)b.p, (float *)x.p, W, num_iter, reg,
                                      2, nullptr, 1, e1.data(), e2.data(), nullptr)))
        return rc;
    if ((rc = device_copy_out(x, rec, NI))) return rc;
    double s1 = 0, s2 = 0;
    for (int w = 0; w < W; ++w) s1 += e1[w], s2 += e2[w];
    if (err_img) *err_img = s1;
    if (err_reg) *err_reg = s2;
    return MSOT_OK;
}

}  // extern "C"
