// analytic.cu -- the reference's analytic reconstructors on the GPU.
//
//   msot_dmas_cf            <- reconstruction_backprojection/dmas_cf.m:19-107
//   msot_backproject_waveeq <- reconstruction_backprojection/backproject_waveeq.m:1-50
//
// Both index the sinogram at the nearest sample of the pixel-to-detector
// travel time, round((|x_p - x_d| / c - t_1) fs + 1) (dmas_cf.m:69-74,
// backproject_waveeq.m:36-41).  That index is computed in FP64 with every
// operation rounded separately (no contraction into FMA), so it rounds exactly
// as the FP64 reference does; an index outside the sinogram, where MATLAB
// raises an error, is reported as MSOT_ERANGE.  Sums over detectors are FP64.

#include <cmath>
#include <vector>

#include "common.cuh"

namespace msot {

// idx[d][p] = 0-based nearest sample index of pixel p for detector d
__global__ void k_nearest_index(const double *__restrict__ cosa, const double *__restrict__ sina,
                                const double *__restrict__ xv, const double *__restrict__ zv,
                                int nx, int nz, int D, double R, double c, double fs,
                                double acq1, int T, int32_t *__restrict__ idx, int *err) {
    const int P = nx * nz;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const int d = blockIdx.y;
    if (p >= P) return;
    const int ix = p / nz, iz = p - ix * nz;
    const double X = xv[ix], Z = zv[iz];
    const double dx = __dadd_rn(X, -__dmul_rn(cosa[d], R));
    const double dz = __dadd_rn(Z, -__dmul_rn(sina[d], R));
    const double dist = __dsqrt_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dz, dz)));
    const double v = __dadd_rn(__dmul_rn(__dadd_rn(__ddiv_rn(dist, c), -acq1), fs), 1.0);
    long i = (long)round(v) - 1;
    if (i < 0 || i >= T) {
        atomicOr(err, 1);
        i = i < 0 ? 0 : T - 1;
    }
    idx[(size_t)d * P + p] = (int32_t)i;
}

__global__ void k_max_abs(const float *__restrict__ x, size_t n, unsigned int *out) {
    float m = 0.f;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
        m = fmaxf(m, fabsf(x[i]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, __float_as_uint(m));  // m >= 0: order preserved
}

// dmas_cf.m:63-105: per pixel and wavelength the four detector sums
__global__ void k_dmas_cf(const float *__restrict__ sig, const int32_t *__restrict__ idx,
                          const unsigned int *__restrict__ maxbits, int P, int D, int T,
                          float *__restrict__ o_dmascf, float *__restrict__ o_dmas,
                          float *__restrict__ o_cf, float *__restrict__ o_das) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const int w = blockIdx.y;
    if (p >= P) return;
    const double inv = 1.0 / (double)__uint_as_float(*maxbits);
    const float *s = sig + (size_t)w * D * T;
    double sos = 0, sqs = 0, num = 0, den = 0;
    for (int d = 0; d < D; ++d) {
        const double v = (double)__ldg(s + (size_t)d * T + __ldg(idx + (size_t)d * P + p)) * inv;
        const double vs = copysign(sqrt(fabs(v)), v);
        sos += vs * vs;
        sqs += vs;
        num += v;
        den += v * v;
    }
    const double dmas = 0.5 * (sqs * sqs - sos);
    const double cf = num * num / (1e-6 + (double)D * den);
    const size_t o = (size_t)w * P + p;
    o_dmascf[o] = (float)(dmas * cf);
    o_dmas[o] = (float)dmas;
    o_cf[o] = (float)cf;
    o_das[o] = (float)num;
}

// backproject_waveeq.m:23-24: cumtrapz(t, sig / c) ./ t per column (FP64 running sum)
__global__ void k_cumtrapz(const float *__restrict__ sig, float *__restrict__ out, int cols,
                           int T, double c, double dt, double n_crop) {
    const int col = blockIdx.x * blockDim.x + threadIdx.x;
    if (col >= cols) return;
    const float *s = sig + (size_t)col * T;
    float *o = out + (size_t)col * T;
    double acc = 0.0, prev = (double)s[0] / c;
    o[0] = 0.f;
    for (int t = 1; t < T; ++t) {
        const double cur = (double)s[t] / c;
        acc += 0.5 * dt * (cur + prev);  // uniform times: t_k - t_{k-1} = dt
        prev = cur;
        o[t] = (float)(acc / ((t + 1 + n_crop) * dt));
    }
}

// backproject_waveeq.m:27: convn(sig, psf, 'same') / sum(psf) over (T, D) of
// each wavelength; psf is m (along T) x n (along D), column-major.
__global__ void k_psf_same(const float *__restrict__ in, float *__restrict__ out,
                           const double *__restrict__ psf, int m, int n, double inv_sum, int D,
                           int T) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int d = blockIdx.y, w = blockIdx.z;
    if (t >= T) return;
    const float *s = in + (size_t)w * D * T;
    const int om = m / 2, on = n / 2;
    double acc = 0.0;
    for (int b = 0; b < n; ++b) {
        const int dd = d + on - b;
        if (dd < 0 || dd >= D) continue;
        for (int a = 0; a < m; ++a) {
            const int tt = t + om - a;
            if (tt < 0 || tt >= T) continue;
            acc += psf[a + (size_t)b * m] * (double)s[(size_t)dd * T + tt];
        }
    }
    out[((size_t)w * D + d) * T + t] = (float)(acc * inv_sum);
}

// backproject_waveeq.m:35-47: nearest-sample gather into the vector field
__global__ void k_bp_gather(const float *__restrict__ y, const int32_t *__restrict__ idx,
                            const double *__restrict__ cosa, const double *__restrict__ sina,
                            int P, int D, int T, double dtc, double *__restrict__ fx,
                            double *__restrict__ fz) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const int w = blockIdx.y;
    if (p >= P) return;
    const float *s = y + (size_t)w * D * T;
    double ax = 0.0, az = 0.0;
    for (int d = 0; d < D; ++d) {
        const double v = (double)__ldg(s + (size_t)d * T + __ldg(idx + (size_t)d * P + p));
        ax += v * cosa[d] * dtc;
        az += v * sina[d] * dtc;
    }
    fx[(size_t)w * P + p] = ax;
    fz[(size_t)w * P + p] = az;
}

// backproject_waveeq.m:49: fliplr(divergence(fov_x, fov_y, fx, fz)); MATLAB
// gradient: central differences inside, one-sided at the borders.
__global__ void k_div_fliplr(const double *__restrict__ fx, const double *__restrict__ fz,
                             const double *__restrict__ xv, const double *__restrict__ zv,
                             int nx, int nz, float *__restrict__ out) {
    const int P = nx * nz;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const int w = blockIdx.y;
    if (p >= P) return;
    const int ix = p / nz, iz = p - ix * nz;
    const double *u = fx + (size_t)w * P, *v = fz + (size_t)w * P;
    double gx, gz;
    if (nx == 1) {
        gx = 0.0;
    } else if (ix == 0) {
        gx = (u[nz + iz] - u[iz]) / (xv[1] - xv[0]);
    } else if (ix == nx - 1) {
        gx = (u[(size_t)ix * nz + iz] - u[(size_t)(ix - 1) * nz + iz]) / (xv[ix] - xv[ix - 1]);
    } else {
        gx = (u[(size_t)(ix + 1) * nz + iz] - u[(size_t)(ix - 1) * nz + iz]) /
             (xv[ix + 1] - xv[ix - 1]);
    }
    if (nz == 1) {
        gz = 0.0;
    } else if (iz == 0) {
        gz = (v[(size_t)ix * nz + 1] - v[(size_t)ix * nz]) / (zv[1] - zv[0]);
    } else if (iz == nz - 1) {
        gz = (v[(size_t)ix * nz + iz] - v[(size_t)ix * nz + iz - 1]) / (zv[iz] - zv[iz - 1]);
    } else {
        gz = (v[(size_t)ix * nz + iz + 1] - v[(size_t)ix * nz + iz - 1]) / (zv[iz + 1] - zv[iz - 1]);
    }
    out[(size_t)w * P + (size_t)(nx - 1 - ix) * nz + iz] = (float)(gx + gz);
}

struct DevMem {
    std::vector<void *> ptrs;
    ~DevMem() {
        for (void *p : ptrs) cudaFree(p);
    }
    template <class T>
    int get(T **p, size_t n) {
        void *q = nullptr;
        if (cudaMalloc(&q, n * sizeof(T)) != cudaSuccess) {
            set_error("analytic: cudaMalloc(%zu) failed", n * sizeof(T));
            return MSOT_ENOMEM;
        }
        ptrs.push_back(q);
        *p = static_cast<T *>(q);
        return MSOT_OK;
    }
    template <class T>
    int put(T **p, const T *h, size_t n, cudaStream_t st) {
        int rc = get(p, n);
        if (rc) return rc;
        MSOT_CUDA_TRY(cudaMemcpyAsync(*p, h, n * sizeof(T), cudaMemcpyHostToDevice, st));
        return MSOT_OK;
    }
};

#define RC(x)                                                                              \
    do {                                                                                   \
        int rc_ = (x);                                                                     \
        if (rc_) return rc_;                                                               \
    } while (0)

// Shared set-up: detector angles (dmas_cf.m:45-46) and the index table.
static int index_table(DevMem &m, int D, int T, const double *x, int nx, const double *z, int nz,
                       double c, double fs, double n_crop, double coverage, double R,
                       cudaStream_t st, int32_t **d_idx, double **d_cos, double **d_sin) {
    std::vector<double> ca(D), sa(D);
    const double off = (180.0 - coverage) / 2.0, step = D > 1 ? coverage / (D - 1) : 0.0;
    const double pi = 3.141592653589793238462643383279502884;
    for (int d = 0; d < D; ++d) {
        const double a = -(off + step * d) * pi / 180.0;
        ca[d] = std::cos(a);
        sa[d] = std::sin(a);
    }
    double *dx, *dz;
    int *derr;
    RC(m.put(d_cos, ca.data(), D, st));
    RC(m.put(d_sin, sa.data(), D, st));
    RC(m.put(&dx, x, nx, st));
    RC(m.put(&dz, z, nz, st));
    RC(m.get(d_idx, (size_t)D * nx * nz));
    RC(m.get(&derr, 1));
    MSOT_CUDA_TRY(cudaMemsetAsync(derr, 0, sizeof(int), st));
    const int P = nx * nz;
    KLAUNCH(k_nearest_index<<<dim3(div_up(P, 256), D), 256, 0, st>>>(
        *d_cos, *d_sin, dx, dz, nx, nz, D, R, c, fs, (1.0 + n_crop) / fs, T, *d_idx, derr));
    MSOT_LAUNCH_CHECK();
    int herr = 0;
    MSOT_CUDA_TRY(cudaMemcpyAsync(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost, st));
    MSOT_CUDA_TRY(cudaStreamSynchronize(st));
    if (herr) {
        set_error("nearest-sample index outside the sinogram (the reference errors here)");
        return MSOT_ERANGE;
    }
    return MSOT_OK;
}

}  // namespace msot

using namespace msot;

extern "C" {

int msot_dmas_cf(const float *d_sig, int W, int D, int T, const double *x, int nx,
                 const double *z, int nz, double c, double fs, double n_crop, double coverage_deg,
                 double radius, float *d_dmas_cf, float *d_dmas, float *d_cf, float *d_das,
                 void *stream) {
    if (!d_sig || !x || !z || !d_dmas_cf || !d_dmas || !d_cf || !d_das || W <= 0 || D <= 1 ||
        T <= 0 || nx <= 0 || nz <= 0) {
        set_error("dmas_cf: bad arguments");
        return MSOT_EINVAL;
    }
    cudaStream_t st = (cudaStream_t)stream;
    DevMem m;
    int32_t *idx;
    double *ca, *sa;
    RC(index_table(m, D, T, x, nx, z, nz, c, fs, n_crop, coverage_deg, radius, st, &idx, &ca, &sa));
    unsigned int *mx;
    RC(m.get(&mx, 1));
    MSOT_CUDA_TRY(cudaMemsetAsync(mx, 0, sizeof(unsigned int), st));
    const size_t n = (size_t)W * D * T;
    KLAUNCH(k_max_abs<<<1024, 256, 0, st>>>(d_sig, n, mx));
    const int P = nx * nz;
    KLAUNCH(k_dmas_cf<<<dim3(div_up(P, 128), W), 128, 0, st>>>(d_sig, idx, mx, P, D, T, d_dmas_cf,
                                                              d_dmas, d_cf, d_das));
    MSOT_LAUNCH_CHECK();
    MSOT_CUDA_TRY(cudaStreamSynchronize(st));
    return MSOT_OK;
}

int msot_backproject_waveeq(const float *d_sig, int W, int D, int T, const double *x, int nx,
                            const double *z, int nz, double c, double fs, double n_crop,
                            double coverage_deg, double radius, const double *psf, int psf_m,
                            int psf_n, const float *d_K, int K_n, float *d_out, void *stream) {
    if (!d_sig || !x || !z || !psf || !d_K || !d_out || W <= 0 || D <= 1 || T <= 1 || nx <= 0 ||
        nz <= 0 || psf_m <= 0 || psf_n <= 0) {
        set_error("backproject_waveeq: bad arguments");
        return MSOT_EINVAL;
    }
    const long crop = std::lround(n_crop);
    if ((double)crop != n_crop || crop < 0 || crop + T > K_n) {
        set_error("backproject_waveeq: K (%d x %d) does not cover samples %ld..%ld", K_n, K_n,
                  crop + 1, crop + T);
        return MSOT_EINVAL;
    }
    double psum = 0.0;
    for (int i = 0; i < psf_m * psf_n; ++i) psum += psf[i];
    if (psum == 0.0) {
        set_error("backproject_waveeq: psf sums to zero");
        return MSOT_EINVAL;
    }
    cudaStream_t st = (cudaStream_t)stream;
    DevMem m;
    int32_t *idx;
    double *ca, *sa, *dpsf, *fx, *fz, *dx, *dz;
    RC(index_table(m, D, T, x, nx, z, nz, c, fs, n_crop, coverage_deg, radius, st, &idx, &ca, &sa));
    RC(m.put(&dpsf, psf, (size_t)psf_m * psf_n, st));
    RC(m.put(&dx, x, nx, st));
    RC(m.put(&dz, z, nz, st));
    float *s1, *s2;
    const size_t n = (size_t)W * D * T;
    const int P = nx * nz;
    RC(m.get(&s1, n));
    RC(m.get(&s2, n));
    RC(m.get(&fx, (size_t)W * P));
    RC(m.get(&fz, (size_t)W * P));
    const double dt = 1.0 / fs;
    KLAUNCH(k_cumtrapz<<<div_up(W * D, 128), 128, 0, st>>>(d_sig, s1, W * D, T, c, dt, n_crop));
    KLAUNCH(k_psf_same<<<dim3(div_up(T, 128), D, W), 128, 0, st>>>(s1, s2, dpsf, psf_m, psf_n,
                                                                 1.0 / psum, D, T));
    MSOT_LAUNCH_CHECK();
    // s1 = K(acq, acq) * s2 * dt : one column-major GEMM over all (d, w)
    // columns, on the tensor cores (gemm_tc.cu)
    const float *Ksub = d_K + (size_t)crop * K_n + crop;
    RC(tc_sgemm(T, D * W, T, (float)dt, Ksub, K_n, s2, T, s1, T, st));
    KLAUNCH(k_bp_gather<<<dim3(div_up(P, 128), W), 128, 0, st>>>(s1, idx, ca, sa, P, D, T, dt * c,
                                                                 fx, fz));
    KLAUNCH(k_div_fliplr<<<dim3(div_up(P, 256), W), 256, 0, st>>>(fx, fz, dx, dz, nx, nz, d_out));
    MSOT_LAUNCH_CHECK();
    MSOT_CUDA_TRY(cudaStreamSynchronize(st));
    return tc_sgemm_check();
}

}  // extern "C"
