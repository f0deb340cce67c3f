// geometry.cu -- the model's geometry tables on the GPU.
//
//   msot_travel_times <- MSOTmodel.m:350-382 (calculate_travel_time with one
//                        speed of sound: straight rays, refraction.m:327):
//                        tau[d][p] = |x_p - x_d| / c * fs - delay - n_crop,
//                        detector angles from Probe.m:112-116.
//
// Computed in FP64 with every operation rounded separately (no contraction),
// the form in which the table is passed to msot_plan_create.
#include <cmath>
#include <vector>

#include "common.cuh"

namespace msot {

// out[d][ix * nz + iz]
__global__ void k_travel_times(const double *__restrict__ xd, const double *__restrict__ zd,
                               const double *__restrict__ xv, const double *__restrict__ zv,
                               int nx, int nz, double inv_c_fs, double offset,
                               double *__restrict__ out) {
    const int P = nx * nz;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const int d = blockIdx.y;
    if (p >= P) return;
    const int ix = p / nz, iz = p - ix * nz;
    const double dx = __dadd_rn(xd[d], -xv[ix]);
    const double dz = __dadd_rn(zd[d], -zv[iz]);
    const double dist = __dsqrt_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dz, dz)));
    out[(size_t)d * P + p] = __dadd_rn(__dmul_rn(dist, inv_c_fs), -offset);
}

}  // namespace msot

using namespace msot;

namespace {

struct DevArrays {
    std::vector<void *> v;
    ~DevArrays() {
        for (void *p : v) cudaFree(p);
    }
    template <class T>
    T *get(size_t n) {
        void *p = nullptr;
        if (cudaMalloc(&p, (n ? n : 1) * sizeof(T)) != cudaSuccess) return nullptr;
        v.push_back(p);
        return static_cast<T *>(p);
    }
};

}  // namespace

extern "C" int msot_travel_times(int n_det, double radius, double coverage_deg, const double *x,
                                 int nx, const double *z, int nz, double c, double fs,
                                 double delay, double n_crop, double *travel) {
    if (n_det < 2 || nx <= 0 || nz <= 0 || !x || !z || !travel || !(c > 0.0) || !(fs > 0.0)) {
        set_error("travel_times: bad arguments");
        return MSOT_EINVAL;
    }
    // Probe.m:112-116: angles off + k * coverage / (D - 1), off = (180 - coverage) / 2,
    // positions (R cos a, -R sin a)
    std::vector<double> xd(n_det), zd(n_det);
    const double off = (180.0 - coverage_deg) / 2.0, step = coverage_deg / (n_det - 1);
    for (int k = 0; k < n_det; ++k) {
        const double a = (off + step * k) * (M_PI / 180.0);
        xd[k] = radius * std::cos(a);
        zd[k] = -radius * std::sin(a);
    }
    const size_t P = (size_t)nx * nz, N = P * n_det;
    DevArrays m;
    double *dxd = m.get<double>(n_det), *dzd = m.get<double>(n_det);
    double *dx = m.get<double>(nx), *dz = m.get<double>(nz), *dout = m.get<double>(N);
    if (!dxd || !dzd || !dx || !dz || !dout) {
        set_error("travel_times: device allocation failed");
        return MSOT_ENOMEM;
    }
    MSOT_CUDA_TRY(cudaMemcpy(dxd, xd.data(), sizeof(double) * n_det, cudaMemcpyHostToDevice));
    MSOT_CUDA_TRY(cudaMemcpy(dzd, zd.data(), sizeof(double) * n_det, cudaMemcpyHostToDevice));
    MSOT_CUDA_TRY(cudaMemcpy(dx, x, sizeof(double) * nx, cudaMemcpyHostToDevice));
    MSOT_CUDA_TRY(cudaMemcpy(dz, z, sizeof(double) * nz, cudaMemcpyHostToDevice));
    const dim3 grid((unsigned)((P + 255) / 256), (unsigned)n_det);
    KLAUNCH(k_travel_times<<<grid, 256>>>(dxd, dzd, dx, dz, nx, nz, fs / c, delay + n_crop,
                                          dout));
    MSOT_LAUNCH_CHECK();
    MSOT_CUDA_TRY(cudaMemcpy(travel, dout, sizeof(double) * N, cudaMemcpyDeviceToHost));
    return MSOT_OK;
}
