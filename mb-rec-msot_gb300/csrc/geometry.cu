// geometry.cu -- the model's geometry tables on the GPU.
//
//   msot_travel_times <- MSOTmodel.m:350-382 (calculate_travel_time with one
//                        speed of sound: straight rays, refraction.m:20-24):
//                        tau[d][p] = |x_p - x_d| / c * fs - delay - n_crop,
//                        detector angles from Probe.m:112-116.
//
//   msot_spmr_tables  <- is_tir_derivation/calculate_polarSPMR.m:21-184 and
//                        MSOTmodel.m:463-480, 586-613 (2-D, single speed of
//                        sound): the polar spatial pixel model response
//                        table of one element, its start/end samples and the
//                        (pixel, detector) -> table column map.  The element's
//                        spatial impulse response, which the reference takes
//                        from Field II (absent), is the Rayleigh integral over
//                        sub_x x sub_y point sources (sub-element centres,
//                        weight area / (2 pi R)); everything after it follows
//                        calculate_polarSPMR.m: convolution with the N-shape
//                        pixel response phi(c t) (-t) (:68-69) and the squared
//                        magnitude of an order-8 Butterworth low pass at fs/2
//                        (:49-53, :74), both at 5 GHz, linear interpolation at
//                        the DAC samples around the travel time (:146-148),
//                        zeroing below 1e-4 of the column maximum (:151-152),
//                        first/last non-zero sample (:158-160) and the crop to
//                        the common half length (:179-183).
//
// Computed in FP64 with every operation rounded separately (no contraction),
// the form in which the tables are passed to msot_plan_create.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <vector>

#include "common.cuh"

namespace msot {

// one point source of an element: position and area
struct PtSrc {
    double x, y, z, area;
};

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

// r[d][p] = |x_p - x_d|, th[d][p] = acos(((x_d - x_p) x_d + (z_d - z_p) z_d) /
// (|x_d| r)) (MSOTmodel.m:605-606); running max of th and min/max of r
// (non-negative doubles order like their bit patterns)
__global__ void k_spmr_polar(const double *__restrict__ xd, const double *__restrict__ zd,
                             const double *__restrict__ xv, const double *__restrict__ zv,
                             int nx, int nz, const double *__restrict__ virt_x,
                             const double *__restrict__ virt_z, double *__restrict__ r_out,
                             double *__restrict__ th_out, unsigned long long *ext) {
    const int P = nx * nz;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const int d = blockIdx.y;
    if (p >= P) return;
    const int ix = p / nz, iz = p - ix * nz;
    // the pixel, or its virtual source for detector d (dual speed of sound)
    const double px = virt_x ? virt_x[(size_t)d * P + p] : xv[ix];
    const double pz = virt_z ? virt_z[(size_t)d * P + p] : zv[iz];
    const double ax = __dadd_rn(xd[d], -px), az = __dadd_rn(zd[d], -pz);
    const double r = __dsqrt_rn(__dadd_rn(__dmul_rn(ax, ax), __dmul_rn(az, az)));
    const double nd = __dsqrt_rn(__dadd_rn(__dmul_rn(xd[d], xd[d]), __dmul_rn(zd[d], zd[d])));
    double cs = __ddiv_rn(__dadd_rn(__dmul_rn(ax, xd[d]), __dmul_rn(az, zd[d])), __dmul_rn(nd, r));
    cs = fmin(1.0, fmax(-1.0, cs));
    const double th = acos(cs);
    r_out[(size_t)d * P + p] = r;
    th_out[(size_t)d * P + p] = th;
    atomicMin(&ext[0], (unsigned long long)__double_as_longlong(r));
    atomicMax(&ext[1], (unsigned long long)__double_as_longlong(r));
    atomicMax(&ext[2], (unsigned long long)__double_as_longlong(th));
}

// idx[d][p] = (round(1 + (r - d_min) / d_step) - 1) * n_angle + 1 + round(th deg / a_step)
// (MSOTmodel.m:472-477, MATLAB round: half away from zero), 1-based
__global__ void k_spmr_index(const double *__restrict__ r, const double *__restrict__ th,
                             size_t n, double d_min, double d_step, double a_step_deg,
                             int n_angle, int n_dist, int32_t *__restrict__ idx, int *err) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double di = round(__dadd_rn(1.0, __ddiv_rn(__dadd_rn(r[i], -d_min), d_step)));
    const double deg = __ddiv_rn(__dmul_rn(th[i], 180.0), M_PI);
    const double ai = __dadd_rn(1.0, round(__ddiv_rn(deg, a_step_deg)));
    if (di < 1.0 || di > n_dist || ai < 1.0 || ai > n_angle) atomicOr(err, 1);
    idx[i] = (int32_t)((di - 1.0) * n_angle + ai);
}

// One table column per (angle, distance) grid point, one thread per DAC
// sample n of the window: sum over the element's point sources of
// a_k g(t_n - R_k / c) with g the filtered N-shape on the 5 GHz grid
// (linear interpolation, calculate_polarSPMR.m:146-148).
// col = di * n_angle + ai; out[col][n], n = 0 .. 2H.
__global__ void k_spmr_columns(const double *__restrict__ g, int gM, double fsF,
                               const PtSrc *__restrict__ src, int n_src, double d_min,
                               double d_step, double a_step_deg, int n_angle, int n_cols,
                               int H, double c, double fs, double *__restrict__ out) {
    const int S0 = 2 * H + 1;
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long)n_cols * S0) return;
    const int col = (int)(i / S0), n = (int)(i - (long)col * S0) - H;
    const int di = col / n_angle, ai = col - di * n_angle;
    const double r = __dadd_rn(d_min, __dmul_rn((double)di, d_step));
    const double th = __ddiv_rn(__dmul_rn(__dmul_rn((double)ai, a_step_deg), M_PI), 180.0);
    const double px = __dmul_rn(r, sin(th)), pz = __dmul_rn(r, cos(th));  // point (x, 0, z)
    const double t = __dadd_rn(__ddiv_rn(r, c), __ddiv_rn((double)n, fs));
    double acc = 0.0;
    for (int k = 0; k < n_src; ++k) {
        const PtSrc s = src[k];
        const double ex = __dadd_rn(px, -s.x), ey = -s.y, ez = __dadd_rn(pz, -s.z);
        const double R = __dsqrt_rn(
            __dadd_rn(__dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey)), __dmul_rn(ez, ez)));
        const double a = __ddiv_rn(s.area, __dmul_rn(2.0 * M_PI, R));
        const double u = __dmul_rn(__dadd_rn(t, -__ddiv_rn(R, c)), fsF);  // fine-grid position
        const double fl = floor(u);
        const long m = (long)fl;
        if (m < -gM || m >= gM) continue;
        const double w = __dadd_rn(u, -fl);
        const double gv = __dadd_rn(__dmul_rn(__dadd_rn(1.0, -w), g[m + gM]),
                                    __dmul_rn(w, g[m + 1 + gM]));
        acc = __dadd_rn(acc, __dmul_rn(a, gv));
    }
    out[i] = acc;
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

// ---------------------------------------------------------------------------
// Dual speed of sound: refraction at the membrane z = m(x) = sum_k a_k x^k
// ---------------------------------------------------------------------------
constexpr int MEM_MAX_COEF = 8;
constexpr int FERMAT_ITERS = 64;  // golden-section steps: 0.618^64 ~ 4e-14 of 2 R

__device__ __forceinline__ double mem_z(const double *a, int n, double x) {
    double z = 0.0;
    for (int k = n - 1; k >= 0; --k) z = fma(z, x, a[k]);
    return z;
}
__device__ __forceinline__ double fermat_time(double x, double px, double pz, double dx, double dz,
                                              const double *a, int n, double inv_cb,
                                              double inv_ca) {
    const double mz = mem_z(a, n, x);
    const double ux = px - x, uz = pz - mz, vx = x - dx, vz = mz - dz;
    return sqrt(ux * ux + uz * uz) * inv_cb + sqrt(vx * vx + vz * vz) * inv_ca;
}

// refraction.m:8-24 / fermat_principle.m:17-24: a pixel below the membrane
// (z > m(x)) reaches detector d along the path through the membrane point
// (x_m, m(x_m)) that minimises |p - q| / c_below + |q - d| / c_above over
// x_m in [-R, R] (golden-section search, FP64); a pixel on the detector side
// travels straight at c_above (x_m = NaN).  out[d][p] = t fs - offset.
__global__ void k_travel_times_dual(const double *__restrict__ xd, const double *__restrict__ zd,
                                    const double *__restrict__ xv, const double *__restrict__ zv,
                                    int nx, int nz, const double *__restrict__ coef, int ncoef,
                                    double radius, double inv_cb, double inv_ca, double fs,
                                    double offset, double *__restrict__ out,
                                    double *__restrict__ xmem, double *__restrict__ vxo,
                                    double *__restrict__ vzo) {
    __shared__ double a[MEM_MAX_COEF];
    if (threadIdx.x < MEM_MAX_COEF) a[threadIdx.x] = threadIdx.x < ncoef ? coef[threadIdx.x] : 0.0;
    __syncthreads();
    const int P = nx * nz;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const int d = blockIdx.y;
    if (p >= P) return;
    const int ix = p / nz, iz = p - ix * nz;
    const double px = xv[ix], pz = zv[iz], dx = xd[d], dz = zd[d];
    double t, xm;
    if (pz > mem_z(a, ncoef, px)) {
        const double g = 0.6180339887498949;  // (sqrt(5) - 1) / 2
        double lo = -radius, hi = radius;
        double x1 = hi - g * (hi - lo), x2 = lo + g * (hi - lo);
        double f1 = fermat_time(x1, px, pz, dx, dz, a, ncoef, inv_cb, inv_ca);
        double f2 = fermat_time(x2, px, pz, dx, dz, a, ncoef, inv_cb, inv_ca);
        for (int it = 0; it < FERMAT_ITERS; ++it) {
            if (f1 < f2) {
                hi = x2;
                x2 = x1;
                f2 = f1;
                x1 = hi - g * (hi - lo);
                f1 = fermat_time(x1, px, pz, dx, dz, a, ncoef, inv_cb, inv_ca);
            } else {
                lo = x1;
                x1 = x2;
                f1 = f2;
                x2 = lo + g * (hi - lo);
                f2 = fermat_time(x2, px, pz, dx, dz, a, ncoef, inv_cb, inv_ca);
            }
        }
        if (f1 < f2) {
            t = f1;
            xm = x1;
        } else {
            t = f2;
            xm = x2;
        }
    } else {
        const double ux = dx - px, uz = dz - pz;
        t = sqrt(ux * ux + uz * uz) * inv_ca;
        xm = __longlong_as_double(0x7ff8000000000000ll);  // NaN: no intersection
    }
    out[(size_t)d * P + p] = t * fs - offset;
    if (xmem) xmem[(size_t)d * P + p] = xm;
    if (vxo) {
        // MSOTmodel.m:585-594: the virtual source on the ray from the detector
        // through the membrane point, at the distance t c_above; the pixel
        // itself where the path does not cross the membrane
        double vx = px, vz = pz;
        if (xm == xm) {
            const double qx = xm - dx, qz = mem_z(a, ncoef, xm) - dz;
            const double s = t / (inv_ca * sqrt(qx * qx + qz * qz));
            vx = dx + qx * s;
            vz = dz + qz * s;
        }
        vxo[(size_t)d * P + p] = vx;
        vzo[(size_t)d * P + p] = vz;
    }
}

extern "C" int msot_travel_times_dual(int n_det, double radius, double coverage_deg,
                                      const double *x, int nx, const double *z, int nz,
                                      double c_below, double c_above, const double *membrane,
                                      int n_coef, double fs, double delay, double n_crop,
                                      double *travel, double *x_mem, double *virt_x,
                                      double *virt_z) {
    if (n_det < 2 || nx <= 0 || nz <= 0 || !x || !z || !travel || !(c_below > 0.0) ||
        !(c_above > 0.0) || !(fs > 0.0) || !(radius > 0.0) || !membrane || n_coef < 1 ||
        n_coef > MEM_MAX_COEF || (!virt_x != !virt_z)) {
        set_error("travel_times_dual: bad arguments (1 to %d membrane coefficients)",
                  MEM_MAX_COEF);
        return MSOT_EINVAL;
    }
    std::vector<double> xd(n_det), zd(n_det);
    const double off = (180.0 - coverage_deg) / 2.0, step = coverage_deg / (n_det - 1);
    for (int k = 0; k < n_det; ++k) {
        const double ang = (off + step * k) * (M_PI / 180.0);
        xd[k] = radius * std::cos(ang);
        zd[k] = -radius * std::sin(ang);
    }
    const size_t P = (size_t)nx * nz, N = P * n_det;
    DevArrays m;
    double *dxd = m.get<double>(n_det), *dzd = m.get<double>(n_det);
    double *dx = m.get<double>(nx), *dz = m.get<double>(nz), *dc = m.get<double>(n_coef);
    double *dout = m.get<double>(N), *dxm = x_mem ? m.get<double>(N) : nullptr;
    double *dvx = virt_x ? m.get<double>(N) : nullptr, *dvz = virt_z ? m.get<double>(N) : nullptr;
    if (!dxd || !dzd || !dx || !dz || !dc || !dout || (x_mem && !dxm) || (virt_x && !dvx) ||
        (virt_z && !dvz)) {
        set_error("travel_times_dual: device allocation failed");
        return MSOT_ENOMEM;
    }
    MSOT_CUDA_TRY(cudaMemcpy(dxd, xd.data(), sizeof(double) * n_det, cudaMemcpyHostToDevice));
    MSOT_CUDA_TRY(cudaMemcpy(dzd, zd.data(), sizeof(double) * n_det, cudaMemcpyHostToDevice));
    MSOT_CUDA_TRY(cudaMemcpy(dx, x, sizeof(double) * nx, cudaMemcpyHostToDevice));
    MSOT_CUDA_TRY(cudaMemcpy(dz, z, sizeof(double) * nz, cudaMemcpyHostToDevice));
    MSOT_CUDA_TRY(cudaMemcpy(dc, membrane, sizeof(double) * n_coef, cudaMemcpyHostToDevice));
    const dim3 grid((unsigned)((P + 255) / 256), (unsigned)n_det);
    KLAUNCH(k_travel_times_dual<<<grid, 256>>>(dxd, dzd, dx, dz, nx, nz, dc, n_coef, radius,
                                               1.0 / c_below, 1.0 / c_above, fs, delay + n_crop,
                                               dout, dxm, dvx, dvz));
    MSOT_LAUNCH_CHECK();
    MSOT_CUDA_TRY(cudaMemcpy(travel, dout, sizeof(double) * N, cudaMemcpyDeviceToHost));
    if (x_mem)
        MSOT_CUDA_TRY(cudaMemcpy(x_mem, dxm, sizeof(double) * N, cudaMemcpyDeviceToHost));
    if (virt_x) {
        MSOT_CUDA_TRY(cudaMemcpy(virt_x, dvx, sizeof(double) * N, cudaMemcpyDeviceToHost));
        MSOT_CUDA_TRY(cudaMemcpy(virt_z, dvz, sizeof(double) * N, cudaMemcpyDeviceToHost));
    }
    return MSOT_OK;
}

// ---------------------------------------------------------------------------
// SPMR tables
// ---------------------------------------------------------------------------
namespace {

// in-place iterative radix-2 FFT (n a power of two), sign -1 forward
void fft_inplace(std::vector<std::complex<double>> &a, int sign) {
    const size_t n = a.size();
    for (size_t i = 1, j = 0; i < n; ++i) {
        size_t bit = n >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) std::swap(a[i], a[j]);
    }
    for (size_t len = 2; len <= n; len <<= 1) {
        const double ang = sign * 2.0 * M_PI / (double)len;
        for (size_t i = 0; i < n; i += len)
            for (size_t k = 0; k < len / 2; ++k) {
                const std::complex<double> w(std::cos(ang * k), std::sin(ang * k));
                const std::complex<double> u = a[i + k], v = a[i + k + len / 2] * w;
                a[i + k] = u + v;
                a[i + k + len / 2] = u - v;
            }
    }
}

struct SpmrSetup {
    double d_min = 0, d_max = 0, d_step = 0, a_step = 0, a_max = 0;
    int n_dist = 0, n_angle = 0;
    std::vector<double> xd, zd;
};

constexpr double SPMR_FSF = 5e9;  // calculate_polarSPMR.m:35

// Filtered N-shape on the 5 GHz grid: q(t) = phi(c t)(-t) over the half
// length of calculate_polarSPMR.m:58-68, times |H|^2 of the order-8 digital
// Butterworth low pass at fs/2 (bilinear: |H|^2 = 1 / (1 + (tan(pi f / fsF) /
// tan(pi fc / fsF))^16)), circular on NF points; g[m + M] for m = -M .. M.
std::vector<double> spmr_nshape(double sigma, double c, double fs, int &M) {
    auto phi = [&](double rr) { return std::exp(-rr * rr / (2.0 * sigma * sigma)); };
    int Hq = 200;
    if (!(std::fabs(phi(Hq / SPMR_FSF * c)) < 1e-3)) {
        for (int k = 0; k <= 16; ++k) {
            const double tb = (1.0 + 0.25 * k) * 1e-7;
            if (std::fabs(phi(tb * c)) < 1e-3) {
                Hq = (int)std::ceil(tb * SPMR_FSF);
                break;
            }
        }
    }
    const size_t NF = 1 << 16;
    std::vector<std::complex<double>> a(NF, 0.0);
    for (int j = -Hq; j <= Hq; ++j) {
        const double t = j / SPMR_FSF;
        a[(j + (long)NF) % NF] = phi(t * c) * (-t);
    }
    fft_inplace(a, -1);
    const double tc = std::tan(M_PI * (fs / 2.0) / SPMR_FSF);
    for (size_t k = 0; k < NF; ++k) {
        const double f = (double)k / (double)NF;  // in units of fsF
        const double ratio = std::tan(M_PI * f) / tc;
        const double h2 = (k == NF / 2) ? 0.0 : 1.0 / (1.0 + std::pow(ratio, 16));
        a[k] *= h2;
    }
    fft_inplace(a, +1);
    M = (int)(NF / 2) - 1;
    std::vector<double> g(2 * M + 2);
    for (int m = -M; m <= M + 1; ++m) g[m + M] = a[(m + (long)NF) % NF].real() / (double)NF;
    return g;
}

int spmr_validate(const msot_spmr_spec *s) {
    if (!s || s->n_det < 2 || s->nx < 2 || s->nz < 2 || !s->x || !s->z || !(s->c > 0) ||
        !(s->fs > 0) || !(s->pixel_sigma > 0) || !(s->elem_width > 0) ||
        !(s->elem_height > 0) || s->sub_x < 1 || s->sub_y < 1 || s->sub_x * s->sub_y > 4096 ||
        s->half_window < 1 || s->half_window > 4096 || s->elem_elev_radius < 0 ||
        (!s->virt_x != !s->virt_z)) {
        set_error("spmr: bad specification");
        return MSOT_EINVAL;
    }
    if (s->elem_elev_radius > 0 && s->elem_elev_radius < s->elem_height / 2) {
        set_error("spmr: elevation radius smaller than half the element height");
        return MSOT_EINVAL;
    }
    return MSOT_OK;
}

// point sources of one element (x along the array, y elevation, z towards
// the field), curved in elevation with radius elem_elev_radius (0 = flat)
std::vector<PtSrc> spmr_sources(const msot_spmr_spec *s) {
    std::vector<PtSrc> v;
    const double dx = s->elem_width / s->sub_x, dy = s->elem_height / s->sub_y;
    for (int i = 0; i < s->sub_x; ++i)
        for (int j = 0; j < s->sub_y; ++j) {
            const double x = -s->elem_width / 2 + (i + 0.5) * dx;
            const double y = -s->elem_height / 2 + (j + 0.5) * dy;
            double z = 0.0, area = dx * dy;
            if (s->elem_elev_radius > 0) {
                const double Re = s->elem_elev_radius;
                z = Re - std::sqrt(Re * Re - y * y);
                area = dx * dy * Re / std::sqrt(Re * Re - y * y);  // arc length of the strip
            }
            v.push_back(PtSrc{x, y, z, area});
        }
    return v;
}

struct DevMemG {
    std::vector<void *> v;
    ~DevMemG() {
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

// the whole computation; outputs are optional (sizes only when null)
int spmr_run(const msot_spmr_spec *s, msot_spmr_info *info, double *sir, int32_t *se,
             int32_t *idx) {
    int rc = spmr_validate(s);
    if (rc) return rc;
    const int D = s->n_det, nx = s->nx, nz = s->nz, P = nx * nz;
    std::vector<double> xd(D), zd(D);
    const double off = (180.0 - s->coverage_deg) / 2.0, step = s->coverage_deg / (D - 1);
    for (int k = 0; k < D; ++k) {
        const double a = (off + step * k) * (M_PI / 180.0);
        xd[k] = s->radius * std::cos(a);
        zd[k] = -s->radius * std::sin(a);
    }
    DevMemG m;
    double *dxd = m.get<double>(D), *dzd = m.get<double>(D), *dx = m.get<double>(nx),
           *dz = m.get<double>(nz), *dr = m.get<double>((size_t)P * D),
           *dth = m.get<double>((size_t)P * D);
    unsigned long long *dext = m.get<unsigned long long>(3);
    int *derr = m.get<int>(1);
    double *dvx = s->virt_x ? m.get<double>((size_t)P * D) : nullptr;
    double *dvz = s->virt_x ? m.get<double>((size_t)P * D) : nullptr;
    if (!dxd || !dzd || !dx || !dz || !dr || !dth || !dext || !derr ||
        (s->virt_x && (!dvx || !dvz))) {
        set_error("spmr: device allocation failed");
        return MSOT_ENOMEM;
    }
    MSOT_CUDA_TRY(cudaMemcpy(dxd, xd.data(), sizeof(double) * D, cudaMemcpyHostToDevice));
    MSOT_CUDA_TRY(cudaMemcpy(dzd, zd.data(), sizeof(double) * D, cudaMemcpyHostToDevice));
    MSOT_CUDA_TRY(cudaMemcpy(dx, s->x, sizeof(double) * nx, cudaMemcpyHostToDevice));
    MSOT_CUDA_TRY(cudaMemcpy(dz, s->z, sizeof(double) * nz, cudaMemcpyHostToDevice));
    const unsigned long long ext0[3] = {~0ull, 0ull, 0ull};
    MSOT_CUDA_TRY(cudaMemcpy(dext, ext0, sizeof(ext0), cudaMemcpyHostToDevice));
    MSOT_CUDA_TRY(cudaMemset(derr, 0, sizeof(int)));
    if (s->virt_x) {
        MSOT_CUDA_TRY(cudaMemcpy(dvx, s->virt_x, sizeof(double) * P * D, cudaMemcpyHostToDevice));
        MSOT_CUDA_TRY(cudaMemcpy(dvz, s->virt_z, sizeof(double) * P * D, cudaMemcpyHostToDevice));
    }
    KLAUNCH(k_spmr_polar<<<dim3((unsigned)((P + 255) / 256), (unsigned)D), 256>>>(
        dxd, dzd, dx, dz, nx, nz, dvx, dvz, dr, dth, dext));
    MSOT_LAUNCH_CHECK();
    unsigned long long ext[3];
    MSOT_CUDA_TRY(cudaMemcpy(ext, dext, sizeof(ext), cudaMemcpyDeviceToHost));
    double rmin, rmax, thmax;
    std::memcpy(&rmin, &ext[0], 8);
    std::memcpy(&rmax, &ext[1], 8);
    std::memcpy(&thmax, &ext[2], 8);
    // MSOTmodel.m:600-613 (the azimuth bound exactly as written there)
    const double res = std::min(s->x[1] - s->x[0], s->z[1] - s->z[0]);
    const double d_step = res * (1450.0 / s->c);
    const double d_min = rmin - d_step, d_max = rmax + d_step;
    const double a_step = std::atan2(d_step, d_max) / M_PI * 180.0;
    const double a_max = std::ceil((thmax / M_PI * 180.0) * a_step) / a_step;
    // calculate_polarSPMR.m:22-25
    const int n_dist = (int)std::ceil((d_max - d_min) / d_step) + 1;
    const int n_angle = (int)std::ceil(a_max / a_step) + 1;
    const int NS = n_dist * n_angle, H = s->half_window, S0 = 2 * H + 1;
    int M = 0;
    const std::vector<double> g = spmr_nshape(s->pixel_sigma, s->c, s->fs, M);
    const std::vector<PtSrc> src = spmr_sources(s);
    double *dg = m.get<double>(g.size()), *dout = m.get<double>((size_t)NS * S0);
    PtSrc *dsrc = m.get<PtSrc>(src.size());
    if (!dg || !dout || !dsrc) {
        set_error("spmr: device allocation failed");
        return MSOT_ENOMEM;
    }
    MSOT_CUDA_TRY(cudaMemcpy(dg, g.data(), sizeof(double) * g.size(), cudaMemcpyHostToDevice));
    MSOT_CUDA_TRY(cudaMemcpy(dsrc, src.data(), sizeof(PtSrc) * src.size(),
                             cudaMemcpyHostToDevice));
    const long nthr = (long)NS * S0;
    KLAUNCH(k_spmr_columns<<<(unsigned)((nthr + 255) / 256), 256>>>(
        dg, M, SPMR_FSF, dsrc, (int)src.size(), d_min, d_step, a_step, n_angle, NS, H, s->c,
        s->fs, dout));
    MSOT_LAUNCH_CHECK();
    std::vector<double> tab((size_t)NS * S0);
    MSOT_CUDA_TRY(cudaMemcpy(tab.data(), dout, sizeof(double) * tab.size(),
                             cudaMemcpyDeviceToHost));
    // calculate_polarSPMR.m:151-160, 179-183 (1-based start / end)
    std::vector<int> st(NS), en(NS);
    for (int col = 0; col < NS; ++col) {
        double *v = tab.data() + (size_t)col * S0;
        double mx = 0.0;
        for (int k = 0; k < S0; ++k) mx = std::max(mx, std::fabs(v[k]));
        for (int k = 0; k < S0; ++k)
            if (std::fabs(v[k]) < mx * 1e-4) v[k] = 0.0;
        int a = -1, b = -1;
        for (int k = 0; k < S0; ++k)
            if (v[k] != 0.0) {
                if (a < 0) a = k;
                b = k;
            }
        if (a < 0) {
            set_error("spmr: an all-zero column (%d); widen half_window", col);
            return MSOT_ERANGE;
        }
        if (a == 0 || b == S0 - 1) {
            set_error("spmr: column %d reaches the window edge; widen half_window", col);
            return MSOT_ERANGE;
        }
        st[col] = a + 1;
        en[col] = b + 1;
    }
    int hmax = 0;
    for (int col = 0; col < NS; ++col)
        hmax = std::max(hmax, std::max(H + 1 - st[col], en[col] - H - 1) + 1);
    const int h = std::min(hmax, H), S = 2 * h + 1, shift = H - h;
    if (info) {
        info->d_min = d_min;
        info->d_step = d_step;
        info->a_step_deg = a_step;
        info->n_dist = n_dist;
        info->n_angle = n_angle;
        info->sir_len = S;
        info->n_sir = NS;
    }
    if (sir)
        for (int col = 0; col < NS; ++col)
            std::copy(tab.begin() + (size_t)col * S0 + shift,
                      tab.begin() + (size_t)col * S0 + shift + S, sir + (size_t)col * S);
    if (se)
        for (int col = 0; col < NS; ++col) {
            se[2 * col] = st[col] - shift;
            se[2 * col + 1] = en[col] - shift;
        }
    if (idx) {
        int32_t *didx = m.get<int32_t>((size_t)P * D);
        if (!didx) {
            set_error("spmr: device allocation failed");
            return MSOT_ENOMEM;
        }
        const size_t n = (size_t)P * D;
        KLAUNCH(k_spmr_index<<<(unsigned)((n + 255) / 256), 256>>>(
            dr, dth, n, d_min, d_step, a_step, n_angle, n_dist, didx, derr));
        MSOT_LAUNCH_CHECK();
        int err = 0;
        MSOT_CUDA_TRY(cudaMemcpy(&err, derr, sizeof(int), cudaMemcpyDeviceToHost));
        if (err) {
            set_error("spmr: a pixel maps outside the polar table");
            return MSOT_ERANGE;
        }
        MSOT_CUDA_TRY(cudaMemcpy(idx, didx, sizeof(int32_t) * n, cudaMemcpyDeviceToHost));
    }
    return MSOT_OK;
}

}  // namespace

extern "C" int msot_spmr_query(const msot_spmr_spec *spec, msot_spmr_info *info) {
    if (!info) {
        set_error("spmr_query: null info");
        return MSOT_EINVAL;
    }
    return spmr_run(spec, info, nullptr, nullptr, nullptr);
}

extern "C" int msot_spmr_tables(const msot_spmr_spec *spec, double *sir, int32_t *start_end,
                                int32_t *sir_idx) {
    if (!sir || !start_end || !sir_idx) {
        set_error("spmr_tables: null output");
        return MSOT_EINVAL;
    }
    return spmr_run(spec, nullptr, sir, start_end, sir_idx);
}
