// preprocess.cu -- raw-sinogram pre-processing on the GPU, in the order of
// reconstruction_example_script.m:24-26:
//   crop_first_n_signals.m:2               drop the first n_crop samples
//   apply_butterworth_window_to_sinogram.m:5-9
//       x <- mean + (x - mean) |h(t)|, h = freqz of an order-n Butterworth
//       band-pass with cut-offs [low, high] / T (in samples), T points on
//       [0, pi)
//   filter_butter_zero_phase.m:16-48 (use_fft = true)
//       demean when fmin > 0; x <- ifft(|H|^2 fft(x)), H the order-8
//       low-pass (fmax) times the order-2 high-pass (fmin) on T whole-circle
//       bins
// along the time axis of every column (sinogram layout [W][D][T], t fastest
// = MATLAB T x D x W).
//
// The Butterworth designs follow the published analog-prototype method
// (poles -exp(i pi m / 2N), m = -N+1, -N+3, .., N-1; frequency transform with
// pre-warped cut-offs 4 tan(pi Wn / 2); bilinear transform at fs = 2), as in
// MATLAB's and scipy's butter; the responses are evaluated from the
// zero-pole-gain form.  Host FP64.
//
// GPU: k_prep_columns (one CTA per column: crop, window, demean; FP64 means)
// and, for the zero-phase filter, the circular convolution with
// h = ifft(|H|^2) as one FP32 GEMM with the T x T circulant (cuBLAS SGEMM,
// a plain library GEMM): 2 T^2 flops per column at the SGEMM rate instead of
// an arbitrary-length FFT.

#include <cmath>
#include <complex>
#include <cstring>
#include <vector>

#include "common.cuh"

namespace msot {

using cd = std::complex<double>;

// Butterworth zeros, poles and gain of the digital filter (type 0 low-pass,
// 1 high-pass, 2 band-pass; wn in units of the Nyquist frequency)
static void butter_zpk(int N, double wn1, double wn2, int type, std::vector<cd> &z,
                       std::vector<cd> &p, double &k) {
    z.clear();
    p.clear();
    k = 1.0;
    for (int m = -N + 1; m <= N - 1; m += 2) p.push_back(-std::exp(cd(0.0, M_PI * m / (2.0 * N))));
    const double fs = 2.0;
    auto warp = [&](double w) { return 2.0 * fs * std::tan(M_PI * w / fs); };
    if (type == 0) {
        const double wo = warp(wn1);
        for (auto &q : p) q *= wo;
        k *= std::pow(wo, (double)p.size());
    } else if (type == 1) {
        const double wo = warp(wn1);
        cd prod = 1.0;
        for (auto q : p) prod *= -q;
        k *= std::real(cd(1.0) / prod);
        for (auto &q : p) q = wo / q;
        z.assign(p.size(), cd(0.0));
    } else {
        const double w1 = warp(wn1), w2 = warp(wn2);
        const double bw = w2 - w1, wo = std::sqrt(w1 * w2);
        std::vector<cd> hi, lo;
        for (auto q : p) {
            const cd ql = q * (bw / 2.0);
            const cd r = std::sqrt(ql * ql - wo * wo);
            hi.push_back(ql + r);
            lo.push_back(ql - r);
        }
        k *= std::pow(bw, (double)p.size());
        z.assign(p.size(), cd(0.0));
        p = hi;
        p.insert(p.end(), lo.begin(), lo.end());
    }
    const double fs2 = 2.0 * fs;
    cd num = 1.0, den = 1.0;
    for (auto q : z) num *= fs2 - q;
    for (auto q : p) den *= fs2 - q;
    for (auto &q : z) q = (fs2 + q) / (fs2 - q);
    for (auto &q : p) q = (fs2 + q) / (fs2 - q);
    while (z.size() < p.size()) z.push_back(-1.0);
    k *= std::real(num / den);
}

// |H(e^{i w})| of a zero-pole-gain filter
static double zpk_mag(const std::vector<cd> &z, const std::vector<cd> &p, double k, double w) {
    const cd e = std::exp(cd(0.0, w));
    cd h = k;
    for (auto q : z) h *= e - q;
    for (auto q : p) h /= e - q;
    return std::abs(h);
}

__device__ __forceinline__ double block_sum(double v, double *red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    __syncthreads();  // red is reused between calls
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += red[i];
    return s;
}

// one CTA per column: x = raw[n_crop .. n_crop + T); window; demean
__global__ void __launch_bounds__(256) k_prep_columns(const float *__restrict__ raw, int T_raw,
                                                      int n_crop, int T,
                                                      const float *__restrict__ win, int demean,
                                                      float *__restrict__ out) {
    extern __shared__ float col[];
    __shared__ double red[8];
    const float *src = raw + (size_t)blockIdx.x * T_raw + n_crop;
    double s = 0.0;
    for (int t = threadIdx.x; t < T; t += blockDim.x) {
        const float v = src[t];
        col[t] = v;
        s += v;
    }
    if (win) {
        const double m = block_sum(s, red) / T;
        s = 0.0;
        for (int t = threadIdx.x; t < T; t += blockDim.x) {
            const float v = (float)(m + ((double)col[t] - m) * (double)win[t]);
            col[t] = v;
            s += v;
        }
    }
    float *dst = out + (size_t)blockIdx.x * T;
    if (demean) {
        const float m = (float)(block_sum(s, red) / T);
        for (int t = threadIdx.x; t < T; t += blockDim.x) dst[t] = col[t] - m;
    } else {
        for (int t = threadIdx.x; t < T; t += blockDim.x) dst[t] = col[t];
    }
}

}  // namespace msot

using namespace msot;

struct msot_prep {
    int T_raw = 0, n_crop = 0, T = 0, max_cols = 0, demean = 0;
    float *win = nullptr;   // [T] window |h|, or null
    float *circ = nullptr;  // [T][T] circulant of ifft(|H|^2) (column-major), or null
    float *work = nullptr;  // [max_cols][T] GEMM input
    ~msot_prep() {
        cudaFree(win);
        cudaFree(circ);
        cudaFree(work);
    }
};

extern "C" {

int msot_butter_response(int order, int type, double wn1, double wn2, int n, int whole,
                         double *mag) {
    if (order < 1 || order > 16 || type < 0 || type > 2 || n < 1 || !mag || !(wn1 > 0) ||
        !(wn1 < 1) || (type == 2 && !(wn2 > wn1 && wn2 < 1))) {
        set_error("butter_response: bad arguments");
        return MSOT_EINVAL;
    }
    std::vector<cd> z, p;
    double k;
    butter_zpk(order, wn1, wn2, type, z, p, k);
    const double step = (whole ? 2.0 : 1.0) * M_PI / n;
    for (int i = 0; i < n; ++i) mag[i] = zpk_mag(z, p, k, step * i);
    return MSOT_OK;
}

int msot_prep_create(int T_raw, int n_crop, int window_order, double window_low,
                     double window_high, double fs, double fmin, double fmax, int max_cols,
                     msot_prep_t *out) {
    const int T = T_raw - n_crop;
    if (!out || T_raw < 2 || n_crop < 0 || T < 2 || T > 8192 || max_cols < 1 ||
        (window_order > 0 && !(window_low > 0 && window_high > window_low && window_high < T)) ||
        ((fmin > 0 || fmax > 0) && !(fs > 0)) || (fmax > 0 && !(2 * fmax < fs)) ||
        (fmin > 0 && !(2 * fmin < fs))) {
        set_error("prep_create: bad arguments (T = T_raw - n_crop in [2, 8192], window cut-offs "
                  "0 < low < high < T, cut-off frequencies below fs / 2)");
        return MSOT_EINVAL;
    }
    auto *pp = new msot_prep();
    pp->T_raw = T_raw;
    pp->n_crop = n_crop;
    pp->T = T;
    pp->max_cols = max_cols;
    pp->demean = fmin > 0;
    auto fail = [&](cudaError_t e) {
        delete pp;
        set_error("prep_create: %s", cudaGetErrorString(e));
        return MSOT_ECUDA;
    };
    cudaError_t e;
    if (window_order > 0) {
        // apply_butterworth_window_to_sinogram.m:5-7: band-pass on [low, high] / T,
        // |freqz| at T points of [0, pi)
        std::vector<cd> z, p;
        double k;
        butter_zpk(window_order, window_low / T, window_high / T, 2, z, p, k);
        std::vector<float> w(T);
        for (int t = 0; t < T; ++t) w[t] = (float)zpk_mag(z, p, k, M_PI * t / T);
        if ((e = cudaMalloc(&pp->win, sizeof(float) * T)) != cudaSuccess) return fail(e);
        if ((e = cudaMemcpy(pp->win, w.data(), sizeof(float) * T, cudaMemcpyHostToDevice)) !=
            cudaSuccess)
            return fail(e);
    }
    if (fmin > 0 || fmax > 0) {
        // filter_butter_zero_phase.m:27-45: |H|^2 on T whole-circle bins
        std::vector<double> H2(T, 1.0);
        std::vector<cd> z, p;
        double k;
        if (fmax > 0) {
            butter_zpk(8, 2 * fmax / fs, 0, 0, z, p, k);
            for (int i = 0; i < T; ++i) {
                const double m = zpk_mag(z, p, k, 2 * M_PI * i / T);
                H2[i] *= m * m;
            }
        }
        if (fmin > 0) {
            butter_zpk(2, 2 * fmin / fs, 0, 1, z, p, k);
            for (int i = 0; i < T; ++i) {
                const double m = zpk_mag(z, p, k, 2 * M_PI * i / T);
                H2[i] *= m * m;
            }
        }
        // h[n] = (1 / T) sum_k H2[k] cos(2 pi k n / T)  (H2 is even in k)
        std::vector<double> cs(T), h(T);
        for (int i = 0; i < T; ++i) cs[i] = std::cos(2 * M_PI * i / T);
        for (int n = 0; n < T; ++n) {
            double a = 0.0;
            size_t idx = 0;
            for (int kk = 0; kk < T; ++kk) {
                a += H2[kk] * cs[idx];
                idx += n;
                if (idx >= (size_t)T) idx -= T;
            }
            h[n] = a / T;
        }
        // circulant C[t][s] = h[(t - s) mod T], column-major (t fastest)
        std::vector<float> C((size_t)T * T);
        for (int s = 0; s < T; ++s)
            for (int t = 0; t < T; ++t) C[(size_t)s * T + t] = (float)h[(t - s + T) % T];
        if ((e = cudaMalloc(&pp->circ, sizeof(float) * C.size())) != cudaSuccess) return fail(e);
        if ((e = cudaMemcpy(pp->circ, C.data(), sizeof(float) * C.size(),
                            cudaMemcpyHostToDevice)) != cudaSuccess)
            return fail(e);
        if ((e = cudaMalloc(&pp->work, sizeof(float) * (size_t)max_cols * T)) != cudaSuccess)
            return fail(e);
    }
    *out = pp;
    return MSOT_OK;
}

int msot_prep_destroy(msot_prep_t p) {
    delete p;
    return MSOT_OK;
}

int msot_prep_apply(msot_prep_t p, const float *d_raw, float *d_out, int n_cols, void *stream) {
    if (!p || !d_raw || !d_out || n_cols < 1 || n_cols > p->max_cols) {
        set_error("prep_apply: bad arguments (n_cols %d, max %d)", n_cols, p ? p->max_cols : 0);
        return MSOT_EINVAL;
    }
    const size_t in_bytes = sizeof(float) * (size_t)n_cols * p->T_raw;
    const size_t out_bytes = sizeof(float) * (size_t)n_cols * p->T;
    const char *a = reinterpret_cast<const char *>(d_raw), *b = reinterpret_cast<const char *>(d_out);
    if (!p->circ && p->n_crop > 0 && a < b + out_bytes && b < a + in_bytes) {
        set_error("prep_apply: input and output overlap (allowed only without cropping or "
                  "with the filter)");
        return MSOT_EINVAL;
    }
    cudaStream_t st = (cudaStream_t)stream;
    float *dst = p->circ ? p->work : d_out;
    KLAUNCH(k_prep_columns<<<n_cols, 256, sizeof(float) * p->T, st>>>(
        d_raw, p->T_raw, p->n_crop, p->T, p->win, p->demean, dst));
    MSOT_LAUNCH_CHECK();
    // the zero-phase filter: the T x T circulant times the columns, on the
    // tensor cores (gemm_tc.cu)
    if (p->circ) return tc_sgemm(p->T, n_cols, p->T, 1.f, p->circ, p->T, p->work, p->T, d_out,
                                 p->T, st);
    return MSOT_OK;
}

}  // extern "C"
