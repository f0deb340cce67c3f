// tv.cu -- isotropic-TV proximal operator and the TV-regularised
// non-negative solver on the GPU.
//
//   k_tv_prox  <- libraries/SplitBregmanTVdenoising/SB_ITV2.m:20-40 with
//                 DiffOper.m:1-7: split Bregman with lambda = 1, inner
//                 cgs(I + B'B, g - B'(b - d), 1e-5, 100) from zero, outer loop
//                 until ||u_prev - u|| / ||u|| <= 1e-3 (capped at TV_SB_MAX
//                 sweeps).  One CTA per image runs the whole prox on the
//                 device (bounded loops, no host round trips).
//   k_itv      <- ITV.m:5-6 (isotropic TV with MATLAB's gradient: central
//                 differences inside, one-sided at the borders).
//   msot_rec_nn_with_TV_reg <- rec_nn_with_TV_reg.m:20-54 and
//                 nnls_sparsa_based_reg_matrix_less.m:31-85 (lambda 1,
//                 beta 1e-3, w and v from zero); the inner SpaRSA call (:64,
//                 StopCriterion 1, ToleranceA 1e-8) is restated from its
//                 paper (Wright, Nowak & Figueiredo 2009): x+ = Psi(x +
//                 A'r / alpha, tau / alpha), Barzilai-Borwein alpha clipped
//                 to [1e-30, 1e30], non-monotone, no continuation.
//
// DiffOper's B = [kron(I, D); kron(D, I)] with (D v)_i = v_i - v_{i-1} for
// i >= 2 and 0 for i = 1.  On the column-major N x N image (p = ix*N + iz)
// the first block differences along z, the second along x, so (I + B'B) is a
// five-point stencil with one-sided rows at the borders.  Where SB_ITV2.m:34
// divides 0 by 0 (|Bu + b| = 0) the shrinkage here writes d = 0.
//
// All SpaRSA scalars (objective, alpha, mu = tau/alpha, stop flags) live on
// the device, so an outer iteration is a fixed launch sequence with no host
// synchronisation.  coupled = 1 makes the batch one SpaRSA problem (the
// reference's multi-wavelength call: one alpha and one objective over all
// wavelengths); coupled = 0 runs W independent reconstructions.
#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"

namespace msot {

constexpr int TV_THREADS = 1024;
constexpr int TV_SB_MAX = 200;  // split-Bregman sweeps per prox
constexpr int TV_CG_MAX = 100;  // cgs(..., 1e-5, 100)
constexpr int TV_NVEC = 16;     // device work vectors per image
constexpr int TV_RED = 256;     // threads of the reduction-carrying kernels
constexpr double TV_BETA = 1e-3;

// per-group SpaRSA scalars (group = instance, or the whole batch if coupled)
struct TvState {
    double f, alpha, mu;
    int done, pad;
};

struct TvVecs {
    float *u, *up, *rhs, *b1, *b2, *d1, *d2, *x, *r, *rt, *uc, *p, *q, *vh, *uh, *xmin;
};

// sum over the block; every thread gets the result
__device__ double tv_block_sum(double v, double *sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();  // sh may still be read from the previous call
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    if (wid == 0) {
        v = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) sh[32] = v;
    }
    __syncthreads();
    return sh[32];
}

__device__ double tv_dot(const float *a, const float *b, int P, double *sh) {
    float acc = 0.f;
    for (int i = threadIdx.x; i < P; i += blockDim.x) acc = fmaf(a[i], b[i], acc);
    return tv_block_sum((double)acc, sh);
}

// out = (I + B'B) in
__device__ void tv_apply_M(const float *in, float *out, int N) {
    const int P = N * N;
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
        const int ix = i / N, iz = i - ix * N;
        const float c = in[i];
        const float g1 = iz >= 1 ? c - in[i - 1] : 0.f;     // (B1 u)(ix, iz)
        const float g1n = iz + 1 < N ? in[i + 1] - c : 0.f;  // (B1 u)(ix, iz + 1)
        const float g2 = ix >= 1 ? c - in[i - N] : 0.f;     // (B2 u)(ix, iz)
        const float g2n = ix + 1 < N ? in[i + N] - c : 0.f;  // (B2 u)(ix + 1, iz)
        out[i] = c + (g1 - g1n) + (g2 - g2n);
    }
    __syncthreads();
}

// u = cgs(I + B'B, rhs, tol, TV_CG_MAX) from x0 = 0 (Sonneveld's CGS with the
// recursively updated residual; the smallest-residual iterate when it does
// not converge, as MATLAB's cgs returns)
__device__ void tv_cgs(const TvVecs &V, int N, float tol, double *sh) {
    const int P = N * N;
    const double n2b = sqrt(tv_dot(V.rhs, V.rhs, P, sh));
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
        V.x[i] = 0.f;
        V.xmin[i] = 0.f;
        V.r[i] = V.rhs[i];
        V.rt[i] = V.rhs[i];
    }
    __syncthreads();
    bool converged = false;
    if (n2b > 0.0) {
        double normrmin = n2b, rho = 1.0;
        for (int it = 0; it < TV_CG_MAX; ++it) {
            const double rho1 = rho;
            rho = tv_dot(V.rt, V.r, P, sh);
            if (rho == 0.0 || !isfinite(rho)) break;
            const float beta = it ? (float)(rho / rho1) : 0.f;
            for (int i = threadIdx.x; i < P; i += blockDim.x) {
                if (it == 0) {
                    V.uc[i] = V.r[i];
                    V.p[i] = V.r[i];
                } else {
                    const float u = fmaf(beta, V.q[i], V.r[i]);
                    V.uc[i] = u;
                    V.p[i] = fmaf(beta, fmaf(beta, V.p[i], V.q[i]), u);
                }
            }
            __syncthreads();
            tv_apply_M(V.p, V.vh, N);
            const double rtvh = tv_dot(V.rt, V.vh, P, sh);
            if (rtvh == 0.0 || !isfinite(rtvh)) break;
            const float alpha = (float)(rho / rtvh);
            for (int i = threadIdx.x; i < P; i += blockDim.x) {
                const float qq = fmaf(-alpha, V.vh[i], V.uc[i]);
                V.q[i] = qq;
                const float uh = V.uc[i] + qq;
                V.uh[i] = uh;
                V.x[i] = fmaf(alpha, uh, V.x[i]);
            }
            __syncthreads();
            tv_apply_M(V.uh, V.vh, N);  // vh is free again: holds M uh
            for (int i = threadIdx.x; i < P; i += blockDim.x)
                V.r[i] = fmaf(-alpha, V.vh[i], V.r[i]);
            __syncthreads();
            const double normr = sqrt(tv_dot(V.r, V.r, P, sh));
            if (normr <= (double)tol * n2b) {
                converged = true;
                break;
            }
            if (normr < normrmin) {
                normrmin = normr;
                for (int i = threadIdx.x; i < P; i += blockDim.x) V.xmin[i] = V.x[i];
                __syncthreads();
            }
        }
    }
    const float *src = converged ? V.x : V.xmin;
    for (int i = threadIdx.x; i < P; i += blockDim.x) V.u[i] = src[i];
    __syncthreads();
}

// out[w] = SB_ITV2(g[w], mu): mu = st[group].mu for the groups not stopped,
// or mu_const when st is null
__global__ void __launch_bounds__(TV_THREADS)
    k_tv_prox(const float *__restrict__ g_all, const TvState *__restrict__ st, double mu_const,
              int coupled, float *__restrict__ out_all, float *__restrict__ work, int N) {
    __shared__ double sh[33];
    const int w = blockIdx.x, gw = coupled ? 0 : w;
    if (st && st[gw].done) return;
    const int P = N * N;
    float *base = work + (size_t)w * TV_NVEC * P;
    TvVecs V;
    float **fields[TV_NVEC] = {&V.u,  &V.up, &V.rhs, &V.b1, &V.b2, &V.d1, &V.d2, &V.x,
                               &V.r,  &V.rt, &V.uc,  &V.p,  &V.q,  &V.vh, &V.uh, &V.xmin};
    for (int k = 0; k < TV_NVEC; ++k) *fields[k] = base + (size_t)k * P;
    const float *g = g_all + (size_t)w * P;
    const float mu = (float)(st ? st[gw].mu : mu_const);
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
        V.u[i] = g[i];
        V.b1[i] = V.b2[i] = V.d1[i] = V.d2[i] = 0.f;
    }
    __syncthreads();
    for (int it = 0; it < TV_SB_MAX; ++it) {
        // up = u ; rhs = g - B'(b - d)
        for (int i = threadIdx.x; i < P; i += blockDim.x) {
            const int ix = i / N, iz = i - ix * N;
            V.up[i] = V.u[i];
            const float c1 = iz >= 1 ? V.b1[i] - V.d1[i] : 0.f;
            const float c1n = iz + 1 < N ? V.b1[i + 1] - V.d1[i + 1] : 0.f;
            const float c2 = ix >= 1 ? V.b2[i] - V.d2[i] : 0.f;
            const float c2n = ix + 1 < N ? V.b2[i + N] - V.d2[i + N] : 0.f;
            V.rhs[i] = g[i] - ((c1 - c1n) + (c2 - c2n));
        }
        __syncthreads();
        tv_cgs(V, N, 1e-5f, sh);
        // Bub = B u + b ; d = shrink(Bub, mu) ; b = Bub - d
        float dif = 0.f, nrm = 0.f;
        for (int i = threadIdx.x; i < P; i += blockDim.x) {
            const int ix = i / N, iz = i - ix * N;
            const float c = V.u[i];
            const float a1 = (iz >= 1 ? c - V.u[i - 1] : 0.f) + V.b1[i];
            const float a2 = (ix >= 1 ? c - V.u[i - N] : 0.f) + V.b2[i];
            const float s = sqrtf(fmaf(a1, a1, a2 * a2));
            const float f = s > 0.f ? fmaxf(s - mu, 0.f) / s : 0.f;
            V.d1[i] = f * a1;
            V.d2[i] = f * a2;
            V.b1[i] = a1 - f * a1;
            V.b2[i] = a2 - f * a2;
            const float e = V.up[i] - c;
            dif = fmaf(e, e, dif);
            nrm = fmaf(c, c, nrm);
        }
        const double d2 = tv_block_sum((double)dif, sh);
        const double n2 = tv_block_sum((double)nrm, sh);
        if (!(n2 > 0.0) || sqrt(d2 / n2) <= 1e-3) break;
    }
    float *o = out_all + (size_t)w * P;
    for (int i = threadIdx.x; i < P; i += blockDim.x) o[i] = V.u[i];
}

// isotropic TV term of pixel i of the N x N image x
__device__ __forceinline__ float itv_term(const float *x, int i, int N) {
    if (N == 1) return 0.f;
    const int ix = i / N, iz = i - ix * N;
    const float gx = ix == 0 ? x[i + N] - x[i]
                             : (ix == N - 1 ? x[i] - x[i - N] : 0.5f * (x[i + N] - x[i - N]));
    const float gz = iz == 0 ? x[i + 1] - x[i]
                             : (iz == N - 1 ? x[i] - x[i - 1] : 0.5f * (x[i + 1] - x[i - 1]));
    return sqrtf(fmaf(gx, gx, gz * gz));
}

// ---------------------------------------------------------------------------
// SpaRSA on A_aug = [sqrt(lambda) A; sqrt(beta) I], y = [sqrt(lambda) b;
// sqrt(beta) (w + v)], lambda = 1.  The residual is kept split: rs (sinogram
// part) and ri (image part).  Partial sums go to part[q][w][gridDim.x].
// ---------------------------------------------------------------------------
enum TvSum { TS_RS = 0, TS_RI, TS_PHI, TS_DX, TS_AS, TS_N };


__device__ __forceinline__ void tv_store(double v, double *part, int q, int W, double *sh) {
    const double s = tv_block_sum(v, sh);
    if (threadIdx.x == 0) part[((size_t)q * W + blockIdx.y) * gridDim.x + blockIdx.x] = s;
}

#define TV_FOR(n)                                                                          \
    const int w = blockIdx.y;                                                              \
    const size_t base = (size_t)w * (n);                                                   \
    for (size_t i = (size_t)blockIdx.x * TV_RED + threadIdx.x; i < (size_t)(n);            \
         i += (size_t)gridDim.x * TV_RED)

// x = w ; ri = sb (w + v - x) = sb v ; sums ri^2, ITV(x)
__global__ void __launch_bounds__(TV_RED)
    k_tv_begin(const float *__restrict__ wv, const float *__restrict__ vm, float *__restrict__ x,
               float *__restrict__ ri, int N, float sb, int W, double *part) {
    __shared__ double sh[33];
    const size_t P = (size_t)N * N;
    float a_ri = 0.f, a_phi = 0.f;
    TV_FOR(P) {
        const size_t k = base + i;
        x[k] = wv[k];
        const float r = sb * vm[k];
        ri[k] = r;
        a_ri = fmaf(r, r, a_ri);
        a_phi += itv_term(wv + base, (int)i, N);
    }
    tv_store(a_ri, part, TS_RI, W, sh);
    tv_store(a_phi, part, TS_PHI, W, sh);
}

// rs = sl (b - A x) ; sums rs^2
__global__ void __launch_bounds__(TV_RED)
    k_tv_rs0(const float *__restrict__ b, const float *__restrict__ Ax, float *__restrict__ rs,
             size_t n, float sl, int W, double *part) {
    __shared__ double sh[33];
    float a = 0.f;
    TV_FOR(n) {
        const size_t k = base + i;
        const float r = sl * (b[k] - Ax[k]);
        rs[k] = r;
        a = fmaf(r, r, a);
    }
    tv_store(a, part, TS_RS, W, sh);
}

// z = x + (sl A' rs + sb ri) / alpha   (= x - grad / alpha)
__global__ void __launch_bounds__(TV_RED)
    k_tv_z(const float *__restrict__ x, const float *__restrict__ atr, const float *__restrict__ ri,
           const TvState *__restrict__ st, int coupled, float *__restrict__ z, size_t P, float sl,
           float sb) {
    const int gw = coupled ? 0 : (int)blockIdx.y;
    if (st[gw].done) return;
    const float ia = (float)(1.0 / st[gw].alpha);
    TV_FOR(P) {
        const size_t k = base + i;
        z[k] = fmaf(fmaf(sl, atr[k], sb * ri[k]), ia, x[k]);
    }
}

// dx = x+ - x ; ri -= sb dx ; x = x+ ; sums dx^2, ri^2, ITV(x+).  Stopped
// instances keep x (dx = 0).
__global__ void __launch_bounds__(TV_RED)
    k_tv_step(float *__restrict__ x, const float *__restrict__ xn, float *__restrict__ ri,
              float *__restrict__ dx, const TvState *__restrict__ st, int coupled, int N, float sb,
              int W, double *part) {
    __shared__ double sh[33];
    const size_t P = (size_t)N * N;
    const bool done = st[coupled ? 0 : (int)blockIdx.y].done;
    const float *src = done ? x : xn;
    float a_dx = 0.f, a_ri = 0.f, a_phi = 0.f;
    TV_FOR(P) {
        const size_t k = base + i;
        const float d = done ? 0.f : xn[k] - x[k];
        dx[k] = d;
        const float r = fmaf(-sb, d, ri[k]);
        ri[k] = r;
        a_dx = fmaf(d, d, a_dx);
        a_ri = fmaf(r, r, a_ri);
        a_phi += itv_term(src + base, (int)i, N);
        if (!done) x[k] = xn[k];
    }
    tv_store(a_dx, part, TS_DX, W, sh);
    tv_store(a_ri, part, TS_RI, W, sh);
    tv_store(a_phi, part, TS_PHI, W, sh);
}

// rs -= sl A dx ; sums rs^2, (A dx)^2
__global__ void __launch_bounds__(TV_RED)
    k_tv_rs(float *__restrict__ rs, const float *__restrict__ Adx, size_t n, float sl, int W,
            double *part) {
    __shared__ double sh[33];
    float a_rs = 0.f, a_as = 0.f;
    TV_FOR(n) {
        const size_t k = base + i;
        const float ad = Adx[k];
        const float r = fmaf(-sl, ad, rs[k]);
        rs[k] = r;
        a_rs = fmaf(r, r, a_rs);
        a_as = fmaf(ad, ad, a_as);
    }
    tv_store(a_rs, part, TS_RS, W, sh);
    tv_store(a_as, part, TS_AS, W, sh);
}

__device__ double tv_group(const double *part, int q, int g, int W, int G, int coupled) {
    const int w0 = coupled ? 0 : g, w1 = coupled ? W : g + 1;
    double s = 0.0;
    for (int w = w0; w < w1; ++w)
        for (int k = 0; k < G; ++k) s += part[((size_t)q * W + w) * G + k];
    return s;
}

// stage 0: objective of the start point, alpha = 1.
// stage 1: after a step: new objective, BB alpha, stop test (StopCriterion 1).
__global__ void k_tv_scalar(int stage, const double *part, int G, int W, int coupled, double tau,
                            double lambda, double beta, double tol, TvState *st) {
    const int n = coupled ? 1 : W;
    for (int g = threadIdx.x; g < n; g += blockDim.x) {
        TvState &s = st[g];
        if (stage == 1 && s.done) continue;
        const double f = 0.5 * (tv_group(part, TS_RS, g, W, G, coupled) +
                                tv_group(part, TS_RI, g, W, G, coupled)) +
                         tau * tv_group(part, TS_PHI, g, W, G, coupled);
        if (stage == 0) {
            s.f = f;
            s.alpha = 1.0;
            s.done = 0;
        } else {
            const double prev = s.f;
            s.f = f;
            const double dd = tv_group(part, TS_DX, g, W, G, coupled);
            const double dgd = lambda * tv_group(part, TS_AS, g, W, G, coupled) + beta * dd;
            const double a = dgd / (2.2250738585072014e-308 + dd);  // realmin guard
            s.alpha = fmin(1e30, fmax(1e-30, a));
            if (dd == 0.0 || fabs(f - prev) <= tol * fabs(prev)) s.done = 1;
        }
        s.mu = tau / s.alpha;
    }
}

// w = max(x - v, 0) ; v += w - x
__global__ void k_tv_outer(const float *__restrict__ x, float *__restrict__ wv,
                           float *__restrict__ vm, size_t n) {
    for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (size_t)gridDim.x * blockDim.x) {
        const float u = x[k];
        const float wn = fmaxf(u - vm[k], 0.f);
        wv[k] = wn;
        vm[k] += wn - u;
    }
}

// per-instance sum of (a - b)^2 (b may be null), or of ITV(a) when itv_n > 0
__global__ void __launch_bounds__(TV_RED)
    k_tv_sum(const float *__restrict__ a, const float *__restrict__ b, size_t n, int itv_n,
             int W, double *part) {
    __shared__ double sh[33];
    float acc = 0.f;
    TV_FOR(n) {
        if (itv_n) {
            acc += itv_term(a + base, (int)i, itv_n);
        } else {
            const float v = a[base + i] - (b ? b[base + i] : 0.f);
            acc = fmaf(v, v, acc);
        }
    }
    tv_store(acc, part, 0, W, sh);
}

__global__ void k_tv_fold(const double *part, int G, int W, double *out) {
    for (int w = threadIdx.x; w < W; w += blockDim.x) {
        double s = 0.0;
        for (int k = 0; k < G; ++k) s += part[(size_t)w * G + k];
        out[w] = s;
    }
}

}  // namespace msot

using namespace msot;

namespace {

struct DevBufs {
    std::vector<void *> v;
    bool ok = true;
    ~DevBufs() {
        for (void *p : v) cudaFree(p);
    }
    template <class T>
    T *get(size_t n) {
        void *p = nullptr;
        if (cudaMalloc(&p, (n ? n : 1) * sizeof(T)) != cudaSuccess) {
            ok = false;
            return nullptr;
        }
        v.push_back(p);
        return static_cast<T *>(p);
    }
};

int blocks_per_instance(int W) { return std::max(1, std::min(64, (4 * 152 + W - 1) / W)); }

// per-instance sums of (a - b)^2 or ITV(a), copied to the host
int tv_sums(const float *a, const float *b, size_t n, int itv_n, int W, double *part,
            double *dout, std::vector<double> &h, cudaStream_t st) {
    const int G = blocks_per_instance(W);
    KLAUNCH(k_tv_sum<<<dim3(G, W), TV_RED, 0, st>>>(a, b, n, itv_n, W, part));
    KLAUNCH(k_tv_fold<<<1, 256, 0, st>>>(part, G, W, dout));
    MSOT_LAUNCH_CHECK();
    h.resize(W);
    MSOT_CUDA_TRY(cudaMemcpyAsync(h.data(), dout, sizeof(double) * W, cudaMemcpyDeviceToHost, st));
    MSOT_CUDA_TRY(cudaStreamSynchronize(st));
    return MSOT_OK;
}

}  // namespace

extern "C" {

int msot_sb_itv2(const float *d_g, float *d_u, int batch, int n, double mu, void *stream) {
    if (!d_g || !d_u || batch <= 0 || n <= 0 || !(mu >= 0.0)) {
        set_error("sb_itv2: bad arguments");
        return MSOT_EINVAL;
    }
    cudaStream_t st = (cudaStream_t)stream;
    DevBufs b;
    const size_t P = (size_t)n * n;
    float *work = b.get<float>((size_t)batch * TV_NVEC * P);
    if (!b.ok) {
        set_error("sb_itv2: device allocation failed");
        return MSOT_ENOMEM;
    }
    KLAUNCH(k_tv_prox<<<batch, TV_THREADS, 0, st>>>(d_g, nullptr, mu, 1, d_u, work, n));
    MSOT_LAUNCH_CHECK();
    MSOT_CUDA_TRY(cudaStreamSynchronize(st));
    return MSOT_OK;
}

int msot_itv(const float *d_x, double *itv, int batch, int n, void *stream) {
    if (!d_x || !itv || batch <= 0 || n <= 0) {
        set_error("itv: bad arguments");
        return MSOT_EINVAL;
    }
    cudaStream_t st = (cudaStream_t)stream;
    DevBufs b;
    const int G = blocks_per_instance(batch);
    double *part = b.get<double>((size_t)G * batch), *dout = b.get<double>(batch);
    if (!b.ok) {
        set_error("itv: device allocation failed");
        return MSOT_ENOMEM;
    }
    std::vector<double> h;
    int rc = tv_sums(d_x, nullptr, (size_t)n * n, n, batch, part, dout, h, st);
    if (rc) return rc;
    for (int w = 0; w < batch; ++w) itv[w] = h[w];
    return MSOT_OK;
}

int msot_rec_nn_with_TV_reg(msot_plan_t plan, const float *d_b, float *d_rec, int batch,
                            int num_iter, double reg, int sparsa_iter, const float *d_x0,
                            int coupled, double *err_img, double *err_reg, void *stream) {
    if (!plan || !d_b || !d_rec || batch <= 0 || num_iter < 0 || sparsa_iter < 1 ||
        !(reg >= 0.0)) {
        set_error("rec_nn_with_TV_reg: bad arguments");
        return MSOT_EINVAL;
    }
    const Plan &pl = plan->p;
    if (pl.nx != pl.nz) {
        set_error("This TV implementation works only with square images!");
        return MSOT_EINVAL;
    }
    if (batch > pl.max_batch) {
        set_error("rec_nn_with_TV_reg: batch %d exceeds the plan's max_batch %d", batch,
                  pl.max_batch);
        return MSOT_EINVAL;
    }
    cudaStream_t st = (cudaStream_t)stream;
    const int W = batch, N = pl.nx, G = blocks_per_instance(W);
    const size_t P = pl.P, NI = (size_t)W * P, ns = (size_t)pl.D * pl.T, NS = (size_t)W * ns;
    DevBufs bf;
    float *work = bf.get<float>((size_t)W * TV_NVEC * P);
    float *wv = bf.get<float>(NI), *vm = bf.get<float>(NI), *x = bf.get<float>(NI);
    float *xn = bf.get<float>(NI), *z = bf.get<float>(NI), *ri = bf.get<float>(NI);
    float *atr = bf.get<float>(NI), *dx = bf.get<float>(NI);
    float *rs = bf.get<float>(NS), *As = bf.get<float>(NS);
    double *part = bf.get<double>((size_t)TS_N * W * G), *dout = bf.get<double>(W);
    TvState *sv = bf.get<TvState>(W);
    if (!bf.ok) {
        set_error("rec_nn_with_TV_reg: device allocation failed");
        return MSOT_ENOMEM;
    }
    const float sl = 1.f, sb = (float)std::sqrt(TV_BETA);
    const dim3 grid(G, W);
    const unsigned go = (unsigned)std::min<size_t>((NI + 255) / 256, 4096);
    int rc = MSOT_OK;
#define TV_CK(expr)                                                                        \
    if ((rc = (expr)) != MSOT_OK) return rc
    if (d_x0)
        MSOT_CUDA_TRY(cudaMemcpyAsync(wv, d_x0, NI * sizeof(float), cudaMemcpyDeviceToDevice, st));
    else
        MSOT_CUDA_TRY(cudaMemsetAsync(wv, 0, NI * sizeof(float), st));
    MSOT_CUDA_TRY(cudaMemsetAsync(vm, 0, NI * sizeof(float), st));
    for (int outer = 0; outer < num_iter; ++outer) {
        KLAUNCH(k_tv_begin<<<grid, TV_RED, 0, st>>>(wv, vm, x, ri, N, sb, W, part));
        MSOT_LAUNCH_CHECK();
        TV_CK(apply_forward(pl, x, As, W, st));
        KLAUNCH(k_tv_rs0<<<grid, TV_RED, 0, st>>>(d_b, As, rs, ns, sl, W, part));
        KLAUNCH(k_tv_scalar<<<1, 64, 0, st>>>(0, part, G, W, coupled, reg, 1.0, TV_BETA, 1e-8, sv));
        MSOT_LAUNCH_CHECK();
        for (int k = 0; k < sparsa_iter; ++k) {
            TV_CK(apply_transpose(pl, rs, atr, W, st));
            KLAUNCH(k_tv_z<<<grid, TV_RED, 0, st>>>(x, atr, ri, sv, coupled, z, P, sl, sb));
            {
                TimedScope ts(KID_TV_PROX, st);
                KLAUNCH(k_tv_prox<<<W, TV_THREADS, 0, st>>>(z, sv, 0.0, coupled, xn, work, N));
            }
            MSOT_LAUNCH_CHECK();
            KLAUNCH(k_tv_step<<<grid, TV_RED, 0, st>>>(x, xn, ri, dx, sv, coupled, N, sb, W, part));
            MSOT_LAUNCH_CHECK();
            TV_CK(apply_forward(pl, dx, As, W, st));
            KLAUNCH(k_tv_rs<<<grid, TV_RED, 0, st>>>(rs, As, ns, sl, W, part));
            KLAUNCH(k_tv_scalar<<<1, 64, 0, st>>>(1, part, G, W, coupled, reg, 1.0, TV_BETA, 1e-8, sv));
            MSOT_LAUNCH_CHECK();
        }
        KLAUNCH(k_tv_outer<<<go, 256, 0, st>>>(x, wv, vm, NI));
        MSOT_LAUNCH_CHECK();
    }
    MSOT_CUDA_TRY(cudaMemcpyAsync(d_rec, wv, NI * sizeof(float), cudaMemcpyDeviceToDevice, st));
    if (err_img || err_reg) {
        std::vector<double> h;
        if (err_img) {
            TV_CK(apply_forward(pl, wv, As, W, st));
            TV_CK(tv_sums(As, d_b, ns, 0, W, part, dout, h, st));
            for (int w = 0; w < W; ++w) err_img[w] = h[w];
        }
        if (err_reg) {
            TV_CK(tv_sums(wv, nullptr, P, N, W, part, dout, h, st));
            for (int w = 0; w < W; ++w) err_reg[w] = h[w];
        }
    }
    MSOT_CUDA_TRY(cudaStreamSynchronize(st));
#undef TV_CK
    return MSOT_OK;
}

}  // extern "C"
