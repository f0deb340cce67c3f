// solver.cu -- batched non-negative solvers on the GPU.
//
// FP32 vectors and element-wise arithmetic; inner products and norms are
// FP64 sums of per-thread FP32 partial sums (each thread adds at most a few
// dozen elements in FP32), and every Krylov scalar, step size and stopping
// test is FP64.  A batch of W instances is
// solved at once; each instance owns its Krylov scalars (independent
// reconstructions), or the whole batch shares one set (coupled = the W
// wavelengths of one reference call, whose lsqr/cgs see one stacked vector).
//
//   rec_nn_with_L2_reg  -> rec_nn_with_L2_reg.m:24-63, nnls_L2_less.m:27-101,
//                          lsqr (Paige & Saunders) on [sqrt(lam) [A; sqrt(lamL2) I];
//                          sqrt(beta) I] with maxit 2, x0 = w, tol 1e-8.
//   rec_nn_with_L1_eye  -> rec_nn_with_L1_eye_reg.m:21-47,
//                          nnls_L1_eye_matrix_less.m:26-65, cgs on lam A^T A + I.
//   estimate_norm       -> the sigma_max of MSOTmodel.m:277-278 by power
//                          iteration.
#include <cmath>
#include <vector>

#include "common.cuh"

namespace msot {

constexpr int RED_THREADS = 256;

__device__ __forceinline__ double block_sum(double v) {
    __shared__ double sh[RED_THREADS / 32];
    __syncthreads();  // sh may still be read by a previous call
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    if (wid == 0) {
        v = lane < RED_THREADS / 32 ? sh[lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    }
    return v;  // valid in thread 0
}

// grid (nblk, W); each block reduces a strided chunk of instance w.
#define FOR_CHUNK(N)                                                                       \
    const int w = blockIdx.y;                                                              \
    const size_t base = (size_t)w * (N);                                                   \
    for (size_t i = (size_t)blockIdx.x * RED_THREADS + threadIdx.x; i < (size_t)(N);       \
         i += (size_t)gridDim.x * RED_THREADS)

#define STORE_PARTIAL(v, part)                                                             \
    {                                                                                      \
        double s_ = block_sum(v);                                                          \
        if (threadIdx.x == 0) (part)[(size_t)w * gridDim.x + blockIdx.x] = s_;             \
    }

__device__ __forceinline__ int grp(int w, int coupled) { return coupled ? 0 : w; }

// u = a*x + b*u with per-group scalars; partial sums of u^2.
// mode 0: u = sl*b_vec - sl*x          (LSQR init, sinogram part)
// mode 1: u = sl*x - gamma*u           (LSQR step, sinogram part)
__global__ void k_sino_update(const float *__restrict__ x, const float *__restrict__ bvec,
                              float *__restrict__ u, size_t N, int mode, double sl,
                              const Scal *__restrict__ sc, int coupled, double *part) {
    float facc = 0.f;
    const float slf = (float)sl;
    const float g = (float)sc[grp(blockIdx.y, coupled)].gamma;
    const bool done = mode == 1 && sc[grp(blockIdx.y, coupled)].done;
    FOR_CHUNK(N) {
        const size_t k = base + i;
        float v;
        if (mode == 0) {
            v = fmaf(slf, bvec[k], -slf * x[k]);
        } else {
            v = fmaf(slf, x[k], -g * u[k]);
            if (done) v = u[k];
        }
        u[k] = v;
        facc = fmaf(v, v, facc);
    }
    STORE_PARTIAL((double)facc, part);
}

// generic sum of squares of (x - y) (y may be null) per instance
__global__ void k_sumsq(const float *__restrict__ x, const float *__restrict__ y, size_t N,
                        double *part) {
    float facc = 0.f;
    FOR_CHUNK(N) {
        const float v = x[base + i] - (y ? y[base + i] : 0.f);
        facc = fmaf(v, v, facc);
    }
    STORE_PARTIAL((double)facc, part);
}

// LSQR init, image parts: ur = -sl*sr*w ; ub = sb*(w+vm) - sb*w.
// part: sum ur^2 + ub^2 ; part2: sum (w+vm)^2 (for ||b_aug||).
// (lw, ul: the Laplacian block, u_lap = -sl*sr2*del2(w); null without it)
__global__ void k_l2_init_img(const float *__restrict__ wv, const float *__restrict__ vm,
                              float *__restrict__ ur, float *__restrict__ ub, size_t N,
                              double sl, double sr, double sb, int has_reg, double *part,
                              double *part2, const float *__restrict__ lw,
                              float *__restrict__ ul, double sr2) {
    float a1 = 0.f, a2 = 0.f;
    const float c_r = (float)(-sl * sr), c_b = (float)sb, c_l2 = (float)(-sl * sr2);
    FOR_CHUNK(N) {
        const size_t k = base + i;
        const float wd = wv[k], s = wd + vm[k];
        const float r = c_r * wd;
        const float bb = fmaf(c_b, s, -c_b * wd);
        if (has_reg) ur[k] = r;
        ub[k] = bb;
        a1 = fmaf(bb, bb, has_reg ? fmaf(r, r, a1) : a1);
        a2 = fmaf(s, s, a2);
        if (lw) {
            const float r2 = c_l2 * lw[k];
            ul[k] = r2;
            a1 = fmaf(r2, r2, a1);
        }
    }
    STORE_PARTIAL((double)a1, part);
    STORE_PARTIAL((double)a2, part2);
}

// LSQR step, image parts: ur = sl*sr*v - gamma*ur ; ub = sb*v - gamma*ub
// (lv = del2(v), ul: the Laplacian block u_lap = sl*sr2*del2(v) - gamma*u_lap)
__global__ void k_l2_u_img(const float *__restrict__ v, float *__restrict__ ur,
                           float *__restrict__ ub, size_t N, double sl, double sr, double sb,
                           int has_reg, const Scal *__restrict__ sc, int coupled,
                           double *part, const float *__restrict__ lv, float *__restrict__ ul,
                           double sr2) {
    float acc = 0.f;
    const Scal &q = sc[grp(blockIdx.y, coupled)];
    const float g = (float)q.gamma, c_r = (float)(sl * sr), c_b = (float)sb;
    const float c_l2 = (float)(sl * sr2);
    const bool done = q.done;
    FOR_CHUNK(N) {
        const size_t k = base + i;
        const float vd = v[k];
        float r = has_reg ? ur[k] : 0.f, bb = ub[k], r2 = lv ? ul[k] : 0.f;
        if (!done) {
            r = fmaf(c_r, vd, -g * r);
            bb = fmaf(c_b, vd, -g * bb);
            if (has_reg) ur[k] = r;
            ub[k] = bb;
            if (lv) {
                r2 = fmaf(c_l2, lv[k], -g * r2);
                ul[k] = r2;
            }
        }
        acc = fmaf(bb, bb, fmaf(r, r, fmaf(r2, r2, acc)));
    }
    STORE_PARTIAL((double)acc, part);
}

// vt = (sl*(At_us + sr*ur) + sb*ub) / beta ; v = vt - beta*v_old (first: v_old = 0)
// (lul = del2(u_lap): the Laplacian block's transpose, as the reference
// passes it, adds sl*sr2*del2(u_lap))
__global__ void k_l2_v_img(const float *__restrict__ atu, const float *__restrict__ ur,
                           const float *__restrict__ ub, float *__restrict__ v, size_t N,
                           double sl, double sr, double sb, int has_reg, int first,
                           const Scal *__restrict__ sc, int coupled, double *part,
                           const float *__restrict__ lul, double sr2) {
    float acc = 0.f;
    const Scal &q = sc[grp(blockIdx.y, coupled)];
    const bool done = q.done;
    const float ib = (float)(1.0 / q.beta), be = (float)q.beta;
    const float c_l = (float)sl, c_r = (float)(sl * sr), c_b = (float)sb;
    const float c_l2 = (float)(sl * sr2);
    FOR_CHUNK(N) {
        const size_t k = base + i;
        float vv = v[k];
        if (!done) {
            float reg = has_reg ? c_r * ur[k] : 0.f;
            if (lul) reg = fmaf(c_l2, lul[k], reg);
            float vt = fmaf(c_l, atu[k], fmaf(c_b, ub[k], reg)) * ib;
            if (!first) vt = fmaf(-be, vv, vt);
            vv = vt;
            v[k] = vv;
        }
        acc = fmaf(vv, vv, acc);
    }
    STORE_PARTIAL((double)acc, part);
}

// MATLAB del2(U, 1) of every image [W][nx][nz] (z fastest): (the second
// differences along z + along x) / 4, the end values of each line
// extrapolated linearly from the interior (n > 3), copied (n == 3), zero
// (n < 3) -- laplacian_per_wavelength.m:4-8
__device__ __forceinline__ float del2_line(const float *u, int i, int n, int stride) {
    if (n < 3) return 0.f;
    auto D = [&](int k) { return u[(k + 1) * stride] - 2.f * u[k * stride] + u[(k - 1) * stride]; };
    if (i > 0 && i < n - 1) return D(i);
    if (n == 3) return D(1);
    return i == 0 ? 2.f * D(1) - D(2) : 2.f * D(n - 2) - D(n - 3);
}
__global__ void k_del2(const float *__restrict__ in, float *__restrict__ out, int nx, int nz) {
    const size_t N = (size_t)nx * nz;
    FOR_CHUNK(N) {
        const int ix = (int)(i / nz), iz = (int)(i % nz);
        const float *img = in + base;
        const float gz = del2_line(img + (size_t)ix * nz, iz, nz, 1);
        const float gx = del2_line(img + iz, ix, nx, nz);
        out[base + i] = 0.25f * (gx + gz);
    }
}

// Sum of the partials of group g, computed by the whole warp (lane-strided,
// then a butterfly): every lane returns the same value.  The scalar kernels
// below give each warp a group and let lane 0 run the scalar logic; a
// thread-serial FP64 sum over hundreds of partials is slow on GB300.
__device__ double group_sum(const double *p1, int n1, const double *p2, int n2, int g,
                            int W, int coupled) {
    const int lane = threadIdx.x & 31;
    double s = 0.0;
    const int w0 = coupled ? 0 : g, w1 = coupled ? W : g + 1;
    for (int w = w0; w < w1; ++w) {
        if (p1)
            for (int b = lane; b < n1; b += 32) s += p1[(size_t)w * n1 + b];
        if (p2)
            for (int b = lane; b < n2; b += 32) s += p2[(size_t)w * n2 + b];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    return s;
}

#define FOR_GROUP_WARP(G)                                                                  \
    for (int g = (int)(threadIdx.x >> 5); g < (G); g += (int)(blockDim.x >> 5))
#define LANE0_ONLY                                                                         \
    if ((threadIdx.x & 31) != 0) continue

// stage 0: beta after init; stage 1: alpha (init or step); stage 2: LSQR step scalars
__global__ void k_l2_scalar(Scal *sc, int stage, const double *p1, int n1, const double *p2,
                            int n2, const double *p3, int n3, const double *normb2_sino,
                            double sl, double sb, int W, int coupled, double tol) {
    const int G = coupled ? 1 : W;
    FOR_GROUP_WARP(G) {
        Scal &q = sc[g];
        if (stage == 0) {
            const double b2 = group_sum(p1, n1, p2, n2, g, W, coupled);
            const double wv2 = group_sum(p3, n3, nullptr, 0, g, W, coupled);
            LANE0_ONLY;
            q.normb = sqrt(sl * sl * normb2_sino[g] + sb * sb * wv2);
            q.beta = sqrt(b2);
            q.normr = q.beta;
            q.normrmin = q.beta;
            q.phibar = q.beta;
            q.c = 1.0;
            q.s = 0.0;
            q.done = !(q.beta > 0.0) || !isfinite(q.beta);
            q.improved = 0;
        } else if (stage == 1) {
            const double a2 = group_sum(p1, n1, nullptr, 0, g, W, coupled);
            LANE0_ONLY;
            if (!q.done) {
                q.alpha = sqrt(a2);
                if (!(q.alpha > 0.0) || !isfinite(q.alpha)) q.done = 1;
            }
        } else {
            const double b2 = group_sum(p1, n1, p2, n2, g, W, coupled);
            LANE0_ONLY;
            q.improved = 0;
            if (q.done) continue;
            const double beta = sqrt(b2);
            const double thet = -q.s * q.alpha;
            const double rhot = q.c * q.alpha;
            const double rho = sqrt(rhot * rhot + beta * beta);
            if (!(rho > 0.0) || !isfinite(rho)) {
                q.done = 1;
                continue;
            }
            q.c = rhot / rho;
            q.s = -beta / rho;
            q.phi = q.c * q.phibar;
            q.phibar = q.s * q.phibar;
            q.rho = rho;
            q.thet = thet;
            q.beta = beta;
            q.normr = fabs(q.s) * q.normr;
            q.improved = 2;  // x is updated this step (2 = update x, no xmin copy)
            if (q.normr < q.normrmin) {
                q.normrmin = q.normr;
                q.improved = 1;  // update x and xmin
            }
            if (q.normr <= tol * q.normb) q.improved = 3;  // converged: x is final
        }
    }
}

// gamma = alpha / beta for the next u update
__global__ void k_l2_gamma(Scal *sc, int G) {
    for (int g = threadIdx.x; g < G; g += blockDim.x) sc[g].gamma = sc[g].alpha / sc[g].beta;
}

// v /= alpha ; on init also d = 0, x = w, xmin = w
__global__ void k_l2_scale_v(float *v, float *d, float *x, float *xmin, const float *wv,
                             size_t N, int init, const Scal *sc, int coupled) {
    FOR_CHUNK(N) {
        const size_t k = base + i;
        const Scal &q = sc[grp(w, coupled)];
        if (init) {
            d[k] = 0.f;
            x[k] = wv[k];
            xmin[k] = wv[k];
        }
        if (!q.done) v[k] = v[k] * (float)(1.0 / q.alpha);
    }
}

// d = (v - thet*d)/rho ; x += phi*d ; xmin = x when improved
__global__ void k_l2_dx(const float *v, float *d, float *x, float *xmin, size_t N, Scal *sc,
                        int coupled) {
    FOR_CHUNK(N) {
        const size_t k = base + i;
        const Scal &q = sc[grp(w, coupled)];
        if (q.done || q.improved == 0) continue;
        const float dn = fmaf(-(float)q.thet, d[k], v[k]) * (float)(1.0 / q.rho);
        d[k] = dn;
        const float xn = fmaf((float)q.phi, dn, x[k]);
        x[k] = xn;
        if (q.improved != 2) xmin[k] = xn;
    }
}

__global__ void k_l2_mark_converged(Scal *sc, int G) {
    for (int g = threadIdx.x; g < G; g += blockDim.x)
        if (sc[g].improved == 3) sc[g].done = 1;
}

// w = max(xmin - vm, 0) ; vm += w - xmin
__global__ void k_nn_outer(const float *xmin, float *wv, float *vm, size_t N) {
    FOR_CHUNK(N) {
        const size_t k = base + i;
        const float u = xmin[k];
        const float wn = fmaxf(u - vm[k], 0.f);
        wv[k] = wn;
        vm[k] = vm[k] + wn - u;
    }
}

__global__ void k_copy(const float *__restrict__ a, float *__restrict__ b, size_t n) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
        b[i] = a[i];
}

__global__ void k_fill(float *__restrict__ b, float v, size_t n) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
        b[i] = v;
}

__global__ void k_group_sums(const double *part, int nblk, int W, int coupled, double *out) {
    const int G = coupled ? 1 : W;
    FOR_GROUP_WARP(G) {
        const double v = group_sum(part, nblk, nullptr, 0, g, W, coupled);
        if ((threadIdx.x & 31) == 0) out[g] = v;
    }
}

// ---------------------------------------------------------------------------
// workspace
// ---------------------------------------------------------------------------
struct Work {
    int W = 0;
    size_t bytes = 0;
    float *s1 = nullptr, *s2 = nullptr, *s3 = nullptr;  // sinogram vectors
    float *i[12] = {};                                  // image vectors
    double *part = nullptr;                             // partial sums, 4 slots
    Scal *sc = nullptr;
    double *gsum = nullptr;
};

static int nblk_for(size_t N) {
    size_t b = (N + RED_THREADS * 8 - 1) / (RED_THREADS * 8);
    if (b < 1) b = 1;
    if (b > 256) b = 256;
    return (int)b;
}

static void free_work(Work &w) {
    cudaFree(w.s1);
    cudaFree(w.s2);
    cudaFree(w.s3);
    for (auto &p : w.i) cudaFree(p);
    cudaFree(w.part);
    cudaFree(w.sc);
    cudaFree(w.gsum);
    w = Work();
}

static int make_work(const Plan &pl, int W, Work &wk) {
    const size_t NS = (size_t)W * pl.D * pl.T, NI = (size_t)W * pl.P;
    wk.W = W;
#define AL(p, n, T)                                                                        \
    if (cudaMalloc((void **)&(p), (n) * sizeof(T)) != cudaSuccess) {                        \
        free_work(wk);                                                                     \
        set_error("solver workspace allocation failed");                                   \
        return MSOT_ENOMEM;                                                                \
    }
    AL(wk.s1, NS, float);
    AL(wk.s2, NS, float);
    AL(wk.s3, NS, float);
    for (auto &p : wk.i) AL(p, NI, float);
    AL(wk.part, (size_t)4 * W * 256, double);
    AL(wk.sc, (size_t)W, Scal);
    AL(wk.gsum, (size_t)W, double);
#undef AL
    return MSOT_OK;
}

struct Ctx {
    const Plan &pl;
    int W;
    int coupled;
    cudaStream_t st;
    size_t NS, NI;
    int nbs, nbi;
    Work &wk;
    double *P(int slot) const { return wk.part + (size_t)slot * W * 256; }
};

#define TRY(x)                                                                             \
    do {                                                                                   \
        int rc_ = (x);                                                                     \
        if (rc_ != MSOT_OK) return rc_;                                                    \
    } while (0)

static int group_sumsq(const Ctx &c, const float *x, const float *y, size_t N, int nb,
                       std::vector<double> &out) {
    KLAUNCH(k_sumsq<<<dim3(nb, c.W), RED_THREADS, 0, c.st>>>(x, y, N / c.W, c.P(3)));
    MSOT_LAUNCH_CHECK();
    KLAUNCH(k_group_sums<<<1, 1024, 0, c.st>>>(c.P(3), nb, c.W, c.coupled, c.wk.gsum));
    MSOT_LAUNCH_CHECK();
    const int G = c.coupled ? 1 : c.W;
    out.resize(G);
    MSOT_CUDA_TRY(cudaMemcpyAsync(out.data(), c.wk.gsum, sizeof(double) * G,
                                  cudaMemcpyDeviceToHost, c.st));
    MSOT_CUDA_TRY(cudaStreamSynchronize(c.st));
    return MSOT_OK;
}

// One outer iteration of nnls_L2_less: lsqr(maxit = 2, x0 = w), clip, multiplier.
static int l2_outer(const Ctx &c, const float *b, float *wv, float *vm, double sr,
                    int has_reg, const double *normb2, double sr2) {
    const double sl = 1.0, sb = std::sqrt(1e-3);
    Work &k = c.wk;
    float *us = k.s1, *tmp_s = k.s2;
    float *ur = k.i[0], *ub = k.i[1], *v = k.i[2], *d = k.i[3], *x = k.i[4], *xmin = k.i[5],
          *tmp_i = k.i[6];
    // second regulariser (Laplacian): residual block ul, del2 results in tl
    const bool lap = sr2 > 0.0;
    float *ul = lap ? k.i[9] : nullptr, *tl = lap ? k.i[10] : nullptr;
    const int nx = c.pl.nx, nz = c.pl.nz;
    const size_t ns = c.NS / c.W, ni = c.NI / c.W;
    const dim3 gs(c.nbs, c.W), gi(c.nbi, c.W);
    const int G = c.coupled ? 1 : c.W;
    cudaStream_t st = c.st;
    // The sinogram part of u is updated inside the forward operator's
    // convolution where the plan allows it (no A v round trip through HBM);
    // nps = partial sums per instance that the update leaves in P(0).
    const bool fuse = forward_update_fusable(c.pl, c.W);
    int nps = c.nbs;
    // init: u = b_aug - A_aug w
    if (fuse) {
        TRY(apply_forward_update(c.pl, wv, us, b, c.W, 0, (float)sl, k.sc, c.coupled, c.P(0),
                                 &nps, st));
    } else {
        TRY(apply_forward(c.pl, wv, tmp_s, c.W, st));
        KLAUNCH(k_sino_update<<<gs, RED_THREADS, 0, st>>>(tmp_s, b, us, ns, 0, sl, k.sc,
                                                          c.coupled, c.P(0)));
    }
    if (lap) KLAUNCH(k_del2<<<gi, RED_THREADS, 0, st>>>(wv, tl, nx, nz));
    KLAUNCH(k_l2_init_img<<<gi, RED_THREADS, 0, st>>>(wv, vm, ur, ub, ni, sl, sr, sb, has_reg, c.P(1),
                                              c.P(2), tl, ul, sr2));
    KLAUNCH(k_l2_scalar<<<1, 1024, 0, st>>>(k.sc, 0, c.P(0), nps, c.P(1), c.nbi, c.P(2), c.nbi, normb2,
                                   sl, sb, c.W, c.coupled, 1e-8));
    MSOT_LAUNCH_CHECK();
    // v = A_aug^T u / beta
    TRY(apply_transpose(c.pl, us, tmp_i, c.W, st));
    if (lap) KLAUNCH(k_del2<<<gi, RED_THREADS, 0, st>>>(ul, tl, nx, nz));
    KLAUNCH(k_l2_v_img<<<gi, RED_THREADS, 0, st>>>(tmp_i, ur, ub, v, ni, sl, sr, sb, has_reg, 1, k.sc,
                                           c.coupled, c.P(1), tl, sr2));
    KLAUNCH(k_l2_scalar<<<1, 1024, 0, st>>>(k.sc, 1, c.P(1), c.nbi, nullptr, 0, nullptr, 0, nullptr, sl,
                                   sb, c.W, c.coupled, 1e-8));
    KLAUNCH(k_l2_scale_v<<<gi, RED_THREADS, 0, st>>>(v, d, x, xmin, wv, ni, 1, k.sc, c.coupled));
    MSOT_LAUNCH_CHECK();
    for (int it = 0; it < 2; ++it) {
        KLAUNCH(k_l2_gamma<<<1, 256, 0, st>>>(k.sc, G));
        if (fuse) {
            TRY(apply_forward_update(c.pl, v, us, nullptr, c.W, 1, (float)sl, k.sc, c.coupled,
                                     c.P(0), &nps, st));
        } else {
            TRY(apply_forward(c.pl, v, tmp_s, c.W, st));
            KLAUNCH(k_sino_update<<<gs, RED_THREADS, 0, st>>>(tmp_s, nullptr, us, ns, 1, sl, k.sc,
                                                              c.coupled, c.P(0)));
        }
        if (lap) KLAUNCH(k_del2<<<gi, RED_THREADS, 0, st>>>(v, tl, nx, nz));
        KLAUNCH(k_l2_u_img<<<gi, RED_THREADS, 0, st>>>(v, ur, ub, ni, sl, sr, sb, has_reg, k.sc,
                                               c.coupled, c.P(1), tl, ul, sr2));
        KLAUNCH(k_l2_scalar<<<1, 1024, 0, st>>>(k.sc, 2, c.P(0), nps, c.P(1), c.nbi, nullptr, 0,
                                       nullptr, sl, sb, c.W, c.coupled, 1e-8));
        KLAUNCH(k_l2_dx<<<gi, RED_THREADS, 0, st>>>(v, d, x, xmin, ni, k.sc, c.coupled));
        KLAUNCH(k_l2_mark_converged<<<1, 256, 0, st>>>(k.sc, G));
        MSOT_LAUNCH_CHECK();
        if (it == 1) break;  // the last A^T of lsqr only feeds its stopping test
        TRY(apply_transpose(c.pl, us, tmp_i, c.W, st));
        if (lap) KLAUNCH(k_del2<<<gi, RED_THREADS, 0, st>>>(ul, tl, nx, nz));
        KLAUNCH(k_l2_v_img<<<gi, RED_THREADS, 0, st>>>(tmp_i, ur, ub, v, ni, sl, sr, sb, has_reg, 0,
                                               k.sc, c.coupled, c.P(1), tl, sr2));
        KLAUNCH(k_l2_scalar<<<1, 1024, 0, st>>>(k.sc, 1, c.P(1), c.nbi, nullptr, 0, nullptr, 0, nullptr,
                                       sl, sb, c.W, c.coupled, 1e-8));
        KLAUNCH(k_l2_scale_v<<<gi, RED_THREADS, 0, st>>>(v, d, x, xmin, wv, ni, 0, k.sc, c.coupled));
        MSOT_LAUNCH_CHECK();
    }
    KLAUNCH(k_nn_outer<<<gi, RED_THREADS, 0, st>>>(xmin, wv, vm, ni));
    MSOT_LAUNCH_CHECK();
    return MSOT_OK;
}

// Per-plan solver state: the workspace (grown to the largest batch seen) and
// one captured CUDA graph of an outer L2 iteration for the last
// (batch, regulariser, coupling) combination; the graph reads the right-hand
// side from the workspace, so each call copies b there first.
struct SolverCache {
    Work wk;
    cudaStream_t stream = nullptr;  // non-blocking stream the graphs are captured on
    cudaEvent_t ev_in = nullptr, ev_out = nullptr;
    cudaGraphExec_t l2_exec = nullptr;
    int l2_W = -1, l2_has_reg = -1, l2_coupled = -1;
    double l2_sr = -1.0, l2_sr2 = -1.0;
    long l2_kernels = 0;  // kernel nodes in the captured iteration
};

static SolverCache *cache_for(Plan &pl, int W, int &rc) {
    rc = MSOT_OK;
    if (!pl.solver) pl.solver = new SolverCache();
    SolverCache *sc = pl.solver;
    if (!sc->stream) {
        if (cudaStreamCreateWithFlags(&sc->stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&sc->ev_in, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&sc->ev_out, cudaEventDisableTiming) != cudaSuccess) {
            set_error("solver: stream creation failed");
            rc = MSOT_ECUDA;
            return sc;
        }
    }
    if (sc->wk.W < W) {
        if (sc->l2_exec) cudaGraphExecDestroy(sc->l2_exec);
        sc->l2_exec = nullptr;
        sc->l2_W = -1;
        free_work(sc->wk);
        rc = make_work(pl, W, sc->wk);
    }
    return sc;
}

void solver_cache_invalidate(Plan &pl) {
    if (!pl.solver) return;
    if (pl.solver->l2_exec) cudaGraphExecDestroy(pl.solver->l2_exec);
    pl.solver->l2_exec = nullptr;
    pl.solver->l2_W = -1;
}

void solver_cache_free(Plan &pl) {
    if (!pl.solver) return;
    if (pl.solver->l2_exec) cudaGraphExecDestroy(pl.solver->l2_exec);
    if (pl.solver->stream) cudaStreamDestroy(pl.solver->stream);
    if (pl.solver->ev_in) cudaEventDestroy(pl.solver->ev_in);
    if (pl.solver->ev_out) cudaEventDestroy(pl.solver->ev_out);
    free_work(pl.solver->wk);
    delete pl.solver;
    pl.solver = nullptr;
}

static long count_kernel_nodes(cudaGraph_t g) {
    size_t n = 0;
    if (cudaGraphGetNodes(g, nullptr, &n) != cudaSuccess || n == 0) return 0;
    std::vector<cudaGraphNode_t> nodes(n);
    if (cudaGraphGetNodes(g, nodes.data(), &n) != cudaSuccess) return 0;
    long k = 0;
    for (auto nd : nodes) {
        cudaGraphNodeType t;
        if (cudaGraphNodeGetType(nd, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++k;
    }
    return k;
}

static int solve_l2(Plan &pl, const float *b_in, float *rec, int W, int num_iter,
                    double lambdaL2, const float *x0, const float *v0, int coupled,
                    double *err_img, double *err_reg, cudaStream_t user,
                    double lambdaL2_2 = 0.0, double *err_reg2 = nullptr,
                    float *v_out = nullptr) {
    int rc;
    SolverCache *sc = cache_for(pl, W, rc);
    if (rc) return rc;
    // run on the plan's own stream (capturable), ordered after the caller's work
    cudaStream_t st = sc->stream;
    MSOT_CUDA_TRY(cudaEventRecord(sc->ev_in, user));
    MSOT_CUDA_TRY(cudaStreamWaitEvent(st, sc->ev_in, 0));
    Work &wk = sc->wk;
    const size_t NS = (size_t)W * pl.D * pl.T, NI = (size_t)W * pl.P;
    Ctx c{pl, W, coupled, st, NS, NI, nblk_for(NS / W), nblk_for(NI / W), wk};
    const int has_reg = lambdaL2 > 0;
    const double sr = has_reg ? std::sqrt(lambdaL2) : 0.0;
    // incorporate_l2_reg_into_model_functions.m:8-18: the second term only
    // together with the first
    const double sr2 = has_reg && lambdaL2_2 > 0 ? std::sqrt(lambdaL2_2) : 0.0;
    float *wv = wk.i[7], *vm = wk.i[8];
    const float *b = wk.s3;
    int nonfinite = -1;  // first instance whose final residual is NaN / Inf
    do {
        MSOT_CUDA_TRY(cudaMemcpyAsync(wk.s3, b_in, NS * sizeof(float), cudaMemcpyDeviceToDevice, st));
        if (x0)
            KLAUNCH(k_copy<<<256, 256, 0, st>>>(x0, wv, NI));
        else
            KLAUNCH(k_fill<<<256, 256, 0, st>>>(wv, 0.f, NI));
        if (v0)
            KLAUNCH(k_copy<<<256, 256, 0, st>>>(v0, vm, NI));
        else
            KLAUNCH(k_fill<<<256, 256, 0, st>>>(vm, 0.f, NI));
        // ||b||^2 per group enters ||b_aug|| of lsqr's tolerance test
        KLAUNCH(k_sumsq<<<dim3(c.nbs, W), RED_THREADS, 0, st>>>(b, nullptr, NS / W, c.P(3)));
        KLAUNCH(k_group_sums<<<1, 1024, 0, st>>>(c.P(3), c.nbs, W, coupled, wk.gsum));
        if (cudaGetLastError() != cudaSuccess) {
            set_error("solver: launch failed");
            rc = MSOT_ECUDA;
            break;
        }
        int it = 0;
        const bool use_graph = !profiling_enabled() && num_iter > 1;
        const bool have = sc->l2_exec && sc->l2_W == W && sc->l2_has_reg == has_reg &&
                          sc->l2_coupled == coupled && sc->l2_sr == sr && sc->l2_sr2 == sr2;
        if (use_graph && !have) {
            // first iteration eagerly (sets kernel attributes), then capture one
            if ((rc = l2_outer(c, b, wv, vm, sr, has_reg, wk.gsum, sr2))) break;
            ++it;
            if (sc->l2_exec) cudaGraphExecDestroy(sc->l2_exec);
            sc->l2_exec = nullptr;
            cudaGraph_t g = nullptr;
            MSOT_CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed));
            const long before = g_launch_count.load();
            rc = l2_outer(c, b, wv, vm, sr, has_reg, wk.gsum, sr2);
            g_launch_count -= g_launch_count.load() - before;  // counted per replay below
            cudaError_t ce = cudaStreamEndCapture(st, &g);
            if (rc || ce != cudaSuccess) {
                if (g) cudaGraphDestroy(g);
                if (!rc) {
                    set_error("solver: graph capture failed: %s", cudaGetErrorString(ce));
                    rc = MSOT_ECUDA;
                }
                break;
            }
            ce = cudaGraphInstantiate(&sc->l2_exec, g, 0);
            sc->l2_kernels = count_kernel_nodes(g);
            cudaGraphDestroy(g);
            if (ce != cudaSuccess) {
                set_error("solver: graph instantiation failed: %s", cudaGetErrorString(ce));
                sc->l2_exec = nullptr;
                rc = MSOT_ECUDA;
                break;
            }
            sc->l2_W = W;
            sc->l2_has_reg = has_reg;
            sc->l2_coupled = coupled;
            sc->l2_sr = sr;
            sc->l2_sr2 = sr2;
        }
        if (use_graph) {
            for (; it < num_iter; ++it) {
                MSOT_CUDA_TRY(cudaGraphLaunch(sc->l2_exec, st));
                g_launch_count += sc->l2_kernels;
            }
        } else {
            for (; it < num_iter && rc == MSOT_OK; ++it)
                rc = l2_outer(c, b, wv, vm, sr, has_reg, wk.gsum, sr2);
            if (rc) break;
        }
        KLAUNCH(k_copy<<<256, 256, 0, st>>>(wv, rec, NI));
        if (v_out) KLAUNCH(k_copy<<<256, 256, 0, st>>>(vm, v_out, NI));
        if (err_img || err_reg) {
            std::vector<double> e;
            if ((rc = apply_forward(pl, rec, wk.s2, W, st))) break;
            if (err_img) {
                Ctx ci = c;
                ci.coupled = 0;
                if ((rc = group_sumsq(ci, wk.s2, b, NS, c.nbs, e))) break;
                for (int w = 0; w < W; ++w) {
                    err_img[w] = e[w];
                    if (nonfinite < 0 && !std::isfinite(e[w])) nonfinite = w;
                }
            }
            if (err_reg) {
                Ctx ci = c;
                ci.coupled = 0;
                if ((rc = group_sumsq(ci, rec, nullptr, NI, c.nbi, e))) break;
                for (int w = 0; w < W; ++w) err_reg[w] = has_reg ? e[w] : 0.0;
            }
        }
        if (err_reg2) {
            // lCurveErrReg_2 = ||del2(rec)||^2 (rec_nn_with_L2_reg.m:58-63)
            std::vector<double> e;
            if (sr2 > 0.0) {
                KLAUNCH(k_del2<<<dim3(c.nbi, W), RED_THREADS, 0, st>>>(rec, wk.i[10], pl.nx, pl.nz));
                Ctx ci = c;
                ci.coupled = 0;
                if ((rc = group_sumsq(ci, wk.i[10], nullptr, NI, c.nbi, e))) break;
            }
            for (int w = 0; w < W; ++w) err_reg2[w] = sr2 > 0.0 ? e[w] : 0.0;
        }
        cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            set_error("solver: %s", cudaGetErrorString(e));
            rc = MSOT_ECUDA;
        }
    } while (0);
    if (rc == MSOT_OK && nonfinite >= 0) {
        // the reference returns the NaN image silently; here the caller learns
        // of it (the image is still written)
        set_error("rec_nn_with_L2_reg: non-finite residual ||A x - b||^2 for instance %d "
                  "(NaN or Inf in the data or the start)", nonfinite);
        rc = MSOT_ENONFINITE;
    }
    cudaEventRecord(sc->ev_out, st);
    cudaStreamWaitEvent(user, sc->ev_out, 0);
    return rc;
}

// ---------------------------------------------------------------------------
// L1 (identity) NNLS: split Bregman with cgs(lam A^T A + I, rhs, 1e-8, 2)
// ---------------------------------------------------------------------------
__global__ void k_dot(const float *__restrict__ a, const float *__restrict__ b, size_t N,
                      double *part) {
    float acc = 0.f;
    FOR_CHUNK(N) acc = fmaf(a[base + i], b[base + i], acc);
    STORE_PARTIAL((double)acc, part);
}

// d = max(u - bp, 0); rhs = d + bp + lam*atb - lam*eta; cgs init: x = 0, r = rt = rhs.
__global__ void k_l1_rhs(const float *u, const float *bp, const float *atb, float *dv,
                         float *rhs, float *x, float *r, float *rt, float *xmin, size_t N,
                         double lam, double eta, double *part) {
    float acc = 0.f;
    const float lf = (float)lam, le = (float)(lam * eta);
    FOR_CHUNK(N) {
        const size_t k = base + i;
        const float dd = fmaxf(u[k] - bp[k], 0.f);
        dv[k] = dd;
        const float rh = fmaf(lf, atb[k], fmaxf(dd, 0.f) + bp[k]) - le;
        rhs[k] = rh;
        r[k] = rh;
        rt[k] = rh;
        x[k] = 0.f;
        xmin[k] = 0.f;
        acc = fmaf(rh, rh, acc);
    }
    STORE_PARTIAL((double)acc, part);
}

// stage 0: n2b; 1: rho = rt.r; 2: alpha = rho / rt.vh; 3: normr after r update
__global__ void k_cgs_scalar(Scal *sc, int stage, const double *p, int nb, int W, int coupled,
                             double tol) {
    const int G = coupled ? 1 : W;
    FOR_GROUP_WARP(G) {
        Scal &q = sc[g];
        const double v = group_sum(p, nb, nullptr, 0, g, W, coupled);
        LANE0_ONLY;
        if (stage == 0) {
            q.normb = sqrt(v);
            q.normr = q.normb;
            q.normrmin = q.normb;
            q.rho_cg = 1.0;
            q.done = !(q.normb > 0.0) || !isfinite(q.normb);
            q.improved = 0;
            continue;
        }
        if (q.done) {
            q.improved = 0;
            continue;
        }
        if (stage == 1) {
            q.rho1_cg = q.rho_cg;
            q.rho_cg = v;
            if (v == 0.0 || !isfinite(v)) q.done = 1;
        } else if (stage == 2) {
            if (v == 0.0 || !isfinite(v)) {
                q.done = 1;
            } else {
                q.alpha_cg = q.rho_cg / v;
            }
        } else {
            q.normr = sqrt(v);
            q.improved = 0;
            if (q.normr <= tol * q.normb) {
                q.improved = 3;
            } else if (q.normr < q.normrmin) {
                q.normrmin = q.normr;
                q.improved = 1;
            }
        }
    }
}

// direction: first: uc = r, p = uc; else beta = rho/rho1: uc = r + beta q,
// p = uc + beta (q + beta p)
__global__ void k_cgs_dir(const float *r, float *q, float *uc, float *p, size_t N, int first,
                          const Scal *sc, int coupled) {
    FOR_CHUNK(N) {
        const size_t k = base + i;
        const Scal &s = sc[grp(w, coupled)];
        if (s.done) continue;
        if (first) {
            uc[k] = r[k];
            p[k] = r[k];
        } else {
            const float beta = (float)(s.rho_cg / s.rho1_cg);
            const float u = fmaf(beta, q[k], r[k]);
            uc[k] = u;
            p[k] = fmaf(beta, fmaf(beta, p[k], q[k]), u);
        }
    }
}

// y = lam*atav + v ; partial dot(rt, y)
__global__ void k_cgs_op(const float *atav, const float *v, float *y, const float *rt,
                         size_t N, double lam, double *part) {
    float acc = 0.f;
    const float lf = (float)lam;
    FOR_CHUNK(N) {
        const size_t k = base + i;
        const float o = fmaf(lf, atav[k], v[k]);
        y[k] = o;
        acc = fmaf(rt[k], o, acc);
    }
    STORE_PARTIAL((double)acc, part);
}

// q = uc - alpha vh; uh = uc + q; x += alpha uh
__global__ void k_cgs_upd(const float *uc, const float *vh, float *q, float *uh, float *x,
                          size_t N, const Scal *sc, int coupled) {
    FOR_CHUNK(N) {
        const size_t k = base + i;
        const Scal &s = sc[grp(w, coupled)];
        if (s.done) continue;
        const float a = (float)s.alpha_cg;
        const float qq = fmaf(-a, vh[k], uc[k]);
        q[k] = qq;
        const float u = uc[k] + qq;
        uh[k] = u;
        x[k] = fmaf(a, u, x[k]);
    }
}

// r -= alpha (lam atau + uh); partial ||r||^2
__global__ void k_cgs_res(const float *atau, const float *uh, float *r, size_t N, double lam,
                          const Scal *sc, int coupled, double *part) {
    float acc = 0.f;
    const Scal &s = sc[grp(blockIdx.y, coupled)];
    const float lf = (float)lam, a = (float)s.alpha_cg;
    const bool done = s.done;
    FOR_CHUNK(N) {
        const size_t k = base + i;
        float rr = r[k];
        if (!done) {
            rr = fmaf(-a, fmaf(lf, atau[k], uh[k]), rr);
            r[k] = rr;
        }
        acc = fmaf(rr, rr, acc);
    }
    STORE_PARTIAL((double)acc, part);
}

__global__ void k_cgs_keep(const float *x, float *xmin, size_t N, const Scal *sc, int coupled) {
    FOR_CHUNK(N) {
        const size_t k = base + i;
        const Scal &s = sc[grp(w, coupled)];
        if (s.improved) xmin[k] = x[k];
    }
}

__global__ void k_cgs_mark(Scal *sc, int G) {
    for (int g = threadIdx.x; g < G; g += blockDim.x)
        if (sc[g].improved == 3) sc[g].done = 1;
}

// bp += d - u
__global__ void k_l1_bregman(const float *dv, const float *u, float *bp, size_t N) {
    FOR_CHUNK(N) {
        const size_t k = base + i;
        bp[k] = bp[k] + fmaxf(dv[k], 0.f) - u[k];
    }
}

static int normal_op(const Ctx &c, const float *v, float *out_atav) {
    TRY(apply_forward(c.pl, v, c.wk.s2, c.W, c.st));
    return apply_transpose(c.pl, c.wk.s2, out_atav, c.W, c.st);
}

static int solve_l1(const Plan &pl, const float *b, float *rec, int W, int num_iter, double eta,
                    const float *x0, int coupled, double *err_img, double *err_reg,
                    cudaStream_t st) {
    Work wk;
    TRY(make_work(pl, W, wk));
    const size_t NS = (size_t)W * pl.D * pl.T, NI = (size_t)W * pl.P;
    Ctx c{pl, W, coupled, st, NS, NI, nblk_for(NS / W), nblk_for(NI / W), wk};
    const size_t ni = NI / W;
    const dim3 gi(c.nbi, W);
    const int G = coupled ? 1 : W;
    const double lam = 1.0;
    float *u = wk.i[0], *bp = wk.i[1], *atb = wk.i[2], *dv = wk.i[3], *rhs = wk.i[4],
          *x = wk.i[5], *r = wk.i[6], *rt = wk.i[7], *xmin = wk.i[8], *q = wk.i[9],
          *uc = wk.i[10], *p = wk.i[11];
    // vh shares storage with rhs (rhs is only needed for the cgs init)
    float *vh = rhs;
    int rc = MSOT_OK;
    float *atmp = nullptr, *uh = nullptr;
    int nonfinite = -1;  // first instance whose final residual is NaN / Inf
    do {
        if (cudaMalloc(&atmp, NI * sizeof(float)) != cudaSuccess ||
            cudaMalloc(&uh, NI * sizeof(float)) != cudaSuccess) {
            set_error("L1 workspace allocation failed");
            rc = MSOT_ENOMEM;
            break;
        }
        // start value A^T b (rec_nn_with_L1_eye_reg.m:33) unless a warm start is given
        if ((rc = apply_transpose(pl, b, atb, W, st))) break;
        if (x0)
            KLAUNCH(k_copy<<<256, 256, 0, st>>>(x0, u, NI));
        else
            KLAUNCH(k_copy<<<256, 256, 0, st>>>(atb, u, NI));
        KLAUNCH(k_fill<<<256, 256, 0, st>>>(bp, 0.f, NI));
        for (int it = 0; it < num_iter && rc == MSOT_OK; ++it) {
            // reduced storage: every refine_every-th outer iteration runs its
            // operators with the FP32 interpolation input, which corrects the
            // drift the reduced-storage iterations leave in u and the Bregman
            // variable
            pl.image_fmt = (pl.refine_every > 0 && (it + 1) % pl.refine_every == 0)
                               ? 0
                               : pl.storage_fmt;
            KLAUNCH(k_l1_rhs<<<gi, RED_THREADS, 0, st>>>(u, bp, atb, dv, rhs, x, r, rt, xmin, ni, lam, eta,
                                                 c.P(0)));
            KLAUNCH(k_cgs_scalar<<<1, 1024, 0, st>>>(wk.sc, 0, c.P(0), c.nbi, W, coupled, 1e-8));
            for (int ci = 0; ci < 2 && rc == MSOT_OK; ++ci) {
                KLAUNCH(k_dot<<<gi, RED_THREADS, 0, st>>>(rt, r, ni, c.P(0)));
                KLAUNCH(k_cgs_scalar<<<1, 1024, 0, st>>>(wk.sc, 1, c.P(0), c.nbi, W, coupled, 1e-8));
                KLAUNCH(k_cgs_dir<<<gi, RED_THREADS, 0, st>>>(r, q, uc, p, ni, ci == 0, wk.sc, coupled));
                if ((rc = normal_op(c, p, atmp))) break;
                KLAUNCH(k_cgs_op<<<gi, RED_THREADS, 0, st>>>(atmp, p, vh, rt, ni, lam, c.P(0)));
                KLAUNCH(k_cgs_scalar<<<1, 1024, 0, st>>>(wk.sc, 2, c.P(0), c.nbi, W, coupled, 1e-8));
                KLAUNCH(k_cgs_upd<<<gi, RED_THREADS, 0, st>>>(uc, vh, q, uh, x, ni, wk.sc, coupled));
                if ((rc = normal_op(c, uh, atmp))) break;
                KLAUNCH(k_cgs_res<<<gi, RED_THREADS, 0, st>>>(atmp, uh, r, ni, lam, wk.sc, coupled,
                                                      c.P(0)));
                KLAUNCH(k_cgs_scalar<<<1, 1024, 0, st>>>(wk.sc, 3, c.P(0), c.nbi, W, coupled, 1e-8));
                KLAUNCH(k_cgs_keep<<<gi, RED_THREADS, 0, st>>>(x, xmin, ni, wk.sc, coupled));
                KLAUNCH(k_cgs_mark<<<1, 256, 0, st>>>(wk.sc, G));
            }
            if (rc) break;
            KLAUNCH(k_copy<<<256, 256, 0, st>>>(xmin, u, NI));
            KLAUNCH(k_l1_bregman<<<gi, RED_THREADS, 0, st>>>(dv, u, bp, ni));
            if (cudaGetLastError() != cudaSuccess) {
                set_error("L1 solver: launch failed");
                rc = MSOT_ECUDA;
            }
        }
        pl.image_fmt = 0;  // lCurveErrImg with the FP32 operator
        if (rc) break;
        KLAUNCH(k_copy<<<256, 256, 0, st>>>(u, rec, NI));
        if (err_img || err_reg) {
            std::vector<double> e;
            Ctx ci = c;
            ci.coupled = 0;
            if (err_img) {
                if ((rc = apply_forward(pl, rec, wk.s2, W, st))) break;
                if ((rc = group_sumsq(ci, wk.s2, b, NS, c.nbs, e))) break;
                for (int w = 0; w < W; ++w) {
                    err_img[w] = e[w];
                    if (nonfinite < 0 && !std::isfinite(e[w])) nonfinite = w;
                }
            }
            if (err_reg) {
                std::vector<float> h(NI);
                MSOT_CUDA_TRY(cudaMemcpyAsync(h.data(), rec, NI * sizeof(float),
                                              cudaMemcpyDeviceToHost, st));
                MSOT_CUDA_TRY(cudaStreamSynchronize(st));
                for (int w = 0; w < W; ++w) {
                    double s1 = 0;
                    for (size_t k = 0; k < ni; ++k) s1 += std::fabs((double)h[w * ni + k]);
                    err_reg[w] = s1;
                }
            }
        }
        cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            set_error("L1 solver: %s", cudaGetErrorString(e));
            rc = MSOT_ECUDA;
        }
    } while (0);
    pl.image_fmt = pl.storage_fmt;
    if (rc == MSOT_OK && nonfinite >= 0) {
        set_error("rec_nn_with_L1_eye_reg: non-finite residual ||A x - b||^2 for instance %d "
                  "(NaN or Inf in the data or the start)", nonfinite);
        rc = MSOT_ENONFINITE;
    }
    cudaFree(atmp);
    cudaFree(uh);
    free_work(wk);
    return rc;
}

// ---------------------------------------------------------------------------
// sigma_max by power iteration on A^T A (FP64 norms)
// ---------------------------------------------------------------------------
__global__ void k_seed(float *v, size_t n, uint64_t seed) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        uint64_t z = seed + 0x9E3779B97F4A7C15ull * (i + 1);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        v[i] = (float)((double)(z >> 11) * (1.0 / 9007199254740992.0) - 0.5);
    }
}

__global__ void k_scale_by(float *v, size_t n, const double *ss) {
    const double f = 1.0 / sqrt(ss[0]);
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
        v[i] = (float)((double)v[i] * f);
}

static int estimate_norm(const Plan &pl, int iters, uint64_t seed, double *out, cudaStream_t st) {
    Work wk;
    TRY(make_work(pl, 1, wk));
    const size_t NI = pl.P, NS = (size_t)pl.D * pl.T;
    Ctx c{pl, 1, 0, st, NS, NI, nblk_for(NS), nblk_for(NI), wk};
    int rc = MSOT_OK;
    float *v = wk.i[0], *z = wk.i[1];
    do {
        KLAUNCH(k_seed<<<64, 256, 0, st>>>(v, NI, seed));
        KLAUNCH(k_sumsq<<<dim3(c.nbi, 1), RED_THREADS, 0, st>>>(v, nullptr, NI, c.P(0)));
        KLAUNCH(k_group_sums<<<1, 32, 0, st>>>(c.P(0), c.nbi, 1, 0, wk.gsum));
        KLAUNCH(k_scale_by<<<64, 256, 0, st>>>(v, NI, wk.gsum));
        for (int it = 0; it < iters && rc == MSOT_OK; ++it) {
            if ((rc = apply_forward(pl, v, wk.s1, 1, st))) break;
            if ((rc = apply_transpose(pl, wk.s1, z, 1, st))) break;
            KLAUNCH(k_sumsq<<<dim3(c.nbi, 1), RED_THREADS, 0, st>>>(z, nullptr, NI, c.P(0)));
            KLAUNCH(k_group_sums<<<1, 32, 0, st>>>(c.P(0), c.nbi, 1, 0, wk.gsum));
            KLAUNCH(k_scale_by<<<64, 256, 0, st>>>(z, NI, wk.gsum));
            std::swap(v, z);
        }
        if (rc) break;
        if ((rc = apply_forward(pl, v, wk.s1, 1, st))) break;
        std::vector<double> e;
        if ((rc = group_sumsq(c, wk.s1, nullptr, NS, c.nbs, e))) break;
        *out = std::sqrt(e[0]) * pl.norm;
    } while (0);
    free_work(wk);
    return rc;
}

}  // namespace msot

using namespace msot;

extern "C" int msot_rec_nn_with_L2_reg(msot_plan_t plan, const float *d_b, float *d_rec,
                                       int batch, int num_iter, double lambdaL2,
                                       const float *d_x0, int coupled, double *err_img,
                                       double *err_reg, void *stream) {
    if (!plan || !d_b || !d_rec || batch <= 0 || num_iter < 0) {
        set_error("rec_nn_with_L2_reg: bad arguments");
        return MSOT_EINVAL;
    }
    if (batch > plan->p.max_batch) {
        set_error("batch %d exceeds the plan's max_batch %d", batch, plan->p.max_batch);
        return MSOT_EINVAL;
    }
    if (int rc = check_plan_device(plan->p, "solver")) return rc;
    return solve_l2(plan->p, d_b, d_rec, batch, num_iter, lambdaL2, d_x0, nullptr,
                    coupled ? 1 : 0, err_img, err_reg, (cudaStream_t)stream);
}

extern "C" int msot_rec_nn_with_L2_reg_warm(msot_plan_t plan, const float *d_b, float *d_rec,
                                            int batch, int num_iter, double lambdaL2,
                                            const float *d_w0, const float *d_v0, int coupled,
                                            double *err_img, double *err_reg, void *stream) {
    if (!plan || !d_b || !d_rec || batch <= 0 || num_iter < 0 || !d_w0 || !d_v0) {
        set_error("rec_nn_with_L2_reg_warm: bad arguments");
        return MSOT_EINVAL;
    }
    if (batch > plan->p.max_batch) {
        set_error("batch %d exceeds the plan's max_batch %d", batch, plan->p.max_batch);
        return MSOT_EINVAL;
    }
    if (int rc = check_plan_device(plan->p, "solver")) return rc;
    return solve_l2(plan->p, d_b, d_rec, batch, num_iter, lambdaL2, d_w0, d_v0,
                    coupled ? 1 : 0, err_img, err_reg, (cudaStream_t)stream);
}

extern "C" int msot_rec_nn_with_L2_reg_state(msot_plan_t plan, const float *d_b, float *d_rec,
                                             float *d_v, int batch, int num_iter,
                                             double lambdaL2, const float *d_w0,
                                             const float *d_v0, int coupled, double *err_img,
                                             double *err_reg, void *stream) {
    if (!plan || !d_b || !d_rec || !d_v || batch <= 0 || num_iter < 0 || (!d_w0 && d_v0)) {
        set_error("rec_nn_with_L2_reg_state: bad arguments (a v0 needs its w0)");
        return MSOT_EINVAL;
    }
    if (batch > plan->p.max_batch) {
        set_error("batch %d exceeds the plan's max_batch %d", batch, plan->p.max_batch);
        return MSOT_EINVAL;
    }
    if (int rc = check_plan_device(plan->p, "solver")) return rc;
    return solve_l2(plan->p, d_b, d_rec, batch, num_iter, lambdaL2, d_w0, d_v0,
                    coupled ? 1 : 0, err_img, err_reg, (cudaStream_t)stream, 0.0, nullptr, d_v);
}

extern "C" int msot_rec_nn_with_L2_reg_2(msot_plan_t plan, const float *d_b, float *d_rec,
                                         int batch, int num_iter, double lambdaL2,
                                         double lambdaL2_2, const float *d_x0, int coupled,
                                         double *err_img, double *err_reg, double *err_reg2,
                                         void *stream) {
    if (!plan || !d_b || !d_rec || batch <= 0 || num_iter < 0) {
        set_error("rec_nn_with_L2_reg_2: bad arguments");
        return MSOT_EINVAL;
    }
    if (batch > plan->p.max_batch) {
        set_error("batch %d exceeds the plan's max_batch %d", batch, plan->p.max_batch);
        return MSOT_EINVAL;
    }
    if (int rc = check_plan_device(plan->p, "solver")) return rc;
    return solve_l2(plan->p, d_b, d_rec, batch, num_iter, lambdaL2, d_x0, nullptr,
                    coupled ? 1 : 0, err_img, err_reg, (cudaStream_t)stream, lambdaL2_2,
                    err_reg2);
}

extern "C" int msot_laplacian_per_wavelength(const float *d_in, float *d_out, int batch, int nx,
                                             int nz, void *stream) {
    if (!d_in || !d_out || d_in == d_out || batch <= 0 || nx <= 0 || nz <= 0) {
        set_error("laplacian_per_wavelength: bad arguments (in and out must differ)");
        return MSOT_EINVAL;
    }
    const size_t N = (size_t)nx * nz;
    KLAUNCH(k_del2<<<dim3(nblk_for(N), batch), RED_THREADS, 0, (cudaStream_t)stream>>>(
        d_in, d_out, nx, nz));
    MSOT_LAUNCH_CHECK();
    return MSOT_OK;
}

extern "C" int msot_rec_nn_with_L1_eye_reg(msot_plan_t plan, const float *d_b, float *d_rec,
                                           int batch, int num_iter, double reg,
                                           const float *d_x0, int coupled, double *err_img,
                                           double *err_reg, void *stream) {
    if (!plan || !d_b || !d_rec || batch <= 0 || num_iter < 0) {
        set_error("rec_nn_with_L1_eye_reg: bad arguments");
        return MSOT_EINVAL;
    }
    if (batch > plan->p.max_batch) {
        set_error("batch %d exceeds the plan's max_batch %d", batch, plan->p.max_batch);
        return MSOT_EINVAL;
    }
    if (int rc = check_plan_device(plan->p, "solver")) return rc;
    return solve_l1(plan->p, d_b, d_rec, batch, num_iter, reg, d_x0, coupled ? 1 : 0, err_img,
                    err_reg, (cudaStream_t)stream);
}

extern "C" int msot_estimate_norm(msot_plan_t plan, int iters, uint64_t seed, double *sigma_max,
                                  void *stream) {
    if (!plan || !sigma_max || iters < 1) {
        set_error("estimate_norm: bad arguments");
        return MSOT_EINVAL;
    }
    if (int rc = check_plan_device(plan->p, "estimate_norm")) return rc;
    return estimate_norm(plan->p, iters, seed, sigma_max, (cudaStream_t)stream);
}
