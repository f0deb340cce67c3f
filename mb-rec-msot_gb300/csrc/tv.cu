// tv.cu -- isotropic-TV proximal operator and the TV-regularised
// non-negative solver on the GPU.
//
//   k_tv_prox  <- libraries/SplitBregmanTVdenoising/SB_ITV2.m:20-40 with
//                 DiffOper.m:1-7: split Bregman with lambda = 1, inner
//                 cgs(I + B'B, g - B'(b - d), 1e-5, 100) from zero, outer loop
//                 until ||u_prev - u|| / ||u|| <= 1e-3 (capped at TV_SB_MAX
//                 sweeps).  One CTA per image runs the whole prox on the
//                 device (bounded loops, no host round trips), vectors in
//                 global memory.
//   k_tv_prox_cl / k_tv_prox_cl4  the same prox by one thread-block cluster
//                 per image, the image split into column slabs held in
//                 shared memory (neighbours over distributed shared memory);
//                 cl4 handles 4 z-pixels per thread, and its GM form keeps
//                 the vectors in an L2-resident workspace for images too large
//                 for shared memory.  k_tv_prox is the fallback.
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
// msot_autotune (k_tune_fill fills its timing inputs) is also here: it times
// the kernel variants of a plan on its own geometry.
//
// All SpaRSA scalars (objective, alpha, mu = tau/alpha, stop flags) live on
// the device, so an outer iteration is a fixed launch sequence with no host
// synchronisation.  coupled = 1 makes the batch one SpaRSA problem (the
// reference's multi-wavelength call: one alpha and one objective over all
// wavelengths); coupled = 0 runs W independent reconstructions.
#include <cooperative_groups.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
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

// sum over the block (float within warps, double across warps); every
// thread gets the result
__device__ double tv_block_sum(float v, double *sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();  // sh may still be read from the previous call
    if (lane == 0) sh[wid] = (double)v;
    __syncthreads();
    if (wid == 0) {
        double d = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) d += __shfl_down_sync(0xffffffffu, d, o);
        if (lane == 0) sh[32] = d;
    }
    __syncthreads();
    return sh[32];
}

__device__ double tv_dot(const float *a, const float *b, int P, double *sh) {
    float acc = 0.f;
    for (int i = threadIdx.x; i < P; i += blockDim.x) acc = fmaf(a[i], b[i], acc);
    return tv_block_sum(acc, sh);
}

// broadcast flags of the thread-0 scalar logic (FP64 on GB300 is far too
// slow to replicate divisions and square roots across all threads)
enum : int { TVB_BREAK = 1, TVB_CONVERGED = 2, TVB_IMPROVED = 4, TVB_RUN = 8 };
struct TvBcast {
    float beta, alpha;
    int flag;
};

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
__device__ void tv_cgs(const TvVecs &V, int N, double tol, double *sh, TvBcast &bc) {
    const int P = N * N;
    const double n2b2 = tv_dot(V.rhs, V.rhs, P, sh);
    double n2b = 0.0, rho = 0.0, rho1 = 1.0, normrmin = 0.0;  // thread 0 only
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
        V.x[i] = 0.f;
        V.xmin[i] = 0.f;
        V.r[i] = V.rhs[i];
        V.rt[i] = V.rhs[i];
    }
    if (threadIdx.x == 0) {
        n2b = sqrt(n2b2);
        rho = n2b2;  // rt' r of the first step (rt = r = rhs)
        normrmin = n2b;
        bc.flag = n2b > 0.0 ? TVB_RUN : 0;
        bc.beta = 0.f;
    }
    __syncthreads();
    bool converged = false;
    if (bc.flag & TVB_RUN) {
        for (int it = 0; it < TV_CG_MAX; ++it) {
            const float beta = bc.beta;
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
            if (threadIdx.x == 0) {
                if (rtvh == 0.0 || !isfinite(rtvh)) {
                    bc.flag = TVB_BREAK;
                } else {
                    bc.flag = 0;
                    bc.alpha = (float)(rho / rtvh);
                }
            }
            __syncthreads();
            if (bc.flag & TVB_BREAK) break;
            const float alpha = bc.alpha;
            for (int i = threadIdx.x; i < P; i += blockDim.x) {
                const float qq = fmaf(-alpha, V.vh[i], V.uc[i]);
                V.q[i] = qq;
                const float uh = V.uc[i] + qq;
                V.uh[i] = uh;
                V.x[i] = fmaf(alpha, uh, V.x[i]);
            }
            __syncthreads();
            tv_apply_M(V.uh, V.vh, N);  // vh is free again: holds M uh
            float a_rr = 0.f;
            for (int i = threadIdx.x; i < P; i += blockDim.x) {
                const float rv = fmaf(-alpha, V.vh[i], V.r[i]);
                V.r[i] = rv;
                a_rr = fmaf(rv, rv, a_rr);
            }
            const double rr = tv_block_sum(a_rr, sh);
            const double rtr = tv_dot(V.rt, V.r, P, sh);
            if (threadIdx.x == 0) {
                const double normr = sqrt(rr);
                int f = 0;
                if (normr <= tol * n2b) {
                    f = TVB_CONVERGED;
                } else {
                    if (normr < normrmin) {
                        normrmin = normr;
                        f |= TVB_IMPROVED;
                    }
                    rho1 = rho;
                    rho = rtr;  // rt' r of the next step
                    if (rho == 0.0 || !isfinite(rho))
                        f |= TVB_BREAK;
                    else
                        bc.beta = (float)(rho / rho1);
                }
                bc.flag = f;
            }
            __syncthreads();
            const int f = bc.flag;
            if (f & TVB_CONVERGED) {
                converged = true;
                break;
            }
            if (f & TVB_IMPROVED) {
                for (int i = threadIdx.x; i < P; i += blockDim.x) V.xmin[i] = V.x[i];
            }
            if (f & TVB_BREAK) break;
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
    __shared__ TvBcast bc;
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
        tv_cgs(V, N, 1e-5, sh, bc);
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
        const double d2 = tv_block_sum(dif, sh);
        const double n2 = tv_block_sum(nrm, sh);
        if (threadIdx.x == 0) bc.flag = (!(n2 > 0.0) || sqrt(d2 / n2) <= 1e-3) ? TVB_BREAK : 0;
        __syncthreads();
        if (bc.flag & TVB_BREAK) break;
    }
    float *o = out_all + (size_t)w * P;
    for (int i = threadIdx.x; i < P; i += blockDim.x) o[i] = V.u[i];
}

// ---------------------------------------------------------------------------
// Cluster-resident prox: one thread-block cluster of C CTAs per image, CTA
// `rank` owning the column slab ix in [rank*nloc, rank*nloc + nl).  All
// eleven work vectors of the split-Bregman + CGS iteration live in shared
// memory (same layout in every CTA); the stencil's x-neighbours in the
// adjacent slabs are read through distributed shared memory.  Cluster-wide
// sums: every CTA adds the C per-CTA partials in rank order, so all CTAs
// see bitwise-identical scalars and take identical branches.
//
// The Bregman pair (b, d) is carried as Bub = B u + b only: with
// f = max(|Bub| - mu, 0) / |Bub| (0 where |Bub| = 0), d = f Bub,
// b = Bub - d and b - d = b - f Bub, so both are recomputed per pixel.
// ---------------------------------------------------------------------------
// iteration statistics of all prox launches (SB sweeps, CGS steps), read and
// reset by msot_tv_prox_stats
__device__ unsigned long long g_tv_stats[2];

constexpr int TVC_THREADS = 512;
constexpr int TVC_MAXC = 16;  // largest cluster
// u, x, bub1, bub2, r, rt, p (two buffers), q, uc, uh, vh, xmin
constexpr int TVC_NV = 13;
enum TvcVec { V_U = 0, V_X, V_B1, V_B2, V_R, V_RT, V_P0, V_P1, V_Q, V_UC, V_UH, V_VH, V_XMIN };

// Thread mapping inside a slab: thread t owns row iz = t % N of the columns
// lc = t / N, t / N + G, ... (G = TVC_THREADS / N column groups; N <= 512).
struct TvcCtx {
    float *sm;        // this CTA's vectors
    const float *sl;  // left neighbour's vectors (rank - 1), or null
    const float *sr;  // right neighbour's vectors (rank + 1), or null
    int N, nloc, nl, ix0, iz, G, lc0;
    bool zlo, zhi;
};

// the Bregman quantities b = Bub - d and b - d of one pixel from its Bub pair
__device__ __forceinline__ void tvc_bd(float a1, float a2, float mu, float &b1, float &b2,
                                       float &c1, float &c2) {
    const float s = sqrtf(fmaf(a1, a1, a2 * a2));
    const float f = s > 0.f ? fmaxf(s - mu, 0.f) / s : 0.f;
    const float d1 = f * a1, d2 = f * a2;
    b1 = a1 - d1;
    b2 = a2 - d2;
    c1 = b1 - d1;
    c2 = b2 - d2;
}

// value of vector o at the left / right x-neighbour of (lc, iz), element l
__device__ __forceinline__ float tvc_left(const TvcCtx &c, int o, int lc, int l) {
    return lc == 0 ? c.sl[o + (c.nloc - 1) * c.N + c.iz] : c.sm[o + l - c.N];
}
__device__ __forceinline__ float tvc_right(const TvcCtx &c, int o, int lc, int l) {
    return lc == c.nl - 1 ? c.sr[o + c.iz] : c.sm[o + l + c.N];
}

// (I + B'B) of vector oi at (lc, iz) (same stencil as tv_apply_M).  The
// x-neighbours in the adjacent slabs are not read from oi there: halo(base,
// k) recomputes them from that CTA's vectors (base = its shared memory, k =
// the element), with the same float operations the owner used.
template <class Halo>
__device__ __forceinline__ float tvc_M(const TvcCtx &c, int oi, int lc, int l, Halo halo) {
    const float *in = c.sm + oi;
    const int ix = c.ix0 + lc;
    const float v = in[l];
    const float g1 = c.zlo ? v - in[l - 1] : 0.f;
    const float g1n = c.zhi ? in[l + 1] - v : 0.f;
    float g2 = 0.f, g2n = 0.f;
    if (ix >= 1) g2 = v - (lc == 0 ? halo(c.sl, (c.nloc - 1) * c.N + c.iz) : in[l - c.N]);
    if (ix + 1 < c.N) g2n = (lc == c.nl - 1 ? halo(c.sr, c.iz) : in[l + c.N]) - v;
    return v + (g1 - g1n) + (g2 - g2n);
}

// Cluster-wide sums of two per-thread values, returned to every thread.
// Each CTA pushes its two block sums into slot [par][rank] of every CTA of
// the cluster (remote stores, then the barrier), and every thread adds the C
// slots of its own CTA in rank order: bitwise-identical results in all
// threads of all CTAs, so every thread evaluates the scalar recurrences
// itself and all take the same branches (no broadcast barrier).  Sums and
// scalars are FP32 like the vectors: they lie on every CGS step's critical
// path, and FP64 latency on GB300 is long.
__device__ __forceinline__ void tvc_reduce(float a, float b, float &A, float &B, float *wsum,
                                           float *red, int &par, int C, int rank) {
    namespace cg = cooperative_groups;
    cg::cluster_group cl = cg::this_cluster();
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b += __shfl_down_sync(0xffffffffu, b, o);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) {
        wsum[wid] = a;
        wsum[32 + wid] = b;
    }
    __syncthreads();
    if (wid == 0) {
        constexpr int NW = TVC_THREADS / 32;
        float da = lane < NW ? wsum[lane] : 0.f;
        float db = lane < NW ? wsum[32 + lane] : 0.f;
#pragma unroll
        for (int o = NW / 2; o > 0; o >>= 1) {
            da += __shfl_down_sync(0xffffffffu, da, o);
            db += __shfl_down_sync(0xffffffffu, db, o);
        }
        da = __shfl_sync(0xffffffffu, da, 0);
        db = __shfl_sync(0xffffffffu, db, 0);
        if (lane < C) {
            float *dst = cl.map_shared_rank(red, lane) + (par * TVC_MAXC + rank) * 2;
            dst[0] = da;
            dst[1] = db;
        }
    }
    cl.sync();
    const float *src = red + par * TVC_MAXC * 2;
    A = 0.f;
    B = 0.f;
    for (int r = 0; r < C; ++r) {
        A += src[2 * r];
        B += src[2 * r + 1];
    }
    par ^= 1;
}

// loop over this thread's elements (lc, l) of the slab
#define TVC_FOR(c) for (int lc = (c).lc0, l = lc * (c).N + (c).iz; lc < (c).nl; lc += (c).G, l += (c).G * (c).N)

// CGS step structure (per step two cluster barriers, both inside the sums):
//   uc = r + beta q ; p_new = uc + beta (q + beta p_old)     (local)
//   __syncthreads ; vh = M p_new, halo p_new from the neighbour's r, q, p_old
//   sum rt'vh -> alpha
//   q = uc - alpha vh ; uh = uc + q ; x += alpha uh         (local)
//   __syncthreads ; r -= alpha M uh, halo uh from the neighbour's uc, vh
//   sum r'r, rt'r -> convergence, beta
// p alternates between two buffers so that a neighbour can still read p_old
// while this CTA writes p_new; every vector read remotely in a phase was
// written before the barrier that opened the phase.
__global__ void __launch_bounds__(TVC_THREADS, 2)
    k_tv_prox_cl(const float *__restrict__ g_all, const TvState *__restrict__ st, double mu_const,
                 int coupled, float *__restrict__ out_all, int N, int C, int nloc) {
    namespace cg = cooperative_groups;
    extern __shared__ float4 tvc_smem[];
    __shared__ float wsum[64];
    __shared__ float red[2 * TVC_MAXC * 2];
    cg::cluster_group cl = cg::this_cluster();
    const int rank = (int)cl.block_rank();
    const int w = blockIdx.x / C, gw = coupled ? 0 : w;
    if (st && st[gw].done) return;  // uniform over the cluster
    TvcCtx c;
    c.sm = reinterpret_cast<float *>(tvc_smem);
    c.N = N;
    c.nloc = nloc;
    c.ix0 = rank * nloc;
    c.nl = max(0, min(nloc, N - c.ix0));
    c.G = TVC_THREADS / N;
    c.iz = threadIdx.x % N;
    c.lc0 = (int)threadIdx.x / N;
    if (c.lc0 >= c.G) c.lc0 = c.nl;  // idle thread: empty loops
    c.zlo = c.iz >= 1;
    c.zhi = c.iz + 1 < N;
    c.sl = rank > 0 ? cl.map_shared_rank(c.sm, rank - 1) : nullptr;
    c.sr = rank + 1 < C ? cl.map_shared_rank(c.sm, rank + 1) : nullptr;
    const float mu = (float)(st ? st[gw].mu : mu_const);
    const float *g = g_all + (size_t)w * N * N + (size_t)c.ix0 * N;
    const int V = nloc * N;
    float *S = c.sm;
    int ou = V_U * V, ox = V_X * V;  // swapped after every sweep
    const int ob1 = V_B1 * V, ob2 = V_B2 * V, orr = V_R * V, ort = V_RT * V, oq = V_Q * V,
              ouc = V_UC * V, ouh = V_UH * V, ovh = V_VH * V, oxm = V_XMIN * V;
    int op = V_P0 * V, opo = V_P1 * V;  // p_new, p_old
    int par = 0, n_sweeps = 0, n_cg = 0;
    float A = 0.f, B = 0.f;
    float n2b = 0.f, rho = 0.f, rho1 = 1.f, normrmin = 0.f;
    TVC_FOR(c) {
        S[ou + l] = g[l];
        S[ob1 + l] = 0.f;
        S[ob2 + l] = 0.f;
    }
    cl.sync();
    for (int it = 0; it < TV_SB_MAX; ++it) {
        ++n_sweeps;
        // rhs = g - B'(b - d); r = rt = rhs; x = xmin = 0
        float n2 = 0.f;
        TVC_FOR(c) {
            const int ix = c.ix0 + lc;
            float b1, b2, c1, c2, t1, t2, e1, e2;
            tvc_bd(S[ob1 + l], S[ob2 + l], mu, b1, b2, c1, c2);
            float acc = 0.f;
            if (c.zlo) acc += c1;
            if (c.zhi) {
                tvc_bd(S[ob1 + l + 1], S[ob2 + l + 1], mu, t1, t2, e1, e2);
                acc -= e1;
            }
            float acc2 = 0.f;
            if (ix >= 1) acc2 += c2;
            if (ix + 1 < N) {
                tvc_bd(tvc_right(c, ob1, lc, l), tvc_right(c, ob2, lc, l), mu, t1, t2, e1, e2);
                acc2 -= e2;
            }
            const float rhs = g[l] - (acc + acc2);
            S[orr + l] = rhs;
            S[ort + l] = rhs;
            S[ox + l] = 0.f;
            S[oxm + l] = 0.f;
            n2 = fmaf(rhs, rhs, n2);
        }
        tvc_reduce(n2, 0.f, A, B, wsum, red, par, C, rank);
        n2b = sqrtf(A);
        rho = A;  // rt' r of the first step (rt = r = rhs)
        rho1 = 1.f;
        normrmin = n2b;
        float beta_next = 0.f;
        bool converged = false;
        if (n2b > 0.f) {
            for (int cit = 0; cit < TV_CG_MAX; ++cit) {
                ++n_cg;
                const float beta = beta_next;
                {
                    const int t = op;
                    op = opo;
                    opo = t;
                }
                if (cit == 0) {
                    TVC_FOR(c) {
                        const float rv = S[orr + l];
                        S[ouc + l] = rv;
                        S[op + l] = rv;
                    }
                } else {
                    TVC_FOR(c) {
                        const float qv = S[oq + l];
                        const float uv = fmaf(beta, qv, S[orr + l]);
                        S[ouc + l] = uv;
                        S[op + l] = fmaf(beta, fmaf(beta, S[opo + l], qv), uv);
                    }
                }
                __syncthreads();  // p_new complete in this slab
                const bool first = cit == 0;
                const int opo_ = opo;
                auto halo_p = [=](const float *b, int k) {
                    const float rv = b[orr + k];
                    if (first) return rv;
                    const float qv = b[oq + k];
                    const float uv = fmaf(beta, qv, rv);
                    return fmaf(beta, fmaf(beta, b[opo_ + k], qv), uv);
                };
                float a_rtvh = 0.f;
                TVC_FOR(c) {
                    const float vhv = tvc_M(c, op, lc, l, halo_p);
                    S[ovh + l] = vhv;
                    a_rtvh = fmaf(S[ort + l], vhv, a_rtvh);
                }
                tvc_reduce(a_rtvh, 0.f, A, B, wsum, red, par, C, rank);
                if (A == 0.f || !isfinite(A)) break;
                const float alpha = rho / A;
                TVC_FOR(c) {
                    const float uv = S[ouc + l];
                    const float qq = fmaf(-alpha, S[ovh + l], uv);
                    S[oq + l] = qq;
                    const float uh = uv + qq;
                    S[ouh + l] = uh;
                    S[ox + l] = fmaf(alpha, uh, S[ox + l]);
                }
                __syncthreads();  // uh complete in this slab
                auto halo_uh = [=](const float *b, int k) {
                    const float uv = b[ouc + k];
                    return uv + fmaf(-alpha, b[ovh + k], uv);
                };
                float a_rr = 0.f, a_rtr = 0.f;
                TVC_FOR(c) {
                    const float rv = fmaf(-alpha, tvc_M(c, ouh, lc, l, halo_uh), S[orr + l]);
                    S[orr + l] = rv;
                    a_rr = fmaf(rv, rv, a_rr);
                    a_rtr = fmaf(S[ort + l], rv, a_rtr);
                }
                tvc_reduce(a_rr, a_rtr, A, B, wsum, red, par, C, rank);
                int f = 0;
                {
                    const float normr = sqrtf(A);
                    if (normr <= 1e-5f * n2b) {
                        f = TVB_CONVERGED;
                    } else {
                        if (normr < normrmin) {
                            normrmin = normr;
                            f |= TVB_IMPROVED;
                        }
                        rho1 = rho;
                        rho = B;  // rt' r of the next step
                        if (rho == 0.f || !isfinite(rho))
                            f |= TVB_BREAK;
                        else
                            beta_next = rho / rho1;
                    }
                }
                if (f & TVB_CONVERGED) {
                    converged = true;
                    break;
                }
                if (f & TVB_IMPROVED) {
                    TVC_FOR(c) S[oxm + l] = S[ox + l];
                }
                if (f & TVB_BREAK) break;
            }
        }
        if (!converged) {
            TVC_FOR(c) S[ox + l] = S[oxm + l];
        }
        cl.sync();  // new u (in x) complete in every slab
        // Bub = B u + b ; change of u
        float dif = 0.f, nrm = 0.f;
        TVC_FOR(c) {
            float b1, b2, c1, c2;
            tvc_bd(S[ob1 + l], S[ob2 + l], mu, b1, b2, c1, c2);
            const float v = S[ox + l];
            S[ob1 + l] = (c.zlo ? v - S[ox + l - 1] : 0.f) + b1;
            S[ob2 + l] = (c.ix0 + lc >= 1 ? v - tvc_left(c, ox, lc, l) : 0.f) + b2;
            const float e = S[ou + l] - v;
            dif = fmaf(e, e, dif);
            nrm = fmaf(v, v, nrm);
        }
        tvc_reduce(dif, nrm, A, B, wsum, red, par, C, rank);
        const bool stop = !(B > 0.f) || sqrtf(A / B) <= 1e-3f;
        const int t = ou;
        ou = ox;
        ox = t;
        if (stop) break;
    }
    float *o = out_all + (size_t)w * N * N + (size_t)c.ix0 * N;
    TVC_FOR(c) o[l] = S[ou + l];
    if (rank == 0 && threadIdx.x == 0) {
        atomicAdd(&g_tv_stats[0], (unsigned long long)n_sweeps);
        atomicAdd(&g_tv_stats[1], (unsigned long long)n_cg);
    }
    cl.sync();  // no CTA leaves while a neighbour may still read its shared memory
}
#undef TVC_FOR

// ---------------------------------------------------------------------------
// The same cluster prox with 4 consecutive z-pixels per thread (N % 4 == 0):
// 128-bit shared-memory accesses; thread t owns group jz = t % (N/4) (pixels
// 4 jz .. 4 jz + 3) of the columns lc = t / (N/4), ... + G.  The split-Bregman
// sweep is the scalar kernel's; its CGS step is the same recurrence written
// with one CTA barrier less, carrying M p and M q instead of p and uh (M =
// I + B'B is linear, so M p_new = M uc + beta (M q + beta M p_old) and
// M uh = M uc + M q, M q = M uc - alpha M vh):
//   A  uc = r + beta q                                        (local)
//      __syncthreads
//   B  Muc = M uc (halo uc from the neighbour's r, q); vh = Muc + beta (Mq +
//      beta vh); sum rt'vh -> alpha
//   C  Mvh = M vh (halo vh from the neighbour); q = uc - alpha vh;
//      Mq = Muc - alpha Mvh; x += alpha (uc + q); r -= alpha (Muc + Mq);
//      sums r'r, rt'r -> convergence, beta
// Two stencils and two cluster sums per step, as before; every vector read
// remotely in a phase was written before the cluster barrier that opened
// it, and is rewritten only after the next one.
// ---------------------------------------------------------------------------
struct F4 {
    float v[4];
};
__device__ __forceinline__ F4 ld4(const float *p) {
    const float4 a = *reinterpret_cast<const float4 *>(p);
    return F4{{a.x, a.y, a.z, a.w}};
}
__device__ __forceinline__ void st4(float *p, const F4 &a) {
    *reinterpret_cast<float4 *>(p) = make_float4(a.v[0], a.v[1], a.v[2], a.v[3]);
}

struct Tvc4Ctx {
    float *sm;
    const float *sl, *sr;
    int N, nloc, nl, ix0, iz0, G, lc0;
};

// a neighbour slab's float4: shared memory of the neighbour CTA, or (GM)
// global memory written by another SM, read past L1
template <bool GM>
__device__ __forceinline__ F4 ld4n(const float *p) {
    if constexpr (GM) {
        const float4 a = __ldcg(reinterpret_cast<const float4 *>(p));
        return F4{{a.x, a.y, a.z, a.w}};
    } else {
        return ld4(p);
    }
}

// (I + B'B) in of the 4 pixels at (lc, iz0 .. iz0 + 3), element l = lc N + iz0
template <class Halo>
__device__ __forceinline__ F4 tvc4_M(const Tvc4Ctx &c, int oi, int lc, int l, Halo halo) {
    const float *in = c.sm + oi;
    const int ix = c.ix0 + lc;
    const F4 v = ld4(in + l);
    float a[6];
    a[0] = c.iz0 >= 1 ? in[l - 1] : 0.f;
#pragma unroll
    for (int k = 0; k < 4; ++k) a[k + 1] = v.v[k];
    a[5] = c.iz0 + 4 < c.N ? in[l + 4] : 0.f;
    F4 L{}, R{};
    if (ix >= 1) L = lc == 0 ? halo(c.sl, (c.nloc - 1) * c.N + c.iz0) : ld4(in + l - c.N);
    if (ix + 1 < c.N) R = lc == c.nl - 1 ? halo(c.sr, c.iz0) : ld4(in + l + c.N);
    F4 o;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int iz = c.iz0 + k;
        const float x = a[k + 1];
        const float g1 = iz >= 1 ? x - a[k] : 0.f;
        const float g1n = iz + 1 < c.N ? a[k + 2] - x : 0.f;
        const float g2 = ix >= 1 ? x - L.v[k] : 0.f;
        const float g2n = ix + 1 < c.N ? R.v[k] - x : 0.f;
        o.v[k] = x + (g1 - g1n) + (g2 - g2n);
    }
    return o;
}

#define TVC4_FOR(c) for (int lc = (c).lc0, l = lc * (c).N + (c).iz0; lc < (c).nl; lc += (c).G, l += (c).G * (c).N)

template <bool GM>
__global__ void __launch_bounds__(TVC_THREADS, 2)
    k_tv_prox_cl4(const float *__restrict__ g_all, const TvState *__restrict__ st,
                  double mu_const, int coupled, float *__restrict__ out_all, int N, int C,
                  int nloc, float *__restrict__ gwork) {
    namespace cg = cooperative_groups;
    extern __shared__ float4 tvc_smem[];
    __shared__ float wsum[64];
    __shared__ float red[2 * TVC_MAXC * 2];
    cg::cluster_group cl = cg::this_cluster();
    const int rank = (int)cl.block_rank();
    const int w = blockIdx.x / C, gw = coupled ? 0 : w;
    if (st && st[gw].done) return;  // uniform over the cluster
    Tvc4Ctx c;
    c.N = N;
    c.nloc = nloc;
    c.ix0 = rank * nloc;
    c.nl = max(0, min(nloc, N - c.ix0));
    const int NG = N / 4;
    c.G = TVC_THREADS / NG;
    c.iz0 = 4 * ((int)threadIdx.x % NG);
    c.lc0 = (int)threadIdx.x / NG;
    if (c.lc0 >= c.G) c.lc0 = c.nl;  // idle thread
    if constexpr (GM) {
        // slabs of the cluster's CTAs are consecutive in the workspace
        const size_t slab = (size_t)TVC_NV * nloc * N;
        c.sm = gwork + ((size_t)w * C + rank) * slab;
        c.sl = rank > 0 ? c.sm - slab : nullptr;
        c.sr = rank + 1 < C ? c.sm + slab : nullptr;
    } else {
        c.sm = reinterpret_cast<float *>(tvc_smem);
        c.sl = rank > 0 ? cl.map_shared_rank(c.sm, rank - 1) : nullptr;
        c.sr = rank + 1 < C ? cl.map_shared_rank(c.sm, rank + 1) : nullptr;
    }
    const float mu = (float)(st ? st[gw].mu : mu_const);
    const float *g = g_all + (size_t)w * N * N + (size_t)c.ix0 * N;
    const int V = nloc * N;
    float *S = c.sm;
    int ou = V_U * V, ox = V_X * V;
    const int ob1 = V_B1 * V, ob2 = V_B2 * V, orr = V_R * V, ort = V_RT * V, oq = V_Q * V,
              ouc = V_UC * V, ovh = V_VH * V, oxm = V_XMIN * V;
    const int omq = V_P0 * V, omuc = V_P1 * V;  // M q and M uc (no p, no uh here)
    int par = 0, n_sweeps = 0, n_cg = 0;
    float A = 0.f, B = 0.f;
    float n2b = 0.f, rho = 0.f, rho1 = 1.f, normrmin = 0.f;
    const F4 zero4{{0.f, 0.f, 0.f, 0.f}};
    TVC4_FOR(c) {
        st4(S + ou + l, ld4(g + l));
        st4(S + ob1 + l, zero4);
        st4(S + ob2 + l, zero4);
    }
    cl.sync();
    for (int it = 0; it < TV_SB_MAX; ++it) {
        ++n_sweeps;
        float n2 = 0.f;
        TVC4_FOR(c) {
            const int ix = c.ix0 + lc;
            const F4 B1 = ld4(S + ob1 + l), B2 = ld4(S + ob2 + l), G4 = ld4(g + l);
            float c1[5], c2[4];
            for (int k = 0; k < 4; ++k) {
                float b1, b2;
                tvc_bd(B1.v[k], B2.v[k], mu, b1, b2, c1[k], c2[k]);
            }
            if (c.iz0 + 4 < N) {
                float b1, b2, e2;
                tvc_bd(S[ob1 + l + 4], S[ob2 + l + 4], mu, b1, b2, c1[4], e2);
            } else {
                c1[4] = 0.f;
            }
            float e2r[4] = {0.f, 0.f, 0.f, 0.f};
            if (ix + 1 < N) {
                const F4 R1 = lc == c.nl - 1 ? ld4n<GM>(c.sr + ob1 + c.iz0) : ld4(S + ob1 + l + N);
                const F4 R2 = lc == c.nl - 1 ? ld4n<GM>(c.sr + ob2 + c.iz0) : ld4(S + ob2 + l + N);
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    float b1, b2, e1;
                    tvc_bd(R1.v[k], R2.v[k], mu, b1, b2, e1, e2r[k]);
                }
            }
            F4 rh;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int iz = c.iz0 + k;
                float acc = 0.f;
                if (iz >= 1) acc += c1[k];
                if (iz + 1 < N) acc -= c1[k + 1];
                float acc2 = 0.f;
                if (ix >= 1) acc2 += c2[k];
                if (ix + 1 < N) acc2 -= e2r[k];
                rh.v[k] = G4.v[k] - (acc + acc2);
                n2 = fmaf(rh.v[k], rh.v[k], n2);
            }
            st4(S + orr + l, rh);
            st4(S + ort + l, rh);
            st4(S + ox + l, zero4);
            st4(S + oxm + l, zero4);
        }
        tvc_reduce(n2, 0.f, A, B, wsum, red, par, C, rank);
        n2b = sqrtf(A);
        rho = A;
        rho1 = 1.f;
        normrmin = n2b;
        float beta_next = 0.f;
        bool converged = false;
        if (n2b > 0.f) {
            for (int cit = 0; cit < TV_CG_MAX; ++cit) {
                ++n_cg;
                const float beta = beta_next;
                const bool first = cit == 0;
                // A: uc = r + beta q
                TVC4_FOR(c) {
                    const F4 rv = ld4(S + orr + l);
                    if (first) {
                        st4(S + ouc + l, rv);
                    } else {
                        const F4 qv = ld4(S + oq + l);
                        F4 uv;
#pragma unroll
                        for (int k = 0; k < 4; ++k) uv.v[k] = fmaf(beta, qv.v[k], rv.v[k]);
                        st4(S + ouc + l, uv);
                    }
                }
                __syncthreads();
                // B: Muc = M uc (halo uc from the neighbour's r and q);
                //    vh = M p_new = Muc + beta (Mq + beta vh_old)
                auto halo_uc = [=](const float *b, int k) {
                    const F4 rv = ld4n<GM>(b + orr + k);
                    if (first) return rv;
                    const F4 qv = ld4n<GM>(b + oq + k);
                    F4 o;
#pragma unroll
                    for (int m = 0; m < 4; ++m) o.v[m] = fmaf(beta, qv.v[m], rv.v[m]);
                    return o;
                };
                float a_rtvh = 0.f;
                TVC4_FOR(c) {
                    const F4 muc = tvc4_M(c, ouc, lc, l, halo_uc);
                    st4(S + omuc + l, muc);
                    F4 vh = muc;
                    if (!first) {
                        const F4 mq = ld4(S + omq + l), vo = ld4(S + ovh + l);
#pragma unroll
                        for (int k = 0; k < 4; ++k)
                            vh.v[k] = fmaf(beta, fmaf(beta, vo.v[k], mq.v[k]), muc.v[k]);
                    }
                    st4(S + ovh + l, vh);
                    const F4 rt = ld4(S + ort + l);
#pragma unroll
                    for (int k = 0; k < 4; ++k) a_rtvh = fmaf(rt.v[k], vh.v[k], a_rtvh);
                }
                tvc_reduce(a_rtvh, 0.f, A, B, wsum, red, par, C, rank);
                if (A == 0.f || !isfinite(A)) break;
                const float alpha = rho / A;
                // C: Mvh = M vh (halo vh read from the neighbour); q = uc - alpha vh,
                //    Mq = Muc - alpha Mvh, x += alpha (uc + q), r -= alpha (Muc + Mq)
                auto halo_vh = [=](const float *b, int k) { return ld4n<GM>(b + ovh + k); };
                float a_rr = 0.f, a_rtr = 0.f;
                TVC4_FOR(c) {
                    const F4 mv = tvc4_M(c, ovh, lc, l, halo_vh);
                    const F4 uv = ld4(S + ouc + l), vh = ld4(S + ovh + l), muc = ld4(S + omuc + l);
                    const F4 xv = ld4(S + ox + l), rv = ld4(S + orr + l), rt = ld4(S + ort + l);
                    F4 q, mq, xn, rn;
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        q.v[k] = fmaf(-alpha, vh.v[k], uv.v[k]);
                        mq.v[k] = fmaf(-alpha, mv.v[k], muc.v[k]);
                        xn.v[k] = fmaf(alpha, uv.v[k] + q.v[k], xv.v[k]);
                        rn.v[k] = fmaf(-alpha, muc.v[k] + mq.v[k], rv.v[k]);
                        a_rr = fmaf(rn.v[k], rn.v[k], a_rr);
                        a_rtr = fmaf(rt.v[k], rn.v[k], a_rtr);
                    }
                    st4(S + oq + l, q);
                    st4(S + omq + l, mq);
                    st4(S + ox + l, xn);
                    st4(S + orr + l, rn);
                }
                tvc_reduce(a_rr, a_rtr, A, B, wsum, red, par, C, rank);
                int f = 0;
                {
                    const float normr = sqrtf(A);
                    if (normr <= 1e-5f * n2b) {
                        f = TVB_CONVERGED;
                    } else {
                        if (normr < normrmin) {
                            normrmin = normr;
                            f |= TVB_IMPROVED;
                        }
                        rho1 = rho;
                        rho = B;  // rt' r of the next step
                        if (rho == 0.f || !isfinite(rho))
                            f |= TVB_BREAK;
                        else
                            beta_next = rho / rho1;
                    }
                }
                if (f & TVB_CONVERGED) {
                    converged = true;
                    break;
                }
                if (f & TVB_IMPROVED) {
                    TVC4_FOR(c) st4(S + oxm + l, ld4(S + ox + l));
                }
                if (f & TVB_BREAK) break;
            }
        }
        if (!converged) {
            TVC4_FOR(c) st4(S + ox + l, ld4(S + oxm + l));
        }
        cl.sync();
        float dif = 0.f, nrm = 0.f;
        TVC4_FOR(c) {
            const int ix = c.ix0 + lc;
            const F4 B1 = ld4(S + ob1 + l), B2 = ld4(S + ob2 + l), X = ld4(S + ox + l),
                     U = ld4(S + ou + l);
            float xa[5];
            xa[0] = c.iz0 >= 1 ? S[ox + l - 1] : 0.f;
#pragma unroll
            for (int k = 0; k < 4; ++k) xa[k + 1] = X.v[k];
            F4 Lx{};
            if (ix >= 1)
                Lx = lc == 0 ? ld4n<GM>(c.sl + ox + (c.nloc - 1) * N + c.iz0) : ld4(S + ox + l - N);
            F4 n1, n2v;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                float b1, b2, cc1, cc2;
                tvc_bd(B1.v[k], B2.v[k], mu, b1, b2, cc1, cc2);
                const float v = X.v[k];
                n1.v[k] = (c.iz0 + k >= 1 ? v - xa[k] : 0.f) + b1;
                n2v.v[k] = (ix >= 1 ? v - Lx.v[k] : 0.f) + b2;
                const float e = U.v[k] - v;
                dif = fmaf(e, e, dif);
                nrm = fmaf(v, v, nrm);
            }
            st4(S + ob1 + l, n1);
            st4(S + ob2 + l, n2v);
        }
        tvc_reduce(dif, nrm, A, B, wsum, red, par, C, rank);
        const bool stop = !(B > 0.f) || sqrtf(A / B) <= 1e-3f;
        const int t = ou;
        ou = ox;
        ox = t;
        if (stop) break;
    }
    float *o = out_all + (size_t)w * N * N + (size_t)c.ix0 * N;
    TVC4_FOR(c) st4(o + l, ld4(S + ou + l));
    if (rank == 0 && threadIdx.x == 0) {
        atomicAdd(&g_tv_stats[0], (unsigned long long)n_sweeps);
        atomicAdd(&g_tv_stats[1], (unsigned long long)n_cg);
    }
    cl.sync();
}
#undef TVC4_FOR

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


__device__ __forceinline__ void tv_store(float v, double *part, int q, int W, double *sh) {
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

int blocks_per_instance(int W) {
    return std::max(1, std::min(64, (4 * sm_count() + W - 1) / W));
}

// 0: cluster path where it fits, 1: force the global-memory kernel
std::atomic<int> g_prox_path{0};

// cluster geometry of the shared-memory-resident prox for an N x N image:
// the smallest cluster whose slab fits two CTAs per SM (portable sizes up to
// 8), else one CTA per SM (up to 16); none if the image does not fit.
struct TvcGeom {
    int C = 0, nloc = 0;
    size_t smem = 0;
};

// forced cluster size (msot_tune_set), 0 = automatic, -1 = the 16-CTA
// cluster with its vectors in the global-memory workspace
std::atomic<int> g_tv_cluster{0};

TvcGeom tvc_geometry(int N, int force = 0) {
    TvcGeom g;
    if (N > TVC_THREADS) return g;
    if (const int Cf = force ? force : g_tv_cluster.load()) {
        if (Cf < 0) return g;  // no shared-memory geometry: the global-memory form
        const int nloc = (N + Cf - 1) / Cf;
        const size_t bytes = (size_t)TVC_NV * nloc * N * sizeof(float);
        if (bytes <= 225 * 1024) {
            g.C = Cf;
            g.nloc = nloc;
            g.smem = bytes;
        }
        return g;
    }
    const size_t two_per_sm = 113 * 1024, one_per_sm = 225 * 1024;
    for (int pass = 0; pass < 2; ++pass) {
        for (int C = 1; C <= (pass ? 16 : 8); C *= 2) {
            const int nloc = (N + C - 1) / C;
            const size_t bytes = (size_t)TVC_NV * nloc * N * sizeof(float);
            if (bytes <= (pass ? one_per_sm : two_per_sm)) {
                g.C = C;
                g.nloc = nloc;
                g.smem = bytes;
                return g;
            }
        }
    }
    return g;
}

template <class K>
static cudaError_t tvc_config(K kern, const TvcGeom &gm, int W, cudaStream_t st,
                              cudaLaunchConfig_t &cfg, cudaLaunchAttribute *at, bool &fits) {
    cudaError_t e = raise_max_dynamic_smem((const void *)kern, gm.smem);
    if (e != cudaSuccess) return e;
    if (gm.C > 8) {
        e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        if (e != cudaSuccess) return e;
    }
    cfg = cudaLaunchConfig_t{};
    cfg.gridDim = dim3((unsigned)(W * gm.C));
    cfg.blockDim = dim3(TVC_THREADS);
    cfg.dynamicSmemBytes = gm.smem;
    cfg.stream = st;
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = (unsigned)gm.C;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int clusters = 0;
    e = cudaOccupancyMaxActiveClusters(&clusters, kern, &cfg);
    if (e != cudaSuccess || clusters < 1) {
        (void)cudaGetLastError();
        fits = false;
        return cudaSuccess;
    }
    fits = true;
    return cudaSuccess;
}

cudaError_t tvc_launch(const TvcGeom &gm, const float *z, const TvState *sv, double mu,
                       int coupled, float *out, int W, int N, cudaStream_t st, bool &fits) {
    cudaLaunchConfig_t cfg;
    cudaLaunchAttribute at[1];
    // 4 z-pixels per thread where N allows (16-byte aligned groups)
    if (N % 4 == 0 && N / 4 <= TVC_THREADS) {
        cudaError_t e = tvc_config(k_tv_prox_cl4<false>, gm, W, st, cfg, at, fits);
        if (e != cudaSuccess || !fits) return e;
        ++g_launch_count;
        return cudaLaunchKernelEx(&cfg, k_tv_prox_cl4<false>, z, sv, mu, coupled, out, N, gm.C,
                                  gm.nloc, (float *)nullptr);
    }
    cudaError_t e = tvc_config(k_tv_prox_cl, gm, W, st, cfg, at, fits);
    if (e != cudaSuccess || !fits) return e;
    ++g_launch_count;
    return cudaLaunchKernelEx(&cfg, k_tv_prox_cl, z, sv, mu, coupled, out, N, gm.C, gm.nloc);
}

// cluster of 16 CTAs per image with the work vectors in `work` (L2-resident)
// for images too large for shared memory (N % 4 == 0); false if it cannot
// run here
cudaError_t tvc_launch_gm(const float *z, const TvState *sv, double mu, int coupled, float *out,
                          float *work, int W, int N, cudaStream_t st, bool &ran) {
    ran = false;
    const int C = 16, nloc = (N + C - 1) / C;
    // the slabs must fit the workspace of TV_NVEC vectors per image
    if (N % 4 != 0 || N / 4 > TVC_THREADS || (size_t)C * TVC_NV * nloc > (size_t)TV_NVEC * N)
        return cudaSuccess;
    auto kern = k_tv_prox_cl4<true>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(W * C));
    cfg.blockDim = dim3(TVC_THREADS);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = (unsigned)C;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int clusters = 0;
    e = cudaOccupancyMaxActiveClusters(&clusters, kern, &cfg);
    if (e != cudaSuccess || clusters < 1) {
        (void)cudaGetLastError();
        return cudaSuccess;
    }
    ran = true;
    ++g_launch_count;
    return cudaLaunchKernelEx(&cfg, kern, z, sv, mu, coupled, out, N, C, nloc, work);
}

// SB_ITV2 of W images: the cluster kernel where it fits, else the
// global-memory kernel on `work` (TV_NVEC vectors per image)

int tv_prox(const float *z, const TvState *sv, double mu, int coupled, float *out, float *work,
            int W, int N, cudaStream_t st, int cluster) {
    TimedScope ts(KID_TV_PROX, st);
    const TvcGeom gm = tvc_geometry(N, cluster);
    if (g_prox_path.load() == 0 && gm.C) {
        bool fits = false;
        const cudaError_t e = tvc_launch(gm, z, sv, mu, coupled, out, W, N, st, fits);
        if (e != cudaSuccess) {
            set_error("tv prox (cluster %d): %s", gm.C, cudaGetErrorString(e));
            return MSOT_ECUDA;
        }
        if (fits) return MSOT_OK;
    }
    if (!work) {
        set_error("tv prox: no workspace for the global-memory path");
        return MSOT_EINVAL;
    }
    if (g_prox_path.load() == 0) {
        bool ran = false;
        const cudaError_t e = tvc_launch_gm(z, sv, mu, coupled, out, work, W, N, st, ran);
        if (e != cudaSuccess) {
            set_error("tv prox (cluster, global vectors): %s", cudaGetErrorString(e));
            return MSOT_ECUDA;
        }
        if (ran) return MSOT_OK;
    }
    KLAUNCH(k_tv_prox<<<W, TV_THREADS, 0, st>>>(z, sv, mu, coupled, out, work, N));
    MSOT_LAUNCH_CHECK();
    return MSOT_OK;
}

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
    float *work = b.get<float>((size_t)batch * TV_NVEC * P);  // global-memory path only
    if (!b.ok) {
        set_error("sb_itv2: device allocation failed");
        return MSOT_ENOMEM;
    }
    int rc = tv_prox(d_g, nullptr, mu, 1, d_u, work, batch, n, st, 0);
    if (rc) return rc;
    MSOT_CUDA_TRY(cudaStreamSynchronize(st));
    return MSOT_OK;
}

int msot_tv_prox_stats(long long *sweeps, long long *cg_steps) {
    unsigned long long h[2] = {0, 0}, z[2] = {0, 0};
    MSOT_CUDA_TRY(cudaDeviceSynchronize());
    MSOT_CUDA_TRY(cudaMemcpyFromSymbol(h, g_tv_stats, sizeof(h)));
    MSOT_CUDA_TRY(cudaMemcpyToSymbol(g_tv_stats, z, sizeof(z)));
    if (sweeps) *sweeps = (long long)h[0];
    if (cg_steps) *cg_steps = (long long)h[1];
    return MSOT_OK;
}

int msot_tune_set(const char *key, int value) {
    if (key && std::strcmp(key, "adj_prefetch") == 0 && (value == 0 || value == 1)) {
        msot::g_adj_prefetch.store(value);
        return MSOT_OK;
    }
    if (key && std::strcmp(key, "conv_min_blocks") == 0 &&
        (value == 1 || value == 3 || value == 4)) {
        msot::g_conv_min_blocks.store(value);
        return MSOT_OK;
    }
    if (key && std::strcmp(key, "unet_tensor_cores") == 0 && (value == 0 || value == 1)) {
        msot::g_unet_tc.store(value);
        return MSOT_OK;
    }
    if (key && std::strcmp(key, "fwd_staged") == 0 && (value == 0 || value == 1)) {
        msot::g_fwd_staged.store(value);
        return MSOT_OK;
    }
    if (key && std::strcmp(key, "fwd_staged_tile") == 0 &&
        (value == 0 || value == 8 || value == 16 || value == 32 || value == 64)) {
        msot::g_st_force_tt.store(value);
        return MSOT_OK;
    }
    if (key && std::strcmp(key, "fwd_staged_group") == 0 &&
        (value == 0 || value == 1 || value == 2 || value == 4 || value == 8 || value == 16)) {
        msot::g_st_force_g.store(value);
        return MSOT_OK;
    }
    if (key && std::strcmp(key, "fwd_ell") == 0 && (value == 0 || value == 1)) {
        msot::g_fwd_ell.store(value);
        return MSOT_OK;
    }
    if (key && std::strcmp(key, "tv_prox_cluster") == 0 &&
        (value == -1 || value == 0 || value == 1 || value == 2 || value == 4 || value == 8 ||
         value == 16)) {
        g_tv_cluster.store(value);
        return MSOT_OK;
    }
    set_error("tune_set: unknown key or value out of range");
    return MSOT_EINVAL;
}

int msot_tv_prox_path(int path) {
    if (path < 0 || path > 1) {
        set_error("tv_prox_path: 0 (automatic) or 1 (global-memory kernel)");
        return MSOT_EINVAL;
    }
    g_prox_path.store(path);
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

}  // extern "C"

namespace {
// a non-blocking stream that starts after the work queued on `user` and
// makes `user` wait for everything queued on it when it closes
struct TvStream {
    cudaStream_t s = nullptr, user = nullptr;
    cudaEvent_t ev = nullptr;
    int open(cudaStream_t u) {
        user = u;
        if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) {
            set_error("rec_nn_with_TV_reg: stream creation failed");
            return MSOT_ECUDA;
        }
        cudaEventRecord(ev, user);
        cudaStreamWaitEvent(s, ev, 0);
        return MSOT_OK;
    }
    ~TvStream() {
        if (s) {
            cudaEventRecord(ev, s);
            cudaStreamWaitEvent(user, ev, 0);
            cudaStreamSynchronize(s);
            cudaStreamDestroy(s);
        }
        if (ev) cudaEventDestroy(ev);
    }
};
}  // namespace

extern "C" {

int msot_rec_nn_with_TV_reg(msot_plan_t plan, const float *d_b, float *d_rec, int batch,
                            int num_iter, double reg, int sparsa_iter, const float *d_x0,
                            int coupled, double *err_img, double *err_reg, void *stream) {
    if (!plan || !d_b || !d_rec || batch <= 0 || num_iter < 0 || sparsa_iter < 1 ||
        !(reg >= 0.0)) {
        set_error("rec_nn_with_TV_reg: bad arguments");
        return MSOT_EINVAL;
    }
    const Plan &pl = plan->p;
    if (int rc = check_plan_device(pl, "rec_nn_with_TV_reg")) return rc;
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
    // One outer iteration is a fixed launch sequence with device-side scalars
    // (no host synchronisation): the first runs eagerly (kernel attributes),
    // the next is captured once as a CUDA graph on a private stream and
    // replayed for the remaining iterations.
    auto outer_step = [&](cudaStream_t s) -> int {
        int r;
        KLAUNCH(k_tv_begin<<<grid, TV_RED, 0, s>>>(wv, vm, x, ri, N, sb, W, part));
        MSOT_LAUNCH_CHECK();
        if ((r = apply_forward(pl, x, As, W, s))) return r;
        KLAUNCH(k_tv_rs0<<<grid, TV_RED, 0, s>>>(d_b, As, rs, ns, sl, W, part));
        KLAUNCH(k_tv_scalar<<<1, 64, 0, s>>>(0, part, G, W, coupled, reg, 1.0, TV_BETA, 1e-8, sv));
        MSOT_LAUNCH_CHECK();
        for (int k = 0; k < sparsa_iter; ++k) {
            if ((r = apply_transpose(pl, rs, atr, W, s))) return r;
            KLAUNCH(k_tv_z<<<grid, TV_RED, 0, s>>>(x, atr, ri, sv, coupled, z, P, sl, sb));
            if ((r = tv_prox(z, sv, 0.0, coupled, xn, work, W, N, s, pl.tune_tv_cluster)))
                return r;
            KLAUNCH(k_tv_step<<<grid, TV_RED, 0, s>>>(x, xn, ri, dx, sv, coupled, N, sb, W, part));
            MSOT_LAUNCH_CHECK();
            if ((r = apply_forward(pl, dx, As, W, s))) return r;
            KLAUNCH(k_tv_rs<<<grid, TV_RED, 0, s>>>(rs, As, ns, sl, W, part));
            KLAUNCH(k_tv_scalar<<<1, 64, 0, s>>>(1, part, G, W, coupled, reg, 1.0, TV_BETA, 1e-8,
                                                 sv));
            MSOT_LAUNCH_CHECK();
        }
        KLAUNCH(k_tv_outer<<<go, 256, 0, s>>>(x, wv, vm, NI));
        MSOT_LAUNCH_CHECK();
        return MSOT_OK;
    };
    TvStream ps;  // private capturable stream, ordered after the caller's work
    if ((rc = ps.open(st))) return rc;
    const cudaStream_t cs = ps.s;
    if (d_x0)
        MSOT_CUDA_TRY(cudaMemcpyAsync(wv, d_x0, NI * sizeof(float), cudaMemcpyDeviceToDevice, cs));
    else
        MSOT_CUDA_TRY(cudaMemsetAsync(wv, 0, NI * sizeof(float), cs));
    MSOT_CUDA_TRY(cudaMemsetAsync(vm, 0, NI * sizeof(float), cs));
    int outer = 0;
    if (num_iter > 0) {
        TV_CK(outer_step(cs));
        ++outer;
    }
    if (num_iter > 1 && !profiling_enabled()) {
        cudaGraph_t g = nullptr;
        MSOT_CUDA_TRY(cudaStreamBeginCapture(cs, cudaStreamCaptureModeRelaxed));
        const long before = g_launch_count.load();
        rc = outer_step(cs);
        const long captured = g_launch_count.load() - before;
        g_launch_count -= captured;  // counted per replay below
        cudaError_t ce = cudaStreamEndCapture(cs, &g);
        if (rc == MSOT_OK && ce != cudaSuccess) {
            set_error("rec_nn_with_TV_reg: graph capture failed: %s", cudaGetErrorString(ce));
            rc = MSOT_ECUDA;
        }
        cudaGraphExec_t ge = nullptr;
        if (rc == MSOT_OK) {
            ce = cudaGraphInstantiate(&ge, g, 0);
            if (ce != cudaSuccess) {
                set_error("rec_nn_with_TV_reg: graph instantiation failed: %s",
                          cudaGetErrorString(ce));
                rc = MSOT_ECUDA;
            }
        }
        if (g) cudaGraphDestroy(g);
        for (; rc == MSOT_OK && outer < num_iter; ++outer) {
            ce = cudaGraphLaunch(ge, cs);
            if (ce != cudaSuccess) {
                set_error("rec_nn_with_TV_reg: graph launch failed: %s", cudaGetErrorString(ce));
                rc = MSOT_ECUDA;
            }
            g_launch_count += captured;
        }
        if (ge) cudaGraphExecDestroy(ge);
        if (rc) return rc;
    }
    for (; outer < num_iter; ++outer) TV_CK(outer_step(cs));
    MSOT_CUDA_TRY(cudaMemcpyAsync(d_rec, wv, NI * sizeof(float), cudaMemcpyDeviceToDevice, cs));
    if (err_img || err_reg) {
        std::vector<double> h;
        if (err_img) {
            TV_CK(apply_forward(pl, wv, As, W, cs));
            TV_CK(tv_sums(As, d_b, ns, 0, W, part, dout, h, cs));
            for (int w = 0; w < W; ++w) err_img[w] = h[w];
        }
        if (err_reg) {
            TV_CK(tv_sums(wv, nullptr, P, N, W, part, dout, h, cs));
            for (int w = 0; w < W; ++w) err_reg[w] = h[w];
        }
    }
    MSOT_CUDA_TRY(cudaStreamSynchronize(cs));
#undef TV_CK
    return MSOT_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Autotuner: times the variants of the plan's hot kernels on its own geometry
// and batch and keeps the fastest in the plan (Plan::tune_*).
// ---------------------------------------------------------------------------
namespace msot {

// deterministic pseudo-random fill in [0, 1) (integer hash of the index)
__global__ void k_tune_fill(float *a, size_t n, uint32_t seed) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        uint32_t h = (uint32_t)i * 2654435761u ^ seed;
        h ^= h >> 16;
        h *= 2246822519u;
        h ^= h >> 13;
        a[i] = (float)(h >> 8) * (1.0f / 16777216.0f);
    }
}

// mean time of `reps` runs of fn after one warm-up, CUDA events on st
template <class F>
static int tune_time(cudaStream_t st, int reps, double &ms, F fn) {
    int rc = fn();
    if (rc) return rc;
    cudaEvent_t a, b;
    MSOT_CUDA_TRY(cudaEventCreate(&a));
    MSOT_CUDA_TRY(cudaEventCreate(&b));
    cudaEventRecord(a, st);
    for (int r = 0; r < reps && rc == MSOT_OK; ++r) rc = fn();
    cudaEventRecord(b, st);
    const cudaError_t e = cudaEventSynchronize(b);
    float t = 0.f;
    cudaEventElapsedTime(&t, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (rc) return rc;
    if (e != cudaSuccess) {
        set_error("autotune: %s", cudaGetErrorString(e));
        return MSOT_ECUDA;
    }
    ms = t / reps;
    return MSOT_OK;
}

}  // namespace msot

extern "C" int msot_autotune(msot_plan_t plan, int batch, void *stream, msot_tuning *out) {
    if (!plan || batch <= 0 || batch > plan->p.max_batch) {
        set_error("autotune: bad arguments (batch 1 .. max_batch)");
        return MSOT_EINVAL;
    }
    Plan &pl = plan->p;
    if (int rc = check_plan_device(pl, "autotune")) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const size_t NI = (size_t)batch * pl.P, NS = (size_t)batch * pl.D * pl.T;
    const bool tv_ok = pl.nx == pl.nz;
    DevBufs b;
    float *img = b.get<float>(NI), *img2 = b.get<float>(NI), *sino = b.get<float>(NS);
    float *work = tv_ok ? b.get<float>((size_t)batch * TV_NVEC * pl.P) : nullptr;
    if (!b.ok) {
        set_error("autotune: device allocation failed");
        return MSOT_ENOMEM;
    }
    KLAUNCH(k_tune_fill<<<1024, 256, 0, st>>>(img, NI, 12345u));
    KLAUNCH(k_tune_fill<<<1024, 256, 0, st>>>(sino, NS, 777u));
    MSOT_LAUNCH_CHECK();
    int rc;
    msot_tuning res{};
    // DAS forward: kernel (1 staged, 2 per-detector buckets on the CSR table,
    // 4 the same on the interleaved table) and instances per CTA
    // (apply_forward: prefilter, forward, conv)
    {
        double best = 1e30;
        int pick = 0, pick_kernel = 0;
        for (int kernel : {1, 2, 4}) {
            if (kernel == 1 && !pl.st_tt) continue;
            if (kernel == 4 && !pl.fwd_ell_off) continue;
            for (int wt : {16, 8, 4, 2}) {
                if (batch % wt) continue;
                if (kernel == 1 && !fwd_staged_fits(pl, wt)) continue;
                pl.tune_fwd_wt = wt;
                pl.tune_fwd_staged = kernel;
                double ms;
                if ((rc = tune_time(st, 3, ms,
                                    [&] { return apply_forward(pl, img, sino, batch, st); })))
                    return rc;
                if (ms < best) best = ms, pick = wt, pick_kernel = kernel;
            }
        }
        pl.tune_fwd_wt = pick;
        pl.tune_fwd_staged = pick_kernel;
        res.fwd_wt = pick;
        res.fwd_staged = pick_kernel;
        res.fwd_ms = pick ? best : 0.0;
    }
    // DAS adjoint: instances per CTA (apply_transpose)
    {
        double best = 1e30;
        int pick = 0;
        for (int wt : {4, 2, 1}) {
            if (batch % wt) continue;
            pl.tune_adj_wt = wt;
            double ms;
            if ((rc = tune_time(st, 3, ms,
                                [&] { return apply_transpose(pl, sino, img2, batch, st); })))
                return rc;
            if (ms < best) best = ms, pick = wt;
        }
        pl.tune_adj_wt = pick;
        res.adj_wt = pick;
    }
    // IR convolution register cap (apply_transpose: conv, adjoint, prefilter)
    {
        double best = 1e30;
        int pick = 3;
        for (int mb : {1, 3, 4}) {
            pl.tune_conv_mb = mb;
            double ms;
            if ((rc = tune_time(st, 3, ms,
                                [&] { return apply_transpose(pl, sino, img2, batch, st); })))
                return rc;
            if (ms < best) best = ms, pick = mb;
        }
        pl.tune_conv_mb = pick;
        res.conv_min_blocks = pick;
        res.transpose_ms = best;
    }
    // SB_ITV2 cluster size (square grids): the automatic choice, every forced
    // size whose vectors fit in shared memory, and (-1) the 16-CTA cluster on
    // the global-memory workspace, which holds more images at once than
    // 16-CTA clusters of one CTA per SM (a cluster stays inside one GPC)
    res.tv_cluster = 0;
    if (tv_ok) {
        double best = 1e30;
        int pick = 0;
        for (int C : {0, 1, 2, 4, 8, 16, -1}) {
            if (C > 0 && !tvc_geometry(pl.nx, C).C) continue;
            if (C < 0 && pl.nx % 4 != 0) continue;
            double ms;
            if ((rc = tune_time(st, 2, ms, [&] {
                     return tv_prox(img, nullptr, 0.05, 1, img2, work, batch, pl.nx, st, C);
                 })))
                return rc;
            if (ms < best) best = ms, pick = C;
        }
        pl.tune_tv_cluster = pick;
        res.tv_cluster = pick;
        res.tv_prox_ms = best;
    }
    // the solvers' captured graphs hold the old kernels
    solver_cache_invalidate(pl);
    if (out) *out = res;
    MSOT_CUDA_TRY(cudaStreamSynchronize(st));
    return MSOT_OK;
}
