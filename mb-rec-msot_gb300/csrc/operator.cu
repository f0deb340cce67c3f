// operator.cu -- sm_103a kernels of the model-based operator A and A^T.
//
//   k_prefilter2d  the prefilter of Discretization.m:54-72 in one pass: the
//                  2-D filter conj(phi_hat/|phi_hat|^2) of shift_inv_proj.m:67-71
//                  factors into one circular filter per axis for the Gaussian
//                  pixel model; both axes from a shared-memory tile.
//                  k_prefilter (one axis per launch) serves single-axis plans
//                  and the SIR path's pixel order.
//   k_to_pixmajor / k_permute  instance-major image -> the pixel-major (and,
//                  with SIR, tile-permuted) order the interpolation gathers.
//   k_das_fwd3     (das_fwd.cuh, launched from here) forwardDelayAndSumMex.cpp:
//                  72-103 restated exactly by the bucket decomposition of the
//                  tri taps: per (time tile, detector, instances) CTA, bucket
//                  moments over the pixels whose travel time falls in each
//                  sample, then the 2F+2-tap filter over the moments; no
//                  atomics.
//   k_das_adj4 + k_sum_parts  transposeDelayAndSumMex.cpp:67-97: per 64x64
//                  pixel block and detector group, the block's sinogram span
//                  filtered once into bucket tables in shared memory; groups'
//                  partial images summed in fixed order.
//   k_sir_fwd     forwardMex.cpp:118-160 (SIR column convolved with the tri
//                 taps, samples outside [0, T) dropped).
//   k_sir_adj     transposeMex.cpp:115-158 (its exact adjoint).
//   k_conv_fft1k  convolve_with_IR / transpose_convolve_with_IR
//                 (MSOTmodel.m:259-269) by overlap-save with 1024-point FFTs,
//                 two real columns per complex transform, split-complex
//                 packed FP32x2 butterflies; with EPI set it also
//                 writes the L2 solver's LSQR sinogram update (IRs up to 513
//                 taps).  k_conv_fft (4096 points) takes IRs of 514-2049
//                 taps, the direct FIR k_conv longer ones.
//
// Fixed-point travel times: tau_fx = tau * 2^fb (int32).  The taps of a
// (pixel, detector) pair are t in [ceil((tau_fx - r_fx)/2^fb),
// floor((tau_fx + r_fx)/2^fb)] and the weight is 1 - |t - tau| / r, computed
// from the exact integer difference (t << fb) - tau_fx.
#include <algorithm>
#include <mutex>

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "common.cuh"

namespace msot {

// the interpolation input in [W/wt][P][wt] order: FP32 (fmt 0), BF16
// rounded to nearest (1), or FP16 of v times the instance's power-of-two
// scale hsc[w] (2) -- the reduced-storage paths of msot_plan_set_storage
__device__ __forceinline__ void store_interp_input(float *out, size_t i, float v, int fmt,
                                                   const float *hsc, int w) {
    if (fmt == 1)
        reinterpret_cast<__nv_bfloat16 *>(out)[i] = __float2bfloat16_rn(v);
    else if (fmt == 2)
        reinterpret_cast<__half *>(out)[i] = __float2half_rn(v * __ldg(hsc + w));
    else
        out[i] = v;
}

// FP16 storage: the power-of-two scale of each instance, s = 2^(14 - e) with
// gain * max |in| < 2^e, so that every stored value stays below 2^14 (FP16
// holds 65504) and keeps 11 significant bits down to 2^-24 of that; writes
// s to hsc[w] and 1 / s to hsc[stride + w].  One CTA per instance.
__global__ void __launch_bounds__(256) k_h16_scale(const float *__restrict__ in, int P,
                                                   float gain, float *__restrict__ hsc,
                                                   int stride) {
    __shared__ float red[8];
    const float *x = in + (size_t)blockIdx.x * P;
    float m = 0.f;
    for (int i = threadIdx.x; i < P; i += 256) m = fmaxf(m, fabsf(__ldg(x + i)));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < 8; ++k) m = fmaxf(m, red[k]);
        const float g = m * gain;
        int e = 0;
        if (g > 0.f && isfinite(g)) frexpf(g, &e);
        e = max(-100, min(100, e));
        hsc[blockIdx.x] = ldexpf(1.f, 14 - e);
        hsc[stride + blockIdx.x] = ldexpf(1.f, e - 14);
    }
}

__device__ __forceinline__ int tap_lo(int32_t tau, int32_t r_fx, int fb) {
    return -((r_fx - tau) >> fb);
}
__device__ __forceinline__ int tap_hi(int32_t tau, int32_t r_fx, int fb) {
    return (tau + r_fx) >> fb;
}
__device__ __forceinline__ float tri_weight(int t, int32_t tau, int fb, float c1) {
    const float df = (float)((t << fb) - tau);
    return fmaxf(0.f, fmaf(-fabsf(df), c1, 1.f));
}

// ---------------------------------------------------------------------------
// Prefilter: out = scale * sum_k h[k] in[w][pix - k (circular)] along one
// axis.  Output layout: out_mode 0 = [W][P]; 1 = [W][P] with pixel perm[j] at
// position j (scatter order); 2 = [W/wt][P][wt] (pixel-major per instance tile).
// ---------------------------------------------------------------------------
__global__ void k_prefilter(const float *__restrict__ in, float *__restrict__ out,
                            const float *__restrict__ taps, int K, int nx, int nz, int W,
                            int along_x, int transpose, float scale,
                            const int32_t *__restrict__ perm, int out_mode, int wt, int fmt,
                            const float *__restrict__ hsc) {
    const int P = nx * nz;
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long)W * P) return;
    const int w = (int)(idx / P), j = (int)(idx % P);
    const int pix = out_mode == 1 ? __ldg(perm + j) : j;
    const int ix = pix / nz, iz = pix - ix * nz;
    const float *src = in + (size_t)w * P;
    float acc = 0.f;
    for (int k = -K; k <= K; ++k) {
        const float h = __ldg(taps + (transpose ? K - k : K + k));
        int s;
        if (along_x) {
            int a = ix - k;
            a += (a < 0) ? nx : 0;
            a -= (a >= nx) ? nx : 0;
            s = a * nz + iz;
        } else {
            int a = iz - k;
            a += (a < 0) ? nz : 0;
            a -= (a >= nz) ? nz : 0;
            s = ix * nz + a;
        }
        acc = fmaf(h, __ldg(src + s), acc);
    }
    if (out_mode == 2)
        store_interp_input(out, ((size_t)(w / wt) * P + j) * wt + w % wt, acc * scale, fmt, hsc,
                           w);
    else
        out[(size_t)w * P + j] = acc * scale;
}

// ---------------------------------------------------------------------------
// Both prefilter axes in one pass through shared memory.  CTA = (tile of TX
// columns ix, instance w); it stages the columns ix0 - KM .. ix0 + TX + KM - 1
// (circular) of the image, filters every staged column along z into a second
// buffer, then filters along x into the TX output columns.  Each thread
// slides a register window over 8 consecutive outputs, so a tap costs one
// FMA and (8 + 2 KM) / 8 / (2 KM + 1) shared loads.  Taps are zero-padded to
// the compile-time half width KM >= K.  out_mode 0 = [W][P], 2 = [W/wt][P][wt].
// ---------------------------------------------------------------------------
constexpr int PF_TX = 32, PF_R = 8, PF_THREADS = 256;

__device__ __forceinline__ int wrap_mod(int a, int n) {
    a %= n;
    return a < 0 ? a + n : a;
}

template <int KM>
__global__ void __launch_bounds__(PF_THREADS) k_prefilter2d(
    const float *__restrict__ in, float *__restrict__ out, const float *__restrict__ taps_x,
    const float *__restrict__ taps_z, int Kx, int Kz, int nx, int nz, int W, int transpose,
    int out_mode, int wt, int fmt, const float *__restrict__ hsc) {
    constexpr int NC = PF_TX + 2 * KM;  // staged columns
    constexpr int NTAP = 2 * KM + 1;
    constexpr int NW = PF_THREADS / 32;
    extern __shared__ float pf_smem[];
    const int ld = nz | 1;         // odd column stride: lanes over columns hit distinct banks
    float *A = pf_smem;            // [NC][ld] staged input
    float *B = A + NC * ld;        // [NC][ld] z-filtered
    float *hz = B + NC * ld;       // [NTAP] tap for offset k at hz[k + KM]
    float *hx = hz + NTAP;
    const int w = blockIdx.y, ix0 = blockIdx.x * PF_TX;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const float *src = in + (size_t)w * nx * nz;
    for (int k = threadIdx.x; k < NTAP; k += PF_THREADS) {
        const int o = k - KM;
        hz[k] = (o >= -Kz && o <= Kz) ? taps_z[transpose ? Kz - o : Kz + o] : 0.f;
        hx[k] = (o >= -Kx && o <= Kx) ? taps_x[transpose ? Kx - o : Kx + o] : 0.f;
    }
    // stage: one warp per column, lanes along z
    for (int c = warp; c < NC; c += NW) {
        const float *scol = src + (size_t)wrap_mod(ix0 - KM + c, nx) * nz;
        float *dcol = A + c * ld;
        for (int z = lane; z < nz; z += 32) dcol[z] = __ldg(scol + z);
    }
    __syncthreads();
    // z pass, lanes over columns: B[c][z] = sum_k hz[k] A[c][z - k (circular)]
    const int nzc = (nz + PF_R - 1) / PF_R;
    constexpr int NCG = (NC + 31) / 32;
    for (int it = warp; it < NCG * nzc; it += NW) {
        const int cg = it / nzc, z0 = (it - cg * nzc) * PF_R;
        const int c = cg * 32 + lane;
        if (c < NC) {
            const float *col = A + c * ld;
            float win[PF_R + 2 * KM];
#pragma unroll
            for (int i = 0; i < PF_R + 2 * KM; ++i) {
                int z = z0 - KM + i;
                z = (z >= 0 && z < nz) ? z : wrap_mod(z, nz);
                win[i] = col[z];
            }
            float acc[PF_R];
#pragma unroll
            for (int j = 0; j < PF_R; ++j) acc[j] = 0.f;
#pragma unroll
            for (int k = -KM; k <= KM; ++k) {
                const float h = hz[k + KM];
#pragma unroll
                for (int j = 0; j < PF_R; ++j) acc[j] = fmaf(h, win[j - k + KM], acc[j]);
            }
#pragma unroll
            for (int j = 0; j < PF_R; ++j)
                if (z0 + j < nz) B[c * ld + z0 + j] = acc[j];
        }
    }
    __syncthreads();
    // x pass, lanes along z: out[ix0 + c][z] = sum_k hx[k] B[c + KM - k][z]
    constexpr int NXC = PF_TX / PF_R;
    for (int it = threadIdx.x; it < NXC * nz; it += PF_THREADS) {
        const int cc = it / nz, z = it - cc * nz, c0 = cc * PF_R;
        float win[PF_R + 2 * KM];
#pragma unroll
        for (int i = 0; i < PF_R + 2 * KM; ++i) win[i] = B[(c0 + i) * ld + z];
        float acc[PF_R];
#pragma unroll
        for (int j = 0; j < PF_R; ++j) acc[j] = 0.f;
#pragma unroll
        for (int k = -KM; k <= KM; ++k) {
            const float h = hx[k + KM];
#pragma unroll
            for (int j = 0; j < PF_R; ++j) acc[j] = fmaf(h, win[j - k + KM], acc[j]);
        }
#pragma unroll
        for (int j = 0; j < PF_R; ++j) {
            const int ix = ix0 + c0 + j;
            if (ix >= nx) break;
            const size_t p = (size_t)ix * nz + z;
            if (out_mode == 2)
                store_interp_input(out, ((size_t)(w / wt) * nx * nz + p) * wt + w % wt, acc[j],
                                   fmt, hsc, w);
            else
                out[(size_t)w * nx * nz + p] = acc[j];
        }
    }
}

// [W][P] -> [W/wt][P][wt] (pixel-major within each tile of wt instances)
__global__ void k_to_pixmajor(const float *__restrict__ in, float *__restrict__ out, int P,
                              int W, int wt, int fmt, const float *__restrict__ hsc) {
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long)W * P) return;
    const int w = (int)(idx / P), j = (int)(idx % P);
    store_interp_input(out, ((size_t)(w / wt) * P + j) * wt + w % wt, __ldg(in + idx), fmt, hsc,
                       w);
}

// [W][P] -> [W][P] in scatter order (out[w][j] = in[w][perm[j]])
__global__ void k_permute(const float *__restrict__ in, float *__restrict__ out,
                          const int32_t *__restrict__ perm, int P, int W) {
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long)W * P) return;
    const int w = (int)(idx / P), j = (int)(idx % P);
    out[idx] = __ldg(in + (size_t)w * P + __ldg(perm + j));
}

// ---------------------------------------------------------------------------
// Bucket decomposition of the tri interpolation (no SIR).
// For tau = b + f, taps t = b + k, k in [-(F-1), F], have weight
// alpha_k + beta_k f with alpha_k = 1 - |k|/r, beta_k = -1/r (k <= 0) or
// +1/r (k >= 1); tap b - F has weight e1(f) = max(0, (r - F - f)/r) and tap
// b + F + 1 has e2(f) = max(0, (f - (F + 1 - r))/r); no other tap is non-zero.
// This is exactly the reference's tap set ceil(tau - r) .. floor(tau + r).
//
// Forward: per detector the pixels are bucketed by b = floor(tau); each
// bucket reduces four moments sum x, sum f x, sum e1 x, sum e2 x over its
// pixels, and the output is a (2F+2)-tap filter over the moments.
// Adjoint: the sinogram is filtered once per bucket into
// Q_b = (U_b, V_b, s[b-F], s[b+F+1]), U_b = sum alpha_k s[b+k],
// V_b = sum beta_k s[b+k]; each (pixel, detector) then adds
// U + f V + e1 s[b-F] + e2 s[b+F+1].
// ---------------------------------------------------------------------------

// Adjoint by pixel blocks: CTA = (64x64 pixel block, instance tile of WT,
// detector group).  For each detector of its group the CTA stages the
// sinogram samples spanned by the block (plus F+1 on each side) in shared
// memory and builds a bucket table there (each thread filters ADJ_BPT
// consecutive buckets from a register window).  A pixel of bucket b with
// fraction f receives v(f) = U + f V + e1(f) s[b-F] + e2(f) s[b+F+1]
// (U = sum alpha_k s[b+k], V = sum beta_k s[b+k]); as e1 and e2 are linear
// in f on either side of their kinks at f = r - F and f = F + 1 - r, v is
// linear on the three pieces between p1 = min(r - F, F + 1 - r) and
// p2 = max(...), and the table holds (A, B) with v = A + f B per (bucket,
// piece): one 8-byte load and one FMA per (pixel, detector, instance).
// Groups write partial images; k_sum_parts adds them in fixed order.
constexpr int ADJ_BPT = 4;  // buckets per thread when building Q
std::atomic<int> g_adj_prefetch{1};  // next-detector prefetch in k_das_adj4 (msot_tune_set)

// PF > 0: the segment of the next detector is loaded into registers (PF
// samples per instance per thread; needs SL <= PF * BLK_THREADS) while the
// current one is filtered and gathered.
template <int WT, int F, int PF = 0>
__global__ void __launch_bounds__(BLK_THREADS, WT >= 4 ? 2 : 3) k_das_adj4(
    const int32_t *__restrict__ btau, const int2 *__restrict__ bspan,
    const float *__restrict__ s, float *__restrict__ part, int nx, int nz, int nbx, int D,
    int T, int fb, float inv_r, float ce1, float ce2, float p1, float p2, int span_max,
    int det_per_group, size_t part_stride) {
    extern __shared__ float sm[];
    const int SL = ((span_max + ADJ_BPT - 1) / ADJ_BPT) * ADJ_BPT + 2 * F + 2;
    float *seg = sm;  // [WT][SL]
    // [3][span_max][WT]: a bucket's (A, B) pairs of the CTA's instances side
    // by side, so that one 128-bit load gathers two instances
    float2 *Q = reinterpret_cast<float2 *>(sm + ((WT * SL + 3) & ~3));
    const int blk = blockIdx.x, w0 = blockIdx.y * WT, grp = blockIdx.z;
    const int t = threadIdx.x;
    const int bxi = blk % nbx, bzi = blk / nbx;
    const int mask = (1 << fb) - 1;
    const float step = __int_as_float((127 - fb) << 23);
    float acc[BLK_PPT][WT];
#pragma unroll
    for (int k = 0; k < BLK_PPT; ++k)
#pragma unroll
        for (int i = 0; i < WT; ++i) acc[k][i] = 0.f;
    const int d_begin = grp * det_per_group, d_end = min(D, d_begin + det_per_group);
    float pre[PF > 0 ? WT : 1][PF > 0 ? PF : 1];
    auto fetch = [&](int d) {
        const int2 sq = __ldg(bspan + (size_t)blk * D + d);
        const int nq = sq.y - sq.x + 1;
        const int Lq = nq > 0 ? ((nq + ADJ_BPT - 1) / ADJ_BPT) * ADJ_BPT + 2 * F + 2 : 0;
#pragma unroll
        for (int w = 0; w < WT; ++w) {
            const float *src = s + ((size_t)(w0 + w) * D + d) * T;
#pragma unroll
            for (int j = 0; j < PF; ++j) {
                const int k = t + j * BLK_THREADS, tt = sq.x - F + k;
                pre[w][j] = (k < Lq && tt >= 0 && tt < T) ? __ldg(src + tt) : 0.f;
            }
        }
    };
    if constexpr (PF > 0)
        if (d_begin < d_end) fetch(d_begin);
    for (int d = d_begin; d < d_end; ++d) {
        const int2 sp = __ldg(bspan + (size_t)blk * D + d);
        const int nb = sp.y - sp.x + 1;
        if (nb <= 0) {  // block outside the grid: uniform across the CTA
            if constexpr (PF > 0)
                if (d + 1 < d_end) fetch(d + 1);
            continue;
        }
        const int L = ((nb + ADJ_BPT - 1) / ADJ_BPT) * ADJ_BPT + 2 * F + 2;
        if constexpr (PF > 0) {
#pragma unroll
            for (int w = 0; w < WT; ++w)
#pragma unroll
                for (int j = 0; j < PF; ++j) {
                    const int k = t + j * BLK_THREADS;
                    if (k < L) seg[w * SL + k] = pre[w][j];
                }
        } else {
            for (int w = 0; w < WT; ++w) {
                const float *src = s + ((size_t)(w0 + w) * D + d) * T;
                for (int k = t; k < L; k += BLK_THREADS) {
                    const int tt = sp.x - F + k;
                    seg[w * SL + k] = (tt >= 0 && tt < T) ? __ldg(src + tt) : 0.f;
                }
            }
        }
        __syncthreads();
        if constexpr (PF > 0)
            if (d + 1 < d_end) fetch(d + 1);  // in flight during the filter and the gather
        // one bucket per thread: consecutive threads read consecutive samples
        for (int i = t; i < WT * nb; i += BLK_THREADS) {
            const int w = i / nb, bl = i - w * nb;
            const float *g = seg + w * SL + bl + F;  // g[k] = s[b + k]
            float U = 0.f, V = 0.f;
#pragma unroll
            for (int k = -(F - 1); k <= F; ++k) {
                U = fmaf(1.f - (float)(k < 0 ? -k : k) * inv_r, g[k], U);
                V += k <= 0 ? -g[k] : g[k];
            }
            // pieces f < p1, p1 <= f < p2, f >= p2: e1 = ce1 - f / r below
            // r - F, e2 = f / r - ce2 above F + 1 - r
            const float Vr = V * inv_r, sL = g[-F], sH = g[F + 1];
            const float A0 = fmaf(ce1, sL, U), B0 = fmaf(-inv_r, sL, Vr);
            const float A2 = fmaf(-ce2, sH, U), B2 = fmaf(inv_r, sH, Vr);
            const bool lo_first = ce1 <= ce2;  // r - F <= F + 1 - r: e1 ends before e2 starts
            const float A1 = lo_first ? U : fmaf(-ce2, sH, A0);
            const float B1 = lo_first ? Vr : fmaf(inv_r, sH, B0);
            float2 *q = Q + (size_t)bl * WT + w;
            q[0] = make_float2(A0, B0);
            q[(size_t)span_max * WT] = make_float2(A1, B1);
            q[(size_t)2 * span_max * WT] = make_float2(A2, B2);
        }
        __syncthreads();
        const int32_t *tp = btau + ((size_t)blk * D + d) * BLK + t;
#pragma unroll
        for (int k = 0; k < BLK_PPT; ++k) {
            const int32_t tau = __ldg(tp + k * BLK_THREADS);
            if (tau == TAU_PAD) continue;
            const float f = (float)(tau & mask) * step;
            const int bp = (tau >> fb) - sp.x + ((f >= p1) + (f >= p2)) * span_max;
            const float2 *qv = Q + (size_t)bp * WT;
            if constexpr (WT % 2 == 0) {
#pragma unroll
                for (int i = 0; i < WT; i += 2) {
                    const float4 v = *reinterpret_cast<const float4 *>(qv + i);
                    acc[k][i] = fmaf(f, v.y, acc[k][i] + v.x);
                    acc[k][i + 1] = fmaf(f, v.w, acc[k][i + 1] + v.z);
                }
            } else {
#pragma unroll
                for (int i = 0; i < WT; ++i) {
                    const float2 v = qv[i];
                    acc[k][i] = fmaf(f, v.y, acc[k][i] + v.x);
                }
            }
        }
        __syncthreads();
    }
    const size_t P = (size_t)nx * nz;
    float *dst = part + (size_t)grp * part_stride;
    const int iz = bzi * BLK_Z + t % BLK_Z;
#pragma unroll
    for (int k = 0; k < BLK_PPT; ++k) {
        const int ix = bxi * BLK_X + t / BLK_Z + (BLK_THREADS / BLK_Z) * k;
        if (ix >= nx || iz >= nz) continue;
#pragma unroll
        for (int i = 0; i < WT; ++i) dst[(size_t)(w0 + i) * P + (size_t)ix * nz + iz] = acc[k][i];
    }
}

// x[w][p] = scale * sum_g part[g][w][p]   (groups added in order)
__global__ void k_sum_parts(const float *__restrict__ part, float *__restrict__ x, size_t n,
                            int groups, size_t stride, float scale) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        float v = 0.f;
        for (int g = 0; g < groups; ++g) v += __ldg(part + g * stride + i);
        x[i] = v * scale;
    }
}

// ---------------------------------------------------------------------------
// SIR forward: CTA = (detector, pixel slice, WT instances) with the
// detector's output column [WT][T] in shared memory; each (pixel, detector)
// pair deposits the SIR column convolved with its NT tri taps,
// e[m] = sum_i f[i] h[m - i], at output sample tb + m - S/2 by shared-memory
// atomics, dropped outside [0, T) (forwardMex.cpp:139).
// ---------------------------------------------------------------------------
template <int WT, int NT>
__global__ void __launch_bounds__(256) k_sir_fwd(const int32_t *__restrict__ tau_pi,
                                                 const int32_t *__restrict__ sir_pi,
                                                 const float *__restrict__ sir,
                                                 const int2 *__restrict__ sir_se,
                                                 const float *__restrict__ x_pi,
                                                 float *__restrict__ raw, int P, int D, int T,
                                                 int S, int fb, int32_t r_fx, float c1,
                                                 float scale, int nsplit) {
    extern __shared__ float col[];  // [WT][T]
    const int d = blockIdx.x, sp = blockIdx.y, w0 = blockIdx.z * WT;
    for (int i = threadIdx.x; i < WT * T; i += blockDim.x) col[i] = 0.f;
    __syncthreads();
    const int half = S / 2;
    const int j0 = (int)((long)P * sp / nsplit), j1 = (int)((long)P * (sp + 1) / nsplit);
    for (int j = j0 + threadIdx.x; j < j1; j += blockDim.x) {
        const size_t o = (size_t)d * P + j;
        const int32_t tau = __ldg(tau_pi + o);
        const int s = __ldg(sir_pi + o);
        float xv[WT];
#pragma unroll
        for (int i = 0; i < WT; ++i) xv[i] = __ldg(x_pi + (size_t)(w0 + i) * P + j);
        const int tb = tap_lo(tau, r_fx, fb);
        float f[NT];
#pragma unroll
        for (int i = 0; i < NT; ++i) f[i] = tri_weight(tb + i, tau, fb, c1);
        const int2 se = __ldg(sir_se + s);
        const float *h = sir + (size_t)s * S;
        float acc[NT];
#pragma unroll
        for (int i = 0; i < NT; ++i) acc[i] = 0.f;
        const int jb = tb - half;
        for (int k = se.x; k <= se.y; ++k) {
            const float hk = __ldg(h + k);
#pragma unroll
            for (int i = 0; i < NT; ++i) acc[i] = fmaf(f[i], hk, acc[i]);
            const int J = jb + k;
            if (J >= 0 && J < T) {
#pragma unroll
                for (int i = 0; i < WT; ++i) atomicAdd(&col[i * T + J], acc[0] * xv[i]);
            }
#pragma unroll
            for (int i = 0; i < NT - 1; ++i) acc[i] = acc[i + 1];
            acc[NT - 1] = 0.f;
        }
#pragma unroll
        for (int m = 0; m < NT - 1; ++m) {
            const int J = jb + se.y + 1 + m;
            if (J >= 0 && J < T && acc[m] != 0.f) {
#pragma unroll
                for (int i = 0; i < WT; ++i) atomicAdd(&col[i * T + J], acc[m] * xv[i]);
            }
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < WT * T; i += blockDim.x) {
        const int wi = i / T, t = i - wi * T;
        float *dst = raw + ((size_t)(w0 + wi) * D + d) * T + t;
        const float v = col[i] * scale;
        if (nsplit == 1)
            *dst = v;
        else
            atomicAdd(dst, v);
    }
}

// ---------------------------------------------------------------------------
// SIR adjoint: per (pixel, detector) v_k = sum_i f[i] y[tb + i + k - S/2] for
// k in the SIR column's [start, end], x += sum_k h[k] v_k; y outside [0, T)
// counts as zero (transposeMex.cpp:136).
// ---------------------------------------------------------------------------
template <int WT, int NT>
__global__ void __launch_bounds__(256) k_sir_adj(const int32_t *__restrict__ tiles,
                                                 const int32_t *__restrict__ sir_tiles,
                                                 const float *__restrict__ sir,
                                                 const int2 *__restrict__ sir_se,
                                                 const float *__restrict__ raw,
                                                 float *__restrict__ out, int nx, int nz,
                                                 int npx, int D, int T, int S, int fb,
                                                 int32_t r_fx, float c1, float scale) {
    __shared__ float red[4][PATCH][WT];
    const int patch = blockIdx.x, w0 = blockIdx.y * WT;
    const int q = threadIdx.x & (PATCH - 1), g = threadIdx.x / PATCH;
    const int px = patch % npx, pz = patch / npx;
    const int ix = px * PATCH_X + q / PATCH_Z, iz = pz * PATCH_Z + q % PATCH_Z;
    const int half = S / 2;
    const size_t DT = (size_t)D * T;
    float acc[WT];
#pragma unroll
    for (int i = 0; i < WT; ++i) acc[i] = 0.f;
    for (int d = g; d < D; d += 4) {
        const size_t o = ((size_t)patch * D + d) * PATCH + q;
        const int32_t tau = __ldg(tiles + o);
        if (tau == TAU_PAD) continue;
        const int s = __ldg(sir_tiles + o);
        const int tb = tap_lo(tau, r_fx, fb);
        float f[NT];
#pragma unroll
        for (int i = 0; i < NT; ++i) f[i] = tri_weight(tb + i, tau, fb, c1);
        const int2 se = __ldg(sir_se + s);
        const float *h = sir + (size_t)s * S;
        const float *base = raw + ((size_t)w0 * D + d) * T;
        const int jb = tb + se.x - half;
        float win[WT][NT];
#pragma unroll
        for (int i = 0; i < NT; ++i) {
            const int J = jb + i;
            const bool ok = J >= 0 && J < T;
#pragma unroll
            for (int w = 0; w < WT; ++w) win[w][i] = ok ? __ldg(base + w * DT + J) : 0.f;
        }
        for (int k = se.x; k <= se.y; ++k) {
            const float hk = __ldg(h + k);
#pragma unroll
            for (int w = 0; w < WT; ++w) {
                float v = 0.f;
#pragma unroll
                for (int i = 0; i < NT; ++i) v = fmaf(f[i], win[w][i], v);
                acc[w] = fmaf(hk, v, acc[w]);
            }
            const int J = jb + (k - se.x) + NT;
            const bool ok = J >= 0 && J < T;
#pragma unroll
            for (int w = 0; w < WT; ++w) {
#pragma unroll
                for (int i = 0; i < NT - 1; ++i) win[w][i] = win[w][i + 1];
                win[w][NT - 1] = ok ? __ldg(base + w * DT + J) : 0.f;
            }
        }
    }
#pragma unroll
    for (int i = 0; i < WT; ++i) red[g][q][i] = acc[i];
    __syncthreads();
    if (g == 0 && ix < nx && iz < nz) {
        const size_t P = (size_t)nx * nz;
#pragma unroll
        for (int i = 0; i < WT; ++i) {
            const float s = ((red[0][q][i] + red[1][q][i]) + red[2][q][i]) + red[3][q][i];
            out[(size_t)(w0 + i) * P + (size_t)ix * nz + iz] = s * scale;
        }
    }
}

// ---------------------------------------------------------------------------
// IR convolution along t of every (instance, detector) column:
//   out[t] = sum_{k<L} taps[k] in[t + L/2 - k]   (in = 0 outside [0, T)).
// CTA = (t tile of TPT*NTH samples, column).  Each thread keeps TPT outputs
// and a sliding window of TPT inputs in registers; the shared-memory segment
// is padded (one word per 8) so the window loads are bank-conflict free.
// ---------------------------------------------------------------------------
template <int TPT, int NTH>
__global__ void __launch_bounds__(NTH) k_conv(const float *__restrict__ in,
                                              float *__restrict__ out,
                                              const float *__restrict__ taps, int L, int T) {
    constexpr int TT = TPT * NTH;
    extern __shared__ float sm[];
    const int Lp = (L + TPT - 1) / TPT * TPT;
    float *irr = sm;
    float *seg = sm + Lp;
    const int seg_len = TT + Lp + TPT;
    const size_t col = blockIdx.y;
    const int t0 = blockIdx.x * TT;
    const int base_in = t0 + L / 2 - (L - 1);
    const float *src = in + col * T;
    for (int j = threadIdx.x; j < Lp; j += NTH) irr[j] = j < L ? __ldg(taps + L - 1 - j) : 0.f;
    for (int q = threadIdx.x; q < seg_len; q += NTH) {
        const int ti = base_in + q;
        seg[q + (q >> 3)] = (ti >= 0 && ti < T) ? __ldg(src + ti) : 0.f;
    }
    __syncthreads();
    const int o0 = threadIdx.x * TPT;
    float acc[TPT], win[TPT];
#pragma unroll
    for (int i = 0; i < TPT; ++i) {
        acc[i] = 0.f;
        const int q = o0 + i;
        win[i] = seg[q + (q >> 3)];
    }
    for (int j0 = 0; j0 < Lp; j0 += TPT) {
#pragma unroll
        for (int jj = 0; jj < TPT; ++jj) {
            const float c = irr[j0 + jj];
#pragma unroll
            for (int i = 0; i < TPT; ++i) acc[i] = fmaf(c, win[(i + jj) % TPT], acc[i]);
            const int q = o0 + j0 + jj + TPT;
            win[jj] = seg[q + (q >> 3)];
        }
    }
    float *dst = out + col * T + t0 + o0;
#pragma unroll
    for (int i = 0; i < TPT; ++i)
        if (t0 + o0 + i < T) dst[i] = acc[i];
}

// ---------------------------------------------------------------------------
// IR convolution by overlap-save FFT.  Two real columns c1, c2 ride in one
// complex transform: y1 + i y2 = IFFT(FFT(x1 + i x2) H) since the taps are
// real.  CTA = (output block of V = N - L + 1 samples, column pair); N-point
// radix-4 Stockham FFTs in shared memory (N/4 threads, one butterfly each
// per stage); H already holds the 1/N of the inverse transform.
// ---------------------------------------------------------------------------
template <int SIGN>
__device__ __forceinline__ void radix4_stage(const float2 *__restrict__ A, float2 *__restrict__ B,
                                             const float2 *__restrict__ tw, int N, int L,
                                             int tw_step, int j) {
    const int k = j & (L - 1), q = j / L;
    const int Q = N >> 2;
    float2 a[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        float2 v = A[j + r * Q];
        if (r) {
            float2 w = __ldg(tw + r * k * tw_step);
            if (SIGN > 0) w.y = -w.y;
            v = make_float2(v.x * w.x - v.y * w.y, v.x * w.y + v.y * w.x);
        }
        a[r] = v;
    }
    const float2 t0 = make_float2(a[0].x + a[2].x, a[0].y + a[2].y);
    const float2 t1 = make_float2(a[0].x - a[2].x, a[0].y - a[2].y);
    const float2 t2 = make_float2(a[1].x + a[3].x, a[1].y + a[3].y);
    const float2 d = make_float2(a[1].x - a[3].x, a[1].y - a[3].y);
    // t3 = (a1 - a3) * (SIGN * i)
    const float2 t3 = SIGN < 0 ? make_float2(d.y, -d.x) : make_float2(-d.y, d.x);
    float2 *o = B + q * 4 * L + k;
    o[0] = make_float2(t0.x + t2.x, t0.y + t2.y);
    o[L] = make_float2(t1.x + t3.x, t1.y + t3.y);
    o[2 * L] = make_float2(t0.x - t2.x, t0.y - t2.y);
    o[3 * L] = make_float2(t1.x - t3.x, t1.y - t3.y);
}

// bit reversal of a 5-bit index
__host__ __device__ constexpr int brev5(int i) {
    return ((i & 1) << 4) | ((i & 2) << 2) | (i & 4) | ((i & 8) >> 2) | ((i & 16) >> 4);
}

// Split-complex 32-point FFTs on packed FP32x2 arithmetic.  A lane's 32
// complex values are held as R[m] = (re[2m], re[2m+1]), I[m] = (im[2m],
// im[2m+1]), so one packed add / multiply / fma works on two butterflies.
// Radix-2 decimation in frequency (natural order in, bit-reversed out) and
// in time (bit-reversed in, natural out); every stage but the one pairing
// neighbouring elements (half = 1) is packed.  The bit-reversed orders never
// move data: the callers index registers through brev5() at compile time.
// c_p2r / c_p2i hold the stage twiddle pairs (w32^t0, w32^t1), t = j * step
// for the pairs j, j + 1 of the stages half = 16, 8, 4, 2 (15 pairs); c_p2n
// is -c_p2i (the conjugate's imaginary part).
#define MSOT_W32P(a, b) {c_w32r[a], c_w32r[b]}
#define MSOT_W32I(a, b) {c_w32i[a], c_w32i[b]}
#define MSOT_W32N(a, b) {-c_w32i[a], -c_w32i[b]}
constexpr float c_w32r[16] = {1.000000000e+00f,  9.807852804e-01f,  9.238795325e-01f,
                              8.314696123e-01f,  7.071067812e-01f,  5.555702330e-01f,
                              3.826834324e-01f,  1.950903220e-01f,  0.000000000e+00f,
                              -1.950903220e-01f, -3.826834324e-01f, -5.555702330e-01f,
                              -7.071067812e-01f, -8.314696123e-01f, -9.238795325e-01f,
                              -9.807852804e-01f};
constexpr float c_w32i[16] = {0.000000000e+00f,  -1.950903220e-01f, -3.826834324e-01f,
                              -5.555702330e-01f, -7.071067812e-01f, -8.314696123e-01f,
                              -9.238795325e-01f, -9.807852804e-01f, -1.000000000e+00f,
                              -9.807852804e-01f, -9.238795325e-01f, -8.314696123e-01f,
                              -7.071067812e-01f, -5.555702330e-01f, -3.826834324e-01f,
                              -1.950903220e-01f};
#define MSOT_W32_PAIRS(M)                                                                  \
    M(0, 1), M(2, 3), M(4, 5), M(6, 7), M(8, 9), M(10, 11), M(12, 13), M(14, 15), M(0, 2),    \
        M(4, 6), M(8, 10), M(12, 14), M(0, 4), M(8, 12), M(0, 8)
__constant__ float2 c_p2r[15] = {MSOT_W32_PAIRS(MSOT_W32P)};
__constant__ float2 c_p2i[15] = {MSOT_W32_PAIRS(MSOT_W32I)};
__constant__ float2 c_p2n[15] = {MSOT_W32_PAIRS(MSOT_W32N)};
#undef MSOT_W32_PAIRS
#undef MSOT_W32P
#undef MSOT_W32I
#undef MSOT_W32N

// index of the twiddle pair of stage `half`, butterflies j, j + 1
__host__ __device__ constexpr int p2_index(int half, int j) {
    return (half == 16 ? 0 : half == 8 ? 8 : half == 4 ? 12 : 14) + j / 2;
}

__device__ __forceinline__ float2 f2add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 f2sub(float2 a, float2 b) {
    return __ffma2_rn(b, make_float2(-1.f, -1.f), a);
}
// (R, I) <- (R, I) * (WR, WI) for two complex values; NI = -WI
__device__ __forceinline__ void cmul2(float2 &R, float2 &I, float2 WR, float2 WI, float2 NI) {
    const float2 r = __ffma2_rn(I, NI, __fmul2_rn(R, WR));
    const float2 i = __ffma2_rn(I, WR, __fmul2_rn(R, WI));
    R = r;
    I = i;
}
// the same with a table pair q = (re a, re b, im a, im b)
__device__ __forceinline__ void cmul2q(float2 &R, float2 &I, float4 q) {
    cmul2(R, I, make_float2(q.x, q.y), make_float2(q.z, q.w), make_float2(-q.z, -q.w));
}

// SIGN = -1: forward (w32^t), +1: inverse (conjugate twiddles)
template <int SIGN>
__device__ __forceinline__ void fft32_dif2(float2 (&R)[16], float2 (&I)[16]) {
#pragma unroll
    for (int half = 16; half >= 2; half >>= 1) {
#pragma unroll
        for (int b = 0; b < 32; b += 2 * half) {
#pragma unroll
            for (int j = 0; j < half; j += 2) {
                const int a = (b + j) >> 1, c = (b + j + half) >> 1, q = p2_index(half, j);
                const float2 uR = R[a], uI = I[a], wR = R[c], wI = I[c];
                R[a] = f2add(uR, wR);
                I[a] = f2add(uI, wI);
                float2 dR = f2sub(uR, wR), dI = f2sub(uI, wI);
                if (SIGN < 0)
                    cmul2(dR, dI, c_p2r[q], c_p2i[q], c_p2n[q]);
                else
                    cmul2(dR, dI, c_p2r[q], c_p2n[q], c_p2i[q]);
                R[c] = dR;
                I[c] = dI;
            }
        }
    }
#pragma unroll
    for (int m = 0; m < 16; ++m) {  // half = 1: the two elements of a pair
        const float2 r = R[m], i = I[m];
        R[m] = make_float2(r.x + r.y, r.x - r.y);
        I[m] = make_float2(i.x + i.y, i.x - i.y);
    }
}

template <int SIGN>
__device__ __forceinline__ void fft32_dit2(float2 (&R)[16], float2 (&I)[16]) {
#pragma unroll
    for (int m = 0; m < 16; ++m) {  // half = 1
        const float2 r = R[m], i = I[m];
        R[m] = make_float2(r.x + r.y, r.x - r.y);
        I[m] = make_float2(i.x + i.y, i.x - i.y);
    }
#pragma unroll
    for (int half = 2; half <= 16; half <<= 1) {
#pragma unroll
        for (int b = 0; b < 32; b += 2 * half) {
#pragma unroll
            for (int j = 0; j < half; j += 2) {
                const int a = (b + j) >> 1, c = (b + j + half) >> 1, q = p2_index(half, j);
                float2 tR = R[c], tI = I[c];
                if (SIGN < 0)
                    cmul2(tR, tI, c_p2r[q], c_p2i[q], c_p2n[q]);
                else
                    cmul2(tR, tI, c_p2r[q], c_p2n[q], c_p2i[q]);
                const float2 uR = R[a], uI = I[a];
                R[a] = f2add(uR, tR);
                I[a] = f2add(uI, tI);
                R[c] = f2sub(uR, tR);
                I[c] = f2sub(uI, tI);
            }
        }
    }
}

// element e (0 .. 31) of a split-complex register array
__device__ __forceinline__ float &ev(float2 (&A)[16], int e) { return (e & 1) ? A[e >> 1].y : A[e >> 1].x; }

// Epilogue of the convolution for the LSQR sinogram update (EPI 1: u =
// sl*b - sl*y, EPI 2: u = sl*y - gamma*u) with per-CTA partial sums of u^2.
struct ConvEpi {
    const float *b;
    const Scal *sc;
    float sl;
    int coupled, D, nparts;
    double *part;
};

// 1024-point overlap-save convolution by the four-step FFT 1024 = 32 x 32:
// one warp per transform (two real columns as one complex sequence), the
// split-complex packed 32-point FFTs above in registers and two warp-local
// transposes through padded shared memory (re and im planes) per direction.
// EPI != 0 requires every CTA's columns to lie in one instance.  Tables, each
// [16 pairs][32 lanes] of
// (re a, re b, im a, im b): twb = w1024^(lane k1) for the register pair of
// k1 = brev5(2m), brev5(2m + 1); twn = conj w1024^(lane n) for n = 2m,
// 2m + 1; Hb = H[lane + 32 k2] for k2 = brev5(2m), brev5(2m + 1).
template <int FPC, int EPI = 0, int MINB = 1>
__global__ void __launch_bounds__(32 * FPC, MINB) k_conv_fft1k(
    const float *__restrict__ in, float *__restrict__ out, const float4 *__restrict__ twb,
    const float4 *__restrict__ twn, const float4 *__restrict__ Hb, int C, int T, int L,
    ConvEpi epi = {}) {
    __shared__ __align__(16) float SR[FPC][32][34];
    __shared__ __align__(16) float SI[FPC][32][34];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int pair = blockIdx.y * FPC + warp;
    const int c1 = 2 * pair, c2 = c1 + 1;
    if (c1 >= C) return;  // whole warp; no CTA-wide barriers below
    const bool has2 = c2 < C;
    const int V = 1024 - L + 1;
    const int t0 = blockIdx.x * V;
    const int u0 = t0 + L / 2 - (L - 1);
    const float *x1 = in + (size_t)c1 * T;
    const float *x2 = in + (size_t)(has2 ? c2 : c1) * T;
    float2 R[16], I[16];
    if (u0 >= 0 && u0 + 1023 < T) {
#pragma unroll
        for (int n1 = 0; n1 < 32; ++n1) {
            const int u = u0 + 32 * n1 + lane;
            ev(R, n1) = __ldg(x1 + u);
            ev(I, n1) = has2 ? __ldg(x2 + u) : 0.f;
        }
    } else {
#pragma unroll
        for (int n1 = 0; n1 < 32; ++n1) {
            const int u = u0 + 32 * n1 + lane;
            const bool ok = u >= 0 && u < T;
            ev(R, n1) = ok ? __ldg(x1 + u) : 0.f;
            ev(I, n1) = (ok && has2) ? __ldg(x2 + u) : 0.f;
        }
    }
    fft32_dif2<-1>(R, I);  // over n1 (this lane is n2); register e holds k1 = brev5(e)
#pragma unroll
    for (int m = 0; m < 16; ++m) cmul2q(R[m], I[m], __ldg(twb + m * 32 + lane));
    float(*Sr)[34] = SR[warp];
    float(*Si)[34] = SI[warp];
#pragma unroll
    for (int e = 0; e < 32; ++e) {
        Sr[brev5(e)][lane] = ev(R, e);
        Si[brev5(e)][lane] = ev(I, e);
    }
    __syncwarp();
#pragma unroll
    for (int m = 0; m < 16; ++m) {  // this lane is k1 now, n2 in natural order
        R[m] = *reinterpret_cast<const float2 *>(&Sr[lane][2 * m]);
        I[m] = *reinterpret_cast<const float2 *>(&Si[lane][2 * m]);
    }
    __syncwarp();
    fft32_dif2<-1>(R, I);  // over n2: register e holds X[k1 + 32 k2], k2 = brev5(e)
#pragma unroll
    for (int m = 0; m < 16; ++m) cmul2q(R[m], I[m], __ldg(Hb + m * 32 + lane));
    fft32_dit2<1>(R, I);  // inverse over k2: register e holds n1' = e
#pragma unroll
    for (int m = 0; m < 16; ++m) cmul2q(R[m], I[m], __ldg(twn + m * 32 + lane));
#pragma unroll
    for (int e = 0; e < 32; ++e) {
        Sr[e][lane] = ev(R, e);
        Si[e][lane] = ev(I, e);
    }
    __syncwarp();
#pragma unroll
    for (int m = 0; m < 16; ++m) {  // this lane is n1', k1 in natural order
        R[m] = *reinterpret_cast<const float2 *>(&Sr[lane][2 * m]);
        I[m] = *reinterpret_cast<const float2 *>(&Si[lane][2 * m]);
    }
    fft32_dif2<1>(R, I);  // inverse over k1: register e holds y[n1' + 32 n2'], n2' = brev5(e)
    float *y1 = out + (size_t)c1 * T, *y2 = out + (size_t)c2 * T;
    if constexpr (EPI == 0) {
#pragma unroll
        for (int e = 0; e < 32; ++e) {
            const int n = lane + 32 * brev5(e);
            const int t = t0 + n - (L - 1);
            if (n >= L - 1 && t < T) {
                y1[t] = ev(R, e);
                if (has2) y2[t] = ev(I, e);
            }
        }
    } else {
        const int w = c1 / epi.D;
        const Scal &q = epi.sc[epi.coupled ? 0 : w];
        const float g = (float)q.gamma, sl = epi.sl;
        const bool done = EPI == 2 && q.done;
        const float *b1 = epi.b + (size_t)c1 * T, *b2 = epi.b + (size_t)c2 * T;
        float acc = 0.f;
        // chunks of 8 outputs: all loads of a chunk are issued before its
        // stores (the stores could alias the loads of later iterations)
        constexpr int CH = 8;
#pragma unroll
        for (int c0 = 0; c0 < 32; c0 += CH) {
            float l1[CH], l2[CH];
#pragma unroll
            for (int j = 0; j < CH; ++j) {
                const int n = lane + 32 * (c0 + j);
                const int t = t0 + n - (L - 1);
                const bool ok = n >= L - 1 && t < T;
                const float *s1 = EPI == 1 ? b1 : y1, *s2 = EPI == 1 ? b2 : y2;
                l1[j] = ok ? s1[t] : 0.f;
                l2[j] = (ok && has2) ? s2[t] : 0.f;
            }
#pragma unroll
            for (int j = 0; j < CH; ++j) {
                const int n2 = c0 + j, e = brev5(n2);
                const int n = lane + 32 * n2;
                const int t = t0 + n - (L - 1);
                if (n >= L - 1 && t < T) {
                    const float vr = ev(R, e), vi = ev(I, e);
                    float a, bb;
                    if (EPI == 1) {
                        a = fmaf(sl, l1[j], -sl * vr);
                        bb = has2 ? fmaf(sl, l2[j], -sl * vi) : 0.f;
                    } else {
                        a = done ? l1[j] : fmaf(sl, vr, -g * l1[j]);
                        bb = done ? l2[j] : fmaf(sl, vi, -g * l2[j]);
                    }
                    y1[t] = a;
                    if (has2) y2[t] = bb;
                    acc = fmaf(a, a, acc);
                    acc = fmaf(bb, bb, acc);
                }
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
        __shared__ float wacc[FPC];
        if (lane == 0) wacc[warp] = acc;
        __syncthreads();
        if (threadIdx.x == 0) {
            double sum = 0.0;
#pragma unroll
            for (int k = 0; k < FPC; ++k) sum += (double)wacc[k];
            const int per_inst = epi.D / (2 * FPC);  // CTAs (along y) per instance
            const int slot = (blockIdx.y - w * per_inst) * gridDim.x + blockIdx.x;
            epi.part[(size_t)w * epi.nparts + slot] = sum;
        }
    }
}

template <int LOG4N>
__global__ void __launch_bounds__(1 << (2 * LOG4N - 2)) k_conv_fft(
    const float *__restrict__ in, float *__restrict__ out, const float2 *__restrict__ tw,
    const float2 *__restrict__ H, int C, int T, int L) {
    constexpr int N = 1 << (2 * LOG4N), NT = N / 4;
    extern __shared__ float2 fbuf[];
    float2(*buf)[N] = reinterpret_cast<float2(*)[N]>(fbuf);
    const int V = N - L + 1;
    const int t0 = blockIdx.x * V;
    const int c1 = 2 * blockIdx.y, c2 = c1 + 1;
    const bool has2 = c2 < C;
    const int u0 = t0 + L / 2 - (L - 1);
    const float *x1 = in + (size_t)c1 * T;
    const float *x2 = in + (size_t)(has2 ? c2 : c1) * T;
    for (int n = threadIdx.x; n < N; n += NT) {
        const int u = u0 + n;
        const bool ok = u >= 0 && u < T;
        buf[0][n] = make_float2(ok ? __ldg(x1 + u) : 0.f, (ok && has2) ? __ldg(x2 + u) : 0.f);
    }
    __syncthreads();
    int cur = 0;
#pragma unroll
    for (int s = 0, Ls = 1; s < LOG4N; ++s, Ls *= 4) {
        radix4_stage<-1>(buf[cur], buf[cur ^ 1], tw, N, Ls, N / (4 * Ls), threadIdx.x);
        cur ^= 1;
        __syncthreads();
    }
    for (int n = threadIdx.x; n < N; n += NT) {
        const float2 v = buf[cur][n], h = __ldg(H + n);
        buf[cur][n] = make_float2(v.x * h.x - v.y * h.y, v.x * h.y + v.y * h.x);
    }
    __syncthreads();
#pragma unroll
    for (int s = 0, Ls = 1; s < LOG4N; ++s, Ls *= 4) {
        radix4_stage<1>(buf[cur], buf[cur ^ 1], tw, N, Ls, N / (4 * Ls), threadIdx.x);
        cur ^= 1;
        __syncthreads();
    }
    float *y1 = out + (size_t)c1 * T, *y2 = out + (size_t)c2 * T;
    for (int i = threadIdx.x; i < V; i += NT) {
        const int t = t0 + i;
        if (t >= T) break;
        const float2 r = buf[cur][L - 1 + i];
        y1[t] = r.x;
        if (has2) y2[t] = r.y;
    }
}

// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------
// kinks of the adjoint's piecewise-linear bucket response in the fraction f:
// r - F (where e1 reaches zero) and F + 1 - r (where e2 starts)
static float adj_p1(const Plan &pl) {
    return (float)std::min(pl.radius - pl.F, pl.F + 1 - pl.radius);
}
static float adj_p2(const Plan &pl) {
    return (float)std::max(pl.radius - pl.F, pl.F + 1 - pl.radius);
}

static int pick_wt(int W, int T, int max_wt) {
    for (int wt = max_wt; wt > 1; wt >>= 1)
        if (W % wt == 0 && (size_t)wt * T * sizeof(float) <= 160 * 1024) return wt;
    return 1;
}


int launch_prefilter(const Plan &pl, const float *in, float *out, int W, bool transpose,
                     bool along_x, float scale, int out_mode, cudaStream_t st) {
    TimedScope ts_(KID_PREFILTER, st);
    const int K = along_x ? pl.Kx : pl.Kz;
    const float *taps = along_x ? pl.pre_x : pl.pre_z;
    const long n = (long)W * pl.P;
    const int wt = out_mode == 2 ? das_fwd_wt(pl, W) : 1;
    const int fmt = out_mode == 2 ? pl.image_fmt : 0;
    if (fmt == 2)
        KLAUNCH(k_h16_scale<<<W, 256, 0, st>>>(
            in, pl.P, std::fabs(scale) * (along_x ? pl.pre_gain_x : pl.pre_gain_z), pl.h16_sc,
            pl.max_batch));
    KLAUNCH(k_prefilter<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(
        in, out, taps, K, pl.nx, pl.nz, W, along_x, transpose, scale, pl.perm, out_mode, wt, fmt,
        pl.h16_sc));
    MSOT_LAUNCH_CHECK();
    return MSOT_OK;
}

// both axes in one launch where the staged tile fits shared memory; returns
// 1 (nothing launched) when the caller must use the per-axis kernels
template <int KM>
static int prefilter2d_km(const Plan &pl, const float *in, float *out, int W, bool transpose,
                          int out_mode, cudaStream_t st) {
    constexpr int NC = PF_TX + 2 * KM;
    const size_t smem = (size_t)(2 * NC * (pl.nz | 1) + 2 * (2 * KM + 1)) * sizeof(float);
    if (smem > 200 * 1024) return 1;
    MSOT_CUDA_TRY(raise_max_dynamic_smem((const void *)k_prefilter2d<KM>, smem));
    const dim3 grid((unsigned)((pl.nx + PF_TX - 1) / PF_TX), (unsigned)W);
    const int wt = out_mode == 2 ? das_fwd_wt(pl, W) : 1;
    const int fmt = out_mode == 2 ? pl.image_fmt : 0;
    if (fmt == 2)
        KLAUNCH(k_h16_scale<<<W, 256, 0, st>>>(in, pl.P, pl.pre_gain_x * pl.pre_gain_z,
                                               pl.h16_sc, pl.max_batch));
    KLAUNCH(k_prefilter2d<KM><<<grid, PF_THREADS, smem, st>>>(
        in, out, pl.pre_x, pl.pre_z, pl.Kx, pl.Kz, pl.nx, pl.nz, W, transpose ? 1 : 0, out_mode,
        wt, fmt, pl.h16_sc));
    MSOT_LAUNCH_CHECK();
    return MSOT_OK;
}

int launch_prefilter2d(const Plan &pl, const float *in, float *out, int W, bool transpose,
                       int out_mode, cudaStream_t st) {
    if (pl.Kx < 0 || pl.Kz < 0 || (out_mode != 0 && out_mode != 2)) return 1;
    TimedScope ts_(KID_PREFILTER, st);
    const int K = std::max(pl.Kx, pl.Kz);
    if (K <= 8) return prefilter2d_km<8>(pl, in, out, W, transpose, out_mode, st);
    if (K <= 16) return prefilter2d_km<16>(pl, in, out, W, transpose, out_mode, st);
    return 1;
}

int launch_permute(const Plan &pl, const float *in, float *out, int W, cudaStream_t st) {
    TimedScope ts_(KID_PERMUTE, st);
    const long n = (long)W * pl.P;
    KLAUNCH(k_permute<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(in, out, pl.perm, pl.P, W));
    MSOT_LAUNCH_CHECK();
    return MSOT_OK;
}

static int fwd_split(const Plan &pl, int nwt) {
    // enough CTAs to fill the GPU twice over
    int ctas = pl.D * nwt;
    int ns = 1;
    while (ctas * ns < 2 * sm_count() && ns < 8) ns *= 2;
    return ns;
}

int launch_to_pixmajor(const Plan &pl, const float *in, float *out, int W, cudaStream_t st) {
    TimedScope ts_(KID_PERMUTE, st);
    const long n = (long)W * pl.P;
    if (pl.image_fmt == 2)
        KLAUNCH(k_h16_scale<<<W, 256, 0, st>>>(in, pl.P, 1.f, pl.h16_sc, pl.max_batch));
    KLAUNCH(k_to_pixmajor<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(
        in, out, pl.P, W, das_fwd_wt(pl, W), pl.image_fmt, pl.h16_sc));
    MSOT_LAUNCH_CHECK();
    return MSOT_OK;
}

std::atomic<int> g_fwd_staged{1};
std::atomic<int> g_fwd_ell{1};

// the DAS forward kernel: the autotuner's pick, else 4 (the interleaved
// entry table, the fastest on GB300) when msot_tune_set("fwd_ell") is on
// (default) and the plan has the table, else 1 (staged) or 2 (k_das_fwd3 on
// the CSR table) by msot_tune_set("fwd_staged"); all give the same sums
static int fwd_kernel(const Plan &pl) {
    if (pl.tune_fwd_staged) return pl.tune_fwd_staged;
    if (g_fwd_ell.load() && pl.fwd_ell_off) return 4;
    return g_fwd_staged.load() ? 1 : 2;
}

// the staged kernel (das_fwd_staged.cu) where the plan has its tables and
// they fit shared memory at this instance tile, else k_das_fwd3
static bool use_staged(const Plan &pl, int wt) {
    if (pl.image_fmt) return false;  // 16-bit storage is read by k_das_fwd3 only
    return fwd_kernel(pl) == 1 && fwd_staged_fits(pl, wt);
}

// instances per CTA of the DAS forward: the autotuner's pick (16, 8, 4, 2),
// else the largest of 8, 4, 2 dividing W
int das_fwd_wt(const Plan &pl, int W) {
    if (pl.tune_fwd_wt && W % pl.tune_fwd_wt == 0) return pl.tune_fwd_wt;
    return pick_wt(W, 1, 8);
}

int launch_das_forward(const Plan &pl, const float *xpm, float *raw, int W, float scale,
                       cudaStream_t st) {
    TimedScope ts_(KID_INTERP_FWD, st);
    const int wt = das_fwd_wt(pl, W);
    if (use_staged(pl, wt)) return launch_das_forward_staged(pl, xpm, raw, W, wt, scale, st);
    // k_das_fwd3 in the plan's storage format (das_fwd_f32.cu, das_fwd_bf16.cu,
    // das_fwd_f16.cu), on the interleaved entry table where chosen
    const bool ell = fwd_kernel(pl) == 4 && pl.fwd_ell_off;
    if (pl.image_fmt == 1) return das_fwd_run_bf16(pl, xpm, raw, W, scale, nullptr, ell, wt, st);
    if (pl.image_fmt == 2)
        return das_fwd_run_f16(pl, xpm, raw, W, scale, pl.h16_sc + pl.max_batch, ell, wt, st);
    return das_fwd_run_f32(pl, xpm, raw, W, scale, nullptr, ell, wt, st);
}

// DAS adjoint by pixel blocks; raw [W][D][T] -> x [W][P].
template <int WT, int F>
static int das_adj_launch(const Plan &pl, const float *raw, float *x, int W, float scale,
                          cudaStream_t st) {
    const int SL = div_up(pl.blk_span_max, ADJ_BPT) * ADJ_BPT + 2 * F + 2;
    const size_t smem = (size_t)((WT * SL + 3) & ~3) * sizeof(float) +
                        (size_t)WT * 3 * pl.blk_span_max * sizeof(float2);
    int rc;
    const int base = pl.n_blk * (W / WT);
    int groups = std::max(1, std::min(pl.D, div_up(2 * sm_count(), base)));
    groups = std::min(groups, std::max(1, pl.adj_groups_max * pl.max_batch / W));
    groups = std::min(groups, pl.adj_groups_max);
    const int dpg = div_up(pl.D, groups);
    groups = div_up(pl.D, dpg);
    const size_t stride = (size_t)W * pl.P;
    dim3 grid(pl.n_blk, W / WT, groups);
#define ADJ4_LAUNCH(PFV)                                                                   \
    do {                                                                                   \
        if ((rc = set_smem(k_das_adj4<WT, F, PFV>, smem)) != MSOT_OK) return rc;           \
        KLAUNCH(k_das_adj4<WT, F, PFV><<<grid, BLK_THREADS, smem, st>>>(                   \
            pl.blk_tau, pl.blk_span, raw, pl.scr_part, pl.nx, pl.nz, pl.n_blk_x, pl.D, pl.T, \
            pl.frac_bits, pl.inv_r, pl.ce1, pl.ce2, adj_p1(pl), adj_p2(pl), pl.blk_span_max, dpg, \
            stride));                                                                      \
    } while (0)
    // next-detector prefetch when the segment fits PF registers per instance
    if (g_adj_prefetch.load() && SL <= 2 * BLK_THREADS)
        ADJ4_LAUNCH(2);
    else if (g_adj_prefetch.load() && SL <= 4 * BLK_THREADS)
        ADJ4_LAUNCH(4);
    else
        ADJ4_LAUNCH(0);
#undef ADJ4_LAUNCH
    MSOT_LAUNCH_CHECK();
    KLAUNCH(k_sum_parts<<<(unsigned)std::min<size_t>(4096, div_up((int)stride, 256)), 256, 0,
                          st>>>(pl.scr_part, x, stride, groups, stride, scale));
    MSOT_LAUNCH_CHECK();
    return MSOT_OK;
}

template <int WT>
static int das_adj_f(const Plan &pl, const float *raw, float *x, int W, float scale,
                     cudaStream_t st) {
    switch (pl.F) {
        case 0: return das_adj_launch<WT, 0>(pl, raw, x, W, scale, st);
        case 1: return das_adj_launch<WT, 1>(pl, raw, x, W, scale, st);
        case 2: return das_adj_launch<WT, 2>(pl, raw, x, W, scale, st);
        case 3: return das_adj_launch<WT, 3>(pl, raw, x, W, scale, st);
        case 4: return das_adj_launch<WT, 4>(pl, raw, x, W, scale, st);
        case 5: return das_adj_launch<WT, 5>(pl, raw, x, W, scale, st);
        case 6: return das_adj_launch<WT, 6>(pl, raw, x, W, scale, st);
        case 7: return das_adj_launch<WT, 7>(pl, raw, x, W, scale, st);
        case 8: return das_adj_launch<WT, 8>(pl, raw, x, W, scale, st);
        default:
            set_error("DAS adjoint: interpolation radius %g above 9 samples is not supported",
                      pl.radius);
            return MSOT_EINVAL;
    }
}

int launch_das_adjoint(const Plan &pl, const float *raw, float *x, int W, float scale,
                       cudaStream_t st) {
    TimedScope ts_(KID_INTERP_ADJ, st);
    int wt = pick_wt(W, 1, 2);
    if (pl.tune_adj_wt && W % pl.tune_adj_wt == 0) wt = pl.tune_adj_wt;
    if (wt == 4) return das_adj_f<4>(pl, raw, x, W, scale, st);
    if (wt == 2) return das_adj_f<2>(pl, raw, x, W, scale, st);
    return das_adj_f<1>(pl, raw, x, W, scale, st);
}

template <int WT>
static int sir_fwd_nt(const Plan &pl, const float *x_pi, float *raw, float scale, dim3 grid,
                      size_t smem, int ns, cudaStream_t st) {
    int rc;
#define NTCASE(NT)                                                                         \
    if (pl.n_tap <= NT) {                                                                  \
        if ((rc = set_smem(k_sir_fwd<WT, NT>, smem)) != MSOT_OK) return rc;                \
        KLAUNCH(k_sir_fwd<WT, NT><<<grid, 256, smem, st>>>(pl.tau_pi, pl.sir_pi, pl.sir, pl.sir_se, \
                                                   x_pi, raw, pl.P, pl.D, pl.T, pl.S,      \
                                                   pl.frac_bits, pl.r_fx, pl.c1, scale, ns)); \
        MSOT_LAUNCH_CHECK();                                                               \
        return MSOT_OK;                                                                    \
    }
    NTCASE(4) NTCASE(8) NTCASE(12) NTCASE(16) NTCASE(24) NTCASE(32)
#undef NTCASE
    set_error("SIR: interpolation radius too large (%d taps)", pl.n_tap);
    return MSOT_EINVAL;
}

int launch_sir_forward(const Plan &pl, const float *x_pi, float *raw, int W, float scale,
                       cudaStream_t st) {
    TimedScope ts_(KID_INTERP_FWD, st);
    const int wt = pick_wt(W, pl.T, 4);
    const int ns = fwd_split(pl, W / wt);
    if (ns > 1) MSOT_CUDA_TRY(cudaMemsetAsync(raw, 0, sizeof(float) * W * pl.D * pl.T, st));
    const size_t smem = (size_t)wt * pl.T * sizeof(float);
    dim3 grid(pl.D, ns, W / wt);
    switch (wt) {
        case 1: return sir_fwd_nt<1>(pl, x_pi, raw, scale, grid, smem, ns, st);
        case 2: return sir_fwd_nt<2>(pl, x_pi, raw, scale, grid, smem, ns, st);
        default: return sir_fwd_nt<4>(pl, x_pi, raw, scale, grid, smem, ns, st);
    }
}

template <int WT>
static int sir_adj_nt(const Plan &pl, const float *raw, float *x, float scale, dim3 grid,
                      cudaStream_t st) {
#define NTCASE(NT)                                                                         \
    if (pl.n_tap <= NT) {                                                                  \
        KLAUNCH(k_sir_adj<WT, NT><<<grid, 256, 0, st>>>(pl.tau_tiles, pl.sir_tiles, pl.sir,         \
                                                pl.sir_se, raw, x, pl.nx, pl.nz,           \
                                                pl.n_patch_x, pl.D, pl.T, pl.S,            \
                                                pl.frac_bits, pl.r_fx, pl.c1, scale));      \
        MSOT_LAUNCH_CHECK();                                                               \
        return MSOT_OK;                                                                    \
    }
    NTCASE(4) NTCASE(8) NTCASE(12) NTCASE(16) NTCASE(24) NTCASE(32)
#undef NTCASE
    set_error("SIR: interpolation radius too large (%d taps)", pl.n_tap);
    return MSOT_EINVAL;
}

int launch_sir_adjoint(const Plan &pl, const float *raw, float *x, int W, float scale,
                       cudaStream_t st) {
    TimedScope ts_(KID_INTERP_ADJ, st);
    const int wt = pick_wt(W, 1, 2);
    dim3 grid(pl.n_patch, W / wt);
    if (wt == 2) return sir_adj_nt<2>(pl, raw, x, scale, grid, st);
    return sir_adj_nt<1>(pl, raw, x, scale, grid, st);
}

constexpr int CONV_FPC = 4;
// minimum resident CTAs per SM the convolution is compiled for (register
// cap): 1 = unconstrained (about 155 registers, 3 CTAs fit), 3 (the same),
// 4 (128 registers, no spills; the fastest on GB300);
// msot_tune_set("conv_min_blocks")
std::atomic<int> g_conv_min_blocks{4};
static int conv_min_blocks(const Plan &pl) {
    return pl.tune_conv_mb ? pl.tune_conv_mb : g_conv_min_blocks.load();
}

int launch_conv(const Plan &pl, const float *in, float *out, int W, bool transpose,
                cudaStream_t st) {
    TimedScope ts_(KID_CONV, st);
    if (pl.fft_log4n) {
        const int C = W * pl.D;
        const int N = 1 << (2 * pl.fft_log4n), V = N - pl.L + 1;
        dim3 grid(div_up(pl.T, V), div_up(C, 2));
        const float2 *H = transpose ? pl.fft_ha : pl.fft_hf;
        const size_t smem = 2 * (size_t)N * sizeof(float2);
        int rc;
        if (pl.fft_log4n == 5) {
            constexpr int FPC = CONV_FPC;
            dim3 g1(div_up(pl.T, V), div_up(div_up(C, 2), FPC));
            const float4 *Hb = transpose ? pl.fft_hab : pl.fft_hfb;
            switch (conv_min_blocks(pl)) {
            case 3:
                KLAUNCH(k_conv_fft1k<FPC, 0, 3><<<g1, 32 * FPC, 0, st>>>(
                    in, out, pl.fft_twb, pl.fft_twn, Hb, C, pl.T, pl.L));
                break;
            case 4:
                KLAUNCH(k_conv_fft1k<FPC, 0, 4><<<g1, 32 * FPC, 0, st>>>(
                    in, out, pl.fft_twb, pl.fft_twn, Hb, C, pl.T, pl.L));
                break;
            default:
                KLAUNCH(k_conv_fft1k<FPC><<<g1, 32 * FPC, 0, st>>>(in, out, pl.fft_twb,
                                                                    pl.fft_twn, Hb, C, pl.T,
                                                                    pl.L));
            }
        } else {
            if ((rc = set_smem(k_conv_fft<6>, smem)) != MSOT_OK) return rc;
            KLAUNCH(k_conv_fft<6><<<grid, N / 4, smem, st>>>(in, out, pl.fft_tw, H, C, pl.T,
                                                             pl.L));
        }
        MSOT_LAUNCH_CHECK();
        return MSOT_OK;
    }
    constexpr int TPT = 8, NTH = 64, TT = TPT * NTH;
    const int Lp = (pl.L + TPT - 1) / TPT * TPT;
    const int seg_len = TT + Lp + TPT;
    const size_t smem = sizeof(float) * (Lp + seg_len + seg_len / 8 + 1);
    int rc;
    if ((rc = set_smem(k_conv<TPT, NTH>, smem)) != MSOT_OK) return rc;
    dim3 grid(div_up(pl.T, TT), (unsigned)W * pl.D);
    KLAUNCH(k_conv<TPT, NTH><<<grid, NTH, smem, st>>>(in, out, transpose ? pl.ir_adj : pl.ir_fwd,
                                              pl.L, pl.T));
    MSOT_LAUNCH_CHECK();
    return MSOT_OK;
}

bool forward_update_fusable(const Plan &pl, int W) {
    if (pl.L <= 0 || pl.fft_log4n != 5 || pl.D % (2 * CONV_FPC) != 0) return false;
    const int V = 1024 - pl.L + 1;
    const int nparts = (pl.D / (2 * CONV_FPC)) * div_up(pl.T, V);
    return nparts <= 256 && W >= 1;
}

// ---------------------------------------------------------------------------
// chains
// ---------------------------------------------------------------------------
int interp_forward(const Plan &pl, const float *x_pi, float *raw, int W, float scale,
                   cudaStream_t st) {
    return pl.S ? launch_sir_forward(pl, x_pi, raw, W, scale, st)
                : launch_das_forward(pl, x_pi, raw, W, scale, st);
}

int interp_adjoint(const Plan &pl, const float *raw, float *x, int W, float scale,
                   cudaStream_t st) {
    return pl.S ? launch_sir_adjoint(pl, raw, x, W, scale, st)
                : launch_das_adjoint(pl, raw, x, W, scale, st);
}

static int forward_to_raw(const Plan &pl, const float *img, int W, cudaStream_t st);

int apply_forward(const Plan &pl, const float *img, float *sino, int W, cudaStream_t st) {
    int rc;
    if (pl.L > 0) {
        if ((rc = forward_to_raw(pl, img, W, st))) return rc;
        return launch_conv(pl, pl.scr_sino, sino, W, false, st);
    }
    float *xpi = pl.scr_img1;
    const int mode = pl.S ? 1 : 2;  // scatter order (SIR) or pixel-major (bucket moments)
    if ((rc = launch_prefilter2d(pl, img, xpi, W, false, mode, st)) <= 0) {
        if (rc) return rc;
    } else if (pl.Kz >= 0 && pl.Kx >= 0) {
        if ((rc = launch_prefilter(pl, img, pl.scr_img0, W, false, false, 1.f, 0, st)))
            return rc;
        if ((rc = launch_prefilter(pl, pl.scr_img0, xpi, W, false, true, 1.f, mode, st)))
            return rc;
    } else if (pl.Kz >= 0) {
        if ((rc = launch_prefilter(pl, img, xpi, W, false, false, 1.f, mode, st))) return rc;
    } else if (pl.Kx >= 0) {
        if ((rc = launch_prefilter(pl, img, xpi, W, false, true, 1.f, mode, st))) return rc;
    } else if (pl.S) {
        if ((rc = launch_permute(pl, img, xpi, W, st))) return rc;
    } else {
        if ((rc = launch_to_pixmajor(pl, img, xpi, W, st))) return rc;
    }
    return interp_forward(pl, xpi, sino, W, pl.scale, st);
}

// prefilter + interpolation into the plan's sinogram scratch (the
// convolution's input); shared by apply_forward and apply_forward_update
static int forward_to_raw(const Plan &pl, const float *img, int W, cudaStream_t st) {
    int rc;
    float *xpi = pl.scr_img1;
    const int mode = pl.S ? 1 : 2;
    if ((rc = launch_prefilter2d(pl, img, xpi, W, false, mode, st)) <= 0) {
        if (rc) return rc;
    } else if (pl.Kz >= 0 && pl.Kx >= 0) {
        if ((rc = launch_prefilter(pl, img, pl.scr_img0, W, false, false, 1.f, 0, st)))
            return rc;
        if ((rc = launch_prefilter(pl, pl.scr_img0, xpi, W, false, true, 1.f, mode, st)))
            return rc;
    } else if (pl.Kz >= 0) {
        if ((rc = launch_prefilter(pl, img, xpi, W, false, false, 1.f, mode, st))) return rc;
    } else if (pl.Kx >= 0) {
        if ((rc = launch_prefilter(pl, img, xpi, W, false, true, 1.f, mode, st))) return rc;
    } else if (pl.S) {
        if ((rc = launch_permute(pl, img, xpi, W, st))) return rc;
    } else {
        if ((rc = launch_to_pixmajor(pl, img, xpi, W, st))) return rc;
    }
    return interp_forward(pl, xpi, pl.scr_sino, W, 1.f, st);
}

int apply_forward_update(const Plan &pl, const float *img, float *u, const float *b, int W,
                         int mode, float sl, const Scal *sc, int coupled, double *part,
                         int *nparts, cudaStream_t st) {
    if (!forward_update_fusable(pl, W)) return 1;
    int rc;
    if ((rc = forward_to_raw(pl, img, W, st))) return rc;
    TimedScope ts_(KID_CONV, st);
    const int C = W * pl.D, V = 1024 - pl.L + 1;
    const dim3 g1(div_up(pl.T, V), div_up(div_up(C, 2), CONV_FPC));
    ConvEpi e;
    e.b = b;
    e.sc = sc;
    e.sl = sl;
    e.coupled = coupled;
    e.D = pl.D;
    e.nparts = (pl.D / (2 * CONV_FPC)) * (int)g1.x;
    e.part = part;
    *nparts = e.nparts;
    const int mb = conv_min_blocks(pl);
#define CONV_EPI_LAUNCH(EPI, MB)                                                           \
    KLAUNCH(k_conv_fft1k<CONV_FPC, EPI, MB><<<g1, 32 * CONV_FPC, 0, st>>>(                \
        pl.scr_sino, u, pl.fft_twb, pl.fft_twn, pl.fft_hfb, C, pl.T, pl.L, e))
    if (mode == 0) {
        if (mb == 3) CONV_EPI_LAUNCH(1, 3);
        else if (mb == 4) CONV_EPI_LAUNCH(1, 4);
        else CONV_EPI_LAUNCH(1, 1);
    } else {
        if (mb == 3) CONV_EPI_LAUNCH(2, 3);
        else if (mb == 4) CONV_EPI_LAUNCH(2, 4);
        else CONV_EPI_LAUNCH(2, 1);
    }
#undef CONV_EPI_LAUNCH
    MSOT_LAUNCH_CHECK();
    return MSOT_OK;
}

int apply_transpose(const Plan &pl, const float *sino, float *img, int W, cudaStream_t st) {
    int rc;
    const float *src = sino;
    float scale = pl.scale;
    if (pl.L > 0) {
        if ((rc = launch_conv(pl, sino, pl.scr_sino, W, true, st))) return rc;
        src = pl.scr_sino;
        scale = 1.f;
    }
    const bool pre = pl.Kx >= 0 || pl.Kz >= 0;
    float *x = pre ? pl.scr_img0 : img;
    if ((rc = interp_adjoint(pl, src, x, W, scale, st))) return rc;
    if ((rc = launch_prefilter2d(pl, pl.scr_img0, img, W, true, 0, st)) <= 0) return rc;
    if (pl.Kx >= 0 && pl.Kz >= 0) {
        if ((rc = launch_prefilter(pl, pl.scr_img0, pl.scr_img1, W, true, true, 1.f, 0, st)))
            return rc;
        return launch_prefilter(pl, pl.scr_img1, img, W, true, false, 1.f, 0, st);
    }
    if (pl.Kx >= 0) return launch_prefilter(pl, pl.scr_img0, img, W, true, true, 1.f, 0, st);
    if (pl.Kz >= 0) return launch_prefilter(pl, pl.scr_img0, img, W, true, false, 1.f, 0, st);
    return MSOT_OK;
}

}  // namespace msot

namespace msot {
// ---------------------------------------------------------------------------
// Allocation-free variant of the DAS adjoint.
//
// The adjoint keeps one partial image per detector group in scratch memory.
// msot_interp_transpose takes that scratch from the plan; this variant takes
// it from a fixed array that is part of the library image instead, so a call
// allocates no device memory at all.  The array is NOALLOC_PART_FLOATS floats
// (16 MiB) on every device that loads the library, for the lifetime of the
// process.  Host code cannot pass the array's name to a kernel (on the host
// it is only a stand-in symbol), so its device address is looked up once per
// device with cudaGetSymbolAddress, on the first call made with that device
// current.
// ---------------------------------------------------------------------------
constexpr size_t NOALLOC_PART_FLOATS = (size_t)4 << 20;
static __device__ __align__(256) float g_noalloc_part[NOALLOC_PART_FLOATS];

static int noalloc_part_address(float **out) {
    constexpr int kMaxDev = 64;
    static float *addr[kMaxDev] = {};
    static std::mutex mu;
    int dev = 0;
    MSOT_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDev) {
        set_error("noalloc: device index %d not supported", dev);
        return MSOT_EINVAL;
    }
    std::lock_guard<std::mutex> g(mu);
    if (!addr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_part);
        if (e != cudaSuccess || !p) {
            set_error("noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
            return MSOT_ECUDA;
        }
        addr[dev] = static_cast<float *>(p);
    }
    *out = addr[dev];
    return MSOT_OK;
}

template <int WT, int F>
static int das_adj_launch_fixed(const Plan &pl, const float *raw, float *x, int W,
                                cudaStream_t st, float *part) {
    const int SL = div_up(pl.blk_span_max, ADJ_BPT) * ADJ_BPT + 2 * F + 2;
    const size_t smem = (size_t)((WT * SL + 3) & ~3) * sizeof(float) +
                        (size_t)WT * 3 * pl.blk_span_max * sizeof(float2);
    int rc;
    if ((rc = set_smem(k_das_adj4<WT, F>, smem)) != MSOT_OK) return rc;
    const size_t stride = (size_t)W * pl.P;
    const int base = pl.n_blk * (W / WT);
    int groups = std::max(1, std::min(pl.D, div_up(2 * sm_count(), base)));
    groups = std::min<size_t>(groups, NOALLOC_PART_FLOATS / stride);
    const int dpg = div_up(pl.D, groups);
    groups = div_up(pl.D, dpg);
    dim3 grid(pl.n_blk, W / WT, groups);
    // every (group, instance, pixel) element of the array is written by
    // k_das_adj4 before k_sum_parts reads it: nothing needs clearing
    KLAUNCH(k_das_adj4<WT, F><<<grid, BLK_THREADS, smem, st>>>(
        pl.blk_tau, pl.blk_span, raw, part, pl.nx, pl.nz, pl.n_blk_x, pl.D, pl.T,
        pl.frac_bits, pl.inv_r, pl.ce1, pl.ce2, adj_p1(pl), adj_p2(pl), pl.blk_span_max, dpg,
        stride));
    MSOT_LAUNCH_CHECK();
    KLAUNCH(k_sum_parts<<<(unsigned)std::min<size_t>(4096, div_up((int)stride, 256)), 256, 0,
                          st>>>(part, x, stride, groups, stride, 1.f));
    MSOT_LAUNCH_CHECK();
    return MSOT_OK;
}

template <int WT>
static int das_adj_fixed_f(const Plan &pl, const float *raw, float *x, int W, cudaStream_t st,
                           float *part) {
    switch (pl.F) {
        case 0: return das_adj_launch_fixed<WT, 0>(pl, raw, x, W, st, part);
        case 1: return das_adj_launch_fixed<WT, 1>(pl, raw, x, W, st, part);
        case 2: return das_adj_launch_fixed<WT, 2>(pl, raw, x, W, st, part);
        case 3: return das_adj_launch_fixed<WT, 3>(pl, raw, x, W, st, part);
        case 4: return das_adj_launch_fixed<WT, 4>(pl, raw, x, W, st, part);
        case 5: return das_adj_launch_fixed<WT, 5>(pl, raw, x, W, st, part);
        case 6: return das_adj_launch_fixed<WT, 6>(pl, raw, x, W, st, part);
        case 7: return das_adj_launch_fixed<WT, 7>(pl, raw, x, W, st, part);
        case 8: return das_adj_launch_fixed<WT, 8>(pl, raw, x, W, st, part);
        default:
            set_error("DAS adjoint: interpolation radius %g above 9 samples is not supported",
                      pl.radius);
            return MSOT_EINVAL;
    }
}
}  // namespace msot

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
using namespace msot;

static int check_batch(msot_plan_t plan, int batch, const void *a, const void *b) {
    if (!plan || !a || !b || batch <= 0) {
        set_error("null plan/pointer or non-positive batch");
        return MSOT_EINVAL;
    }
    if (batch > plan->p.max_batch) {
        set_error("batch %d exceeds the plan's max_batch %d", batch, plan->p.max_batch);
        return MSOT_EINVAL;
    }
    return check_plan_device(plan->p, "operator");
}

extern "C" {

int msot_forward(msot_plan_t plan, const float *d_img, float *d_sino, int batch, void *stream) {
    int rc = check_batch(plan, batch, d_img, d_sino);
    if (rc) return rc;
    return apply_forward(plan->p, d_img, d_sino, batch, (cudaStream_t)stream);
}

int msot_transpose(msot_plan_t plan, const float *d_sino, float *d_img, int batch,
                   void *stream) {
    int rc = check_batch(plan, batch, d_sino, d_img);
    if (rc) return rc;
    return apply_transpose(plan->p, d_sino, d_img, batch, (cudaStream_t)stream);
}

int msot_interp_forward(msot_plan_t plan, const float *d_coeffs, float *d_raw, int batch,
                        void *stream) {
    int rc = check_batch(plan, batch, d_coeffs, d_raw);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    if (plan->p.S) {
        if ((rc = launch_permute(plan->p, d_coeffs, plan->p.scr_img1, batch, st))) return rc;
    } else {
        if ((rc = launch_to_pixmajor(plan->p, d_coeffs, plan->p.scr_img1, batch, st))) return rc;
    }
    return interp_forward(plan->p, plan->p.scr_img1, d_raw, batch, 1.f, st);
}

int msot_interp_transpose(msot_plan_t plan, const float *d_raw, float *d_coeffs, int batch,
                          void *stream) {
    int rc = check_batch(plan, batch, d_raw, d_coeffs);
    if (rc) return rc;
    return interp_adjoint(plan->p, d_raw, d_coeffs, batch, 1.f, (cudaStream_t)stream);
}

int msot_plan_set_storage(msot_plan_t plan, int image_format, int refine_every) {
    if (!plan || image_format < 0 || image_format > 2 || refine_every < 0) {
        set_error("plan_set_storage: image_format must be 0 (FP32), 1 (BF16) or 2 (FP16) and "
                  "refine_every >= 0");
        return MSOT_EINVAL;
    }
    Plan &pl = plan->p;
    if (image_format && pl.S) {
        set_error("plan_set_storage: 16-bit storage is for plans without SIR");
        return MSOT_EINVAL;
    }
    pl.storage_fmt = pl.image_fmt = image_format;
    pl.refine_every = refine_every;
    solver_cache_invalidate(pl);  // captured graphs hold the previous kernels
    return MSOT_OK;
}

int msot_interp_transpose_noalloc(msot_plan_t plan, const float *d_raw, float *d_coeffs,
                                  int batch, void *stream) {
    if (!plan || !d_raw || !d_coeffs || batch <= 0) {
        set_error("interp_transpose_noalloc: null plan/pointer or non-positive batch");
        return MSOT_EINVAL;
    }
    const Plan &pl = plan->p;
    if (pl.S) {
        set_error("interp_transpose_noalloc: plans with a spatial impulse response are not "
                  "supported");
        return MSOT_EINVAL;
    }
    if (int rc0 = check_plan_device(pl, "interp_transpose_noalloc")) return rc0;
    if ((size_t)batch * pl.P > NOALLOC_PART_FLOATS) {
        set_error("interp_transpose_noalloc: batch x pixels = %zu exceeds the fixed scratch of "
                  "%zu floats",
                  (size_t)batch * pl.P, NOALLOC_PART_FLOATS);
        return MSOT_ERANGE;
    }
    float *part = nullptr;
    int rc = noalloc_part_address(&part);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const int wt = pick_wt(batch, 1, 2);
    if (wt == 2) return das_adj_fixed_f<2>(pl, d_raw, d_coeffs, batch, st, part);
    return das_adj_fixed_f<1>(pl, d_raw, d_coeffs, batch, st, part);
}

}  // extern "C"
