// das_fwd.cuh -- k_das_fwd3, the DAS forward by bucket moments
// (forwardDelayAndSumMex.cpp:72-103 restated per detector bucket; the
// decomposition is described at the bucket section of operator.cu), and its
// launch over the instance tiles and interpolation radii.  Included by one
// translation unit per storage format of the interpolation input
// (das_fwd_f32.cu, das_fwd_bf16.cu, das_fwd_f16.cu), which compile in
// parallel.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <type_traits>

#include "common.cuh"

namespace msot {

// CTA = (tile of TB = 256 - 2F - 2 output samples, detector, WT instances);
// the image is [W/WT][P][WT].
// Phase 1: one bucket per thread reduces the four moments of its pixels,
// loading FWD_UNR (entry, pixel) pairs at a time; phase 2: each output sample
// applies the (2F+2)-tap filter over the bucket moments.
constexpr int FWD_UNR = 2;

// one pixel's WT instance values of the interpolation input, FP32 or BF16
// (widened exactly: a BF16 value is the upper half of its FP32 pattern)
template <int WT>
__device__ __forceinline__ void load_pixel(const float *xp, float (&xv)[WT]) {
    if constexpr (WT % 8 == 0) {
        // one 256-bit load per 8 values (xp is 32-byte aligned: [W/WT][P][WT])
#pragma unroll
        for (int i = 0; i < WT; i += 8)
            asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                : "=f"(xv[i]), "=f"(xv[i + 1]), "=f"(xv[i + 2]), "=f"(xv[i + 3]),
                  "=f"(xv[i + 4]), "=f"(xv[i + 5]), "=f"(xv[i + 6]), "=f"(xv[i + 7])
                : "l"(xp + i));
    } else if constexpr (WT % 4 == 0) {
#pragma unroll
        for (int i = 0; i < WT; i += 4) {
            const float4 v = __ldg(reinterpret_cast<const float4 *>(xp + i));
            xv[i] = v.x; xv[i + 1] = v.y; xv[i + 2] = v.z; xv[i + 3] = v.w;
        }
    } else {
#pragma unroll
        for (int i = 0; i < WT; ++i) xv[i] = __ldg(xp + i);
    }
}
// eight 32-bit words of a 32-byte aligned address in one 256-bit load
__device__ __forceinline__ void ld256(const void *p, uint32_t (&u)[8]) {
    asm("ld.global.nc.v8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=r"(u[0]), "=r"(u[1]), "=r"(u[2]), "=r"(u[3]), "=r"(u[4]), "=r"(u[5]), "=r"(u[6]),
          "=r"(u[7])
        : "l"(p));
}
__device__ __forceinline__ float bf16_lo(uint32_t v) { return __uint_as_float(v << 16); }
__device__ __forceinline__ float bf16_hi(uint32_t v) { return __uint_as_float(v & 0xffff0000u); }
template <int WT>
__device__ __forceinline__ void load_pixel(const __nv_bfloat16 *xp, float (&xv)[WT]) {
    if constexpr (WT % 16 == 0) {
#pragma unroll
        for (int i = 0; i < WT; i += 16) {
            uint32_t u[8];
            ld256(xp + i, u);
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                xv[i + 2 * k] = bf16_lo(u[k]);
                xv[i + 2 * k + 1] = bf16_hi(u[k]);
            }
        }
    } else if constexpr (WT % 8 == 0) {
#pragma unroll
        for (int i = 0; i < WT; i += 8) {
            const uint4 v = __ldg(reinterpret_cast<const uint4 *>(xp + i));
            xv[i] = bf16_lo(v.x); xv[i + 1] = bf16_hi(v.x);
            xv[i + 2] = bf16_lo(v.y); xv[i + 3] = bf16_hi(v.y);
            xv[i + 4] = bf16_lo(v.z); xv[i + 5] = bf16_hi(v.z);
            xv[i + 6] = bf16_lo(v.w); xv[i + 7] = bf16_hi(v.w);
        }
    } else if constexpr (WT % 2 == 0) {
#pragma unroll
        for (int i = 0; i < WT; i += 2) {
            const uint32_t v = __ldg(reinterpret_cast<const unsigned int *>(xp + i));
            xv[i] = bf16_lo(v); xv[i + 1] = bf16_hi(v);
        }
    } else {
        xv[0] = __uint_as_float((uint32_t)__ldg(reinterpret_cast<const unsigned short *>(xp)) << 16);
    }
}

template <int WT>
__device__ __forceinline__ void load_pixel(const __half *xp, float (&xv)[WT]) {
    if constexpr (WT % 16 == 0) {
#pragma unroll
        for (int i = 0; i < WT; i += 16) {
            uint32_t u[8];
            ld256(xp + i, u);
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const float2 f = __half22float2(*reinterpret_cast<const __half2 *>(&u[k]));
                xv[i + 2 * k] = f.x;
                xv[i + 2 * k + 1] = f.y;
            }
        }
    } else if constexpr (WT % 8 == 0) {
#pragma unroll
        for (int i = 0; i < WT; i += 8) {
            const uint4 v = __ldg(reinterpret_cast<const uint4 *>(xp + i));
            const uint32_t u[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const float2 f = __half22float2(*reinterpret_cast<const __half2 *>(&u[k]));
                xv[i + 2 * k] = f.x;
                xv[i + 2 * k + 1] = f.y;
            }
        }
    } else if constexpr (WT % 2 == 0) {
#pragma unroll
        for (int i = 0; i < WT; i += 2) {
            const float2 f = __half22float2(__ldg(reinterpret_cast<const __half2 *>(xp + i)));
            xv[i] = f.x;
            xv[i + 1] = f.y;
        }
    } else {
        xv[0] = __half2float(__ldg(xp));
    }
}

// ELL: the entries come from the interleaved table (Plan::fwd_ell; `ent`
// and `ell_off` are it and its block offsets): a warp's load of the k-th
// entries of its 32 buckets is 256 contiguous bytes instead of 32 separate
// lines, which the L1 data pipe -- this kernel's bound -- serves in two
// wavefronts.  Same entries in the same order per bucket: the same result.
template <int WT, int F, typename XT = float, bool ELL = false>
__global__ void __launch_bounds__(256, WT >= 16 ? 2 : 4) k_das_fwd3(const int32_t *__restrict__ off,
                                                  const int2 *__restrict__ ent,
                                                  const XT *__restrict__ xpm,
                                                  float *__restrict__ raw, int P, int D, int T,
                                                  int W, int fb, float inv_r, float ce1,
                                                  float ce2, float scale,
                                                  const float *__restrict__ inv_s = nullptr,
                                                  const int32_t *__restrict__ ell_off = nullptr) {
    constexpr int NB = 256;
    constexpr int TB = NB - 2 * F - 2;
    extern __shared__ float mom[];  // [4][WT][NB], bucket fastest (dynamic: 4 KB x WT)
    const int d = blockIdx.y, w0 = blockIdx.z * WT;
    const int t0 = blockIdx.x * TB;
    const int b_lo = t0 - F - 1;
    {
        // no pixel of this detector falls in the CTA's buckets (outside its
        // travel-time span): every output of the tile is zero
        const int32_t *o = off + (size_t)d * (T + 1);
        const int bl = max(b_lo, 0), bh = min(b_lo + NB, T);
        if (bl >= bh || __ldg(o + bl) == __ldg(o + bh)) {
            const int t = t0 + (int)threadIdx.x;
            if ((int)threadIdx.x < TB && t < T) {
#pragma unroll
                for (int i = 0; i < WT; ++i) raw[((size_t)(w0 + i) * D + d) * T + t] = 0.f;
            }
            return;
        }
    }
    {
        float m0[WT], m1[WT], m2[WT], m3[WT];
#pragma unroll
        for (int i = 0; i < WT; ++i) m0[i] = m1[i] = m2[i] = m3[i] = 0.f;
        const int b = b_lo + (int)threadIdx.x;
        int j0 = 0, j1 = 0;
        const int2 *e;
        constexpr int ES = ELL ? 32 : 1;  // stride between a thread's entries
        if constexpr (ELL) {
            // the CTA's tiles are the table's: blockIdx.x = tile, warp = 32 buckets
            const int blk = (d * (int)gridDim.x + (int)blockIdx.x) * (NB / 32) +
                            ((int)threadIdx.x >> 5);
            const int s0 = __ldg(ell_off + blk), s1 = __ldg(ell_off + blk + 1);
            j1 = (s1 - s0) >> 5;
            e = ent + s0 + ((int)threadIdx.x & 31);
        } else {
            if (b >= 0 && b < T) {
                const int32_t *o = off + (size_t)d * (T + 1);
                j0 = __ldg(o + b);
                j1 = __ldg(o + b + 1);
            }
            e = ent + (size_t)d * P;
        }
        if (j0 < j1) {
            const int mask = (1 << fb) - 1;
            const float step = __int_as_float((127 - fb) << 23);  // 2^-fb
            // the entries of the next group load while this group's gathers
            // are in flight (one dependent latency per group, not two)
            int2 qn[FWD_UNR];
#pragma unroll
            for (int u = 0; u < FWD_UNR; ++u)
                qn[u] = j0 + u < j1 ? __ldg(e + (size_t)(j0 + u) * ES) : make_int2(0, -1);
            for (int j = j0; j < j1; j += FWD_UNR) {
                int2 q[FWD_UNR];
                float xv[FWD_UNR][WT];
#pragma unroll
                for (int u = 0; u < FWD_UNR; ++u) q[u] = qn[u];
#pragma unroll
                for (int u = 0; u < FWD_UNR; ++u)
                    load_pixel<WT>(xpm + ((size_t)blockIdx.z * P + max(q[u].y, 0)) * WT, xv[u]);
#pragma unroll
                for (int u = 0; u < FWD_UNR; ++u)
                    qn[u] = j + FWD_UNR + u < j1 ? __ldg(e + (size_t)(j + FWD_UNR + u) * ES)
                                                 : make_int2(0, -1);
#pragma unroll
                for (int u = 0; u < FWD_UNR; ++u) {
                    if (q[u].y < 0) break;
                    const float f = (float)(q[u].x & mask) * step;
                    const float e1 = fmaxf(0.f, fmaf(-f, inv_r, ce1));
                    const float e2 = fmaxf(0.f, fmaf(f, inv_r, -ce2));
#pragma unroll
                    for (int i = 0; i < WT; ++i) {
                        m0[i] += xv[u][i];
                        m1[i] = fmaf(f, xv[u][i], m1[i]);
                        m2[i] = fmaf(e1, xv[u][i], m2[i]);
                        m3[i] = fmaf(e2, xv[u][i], m3[i]);
                    }
                }
            }
        }
#pragma unroll
        for (int i = 0; i < WT; ++i) {
            mom[(0 * WT + i) * NB + threadIdx.x] = m0[i];
            mom[(1 * WT + i) * NB + threadIdx.x] = m1[i];
            mom[(2 * WT + i) * NB + threadIdx.x] = m2[i];
            mom[(3 * WT + i) * NB + threadIdx.x] = m3[i];
        }
    }
    __syncthreads();
    const int ti = threadIdx.x;
    const int t = t0 + ti;
    if (ti >= TB || t >= T) return;
    const int base = t - b_lo;  // local index of bucket t
#pragma unroll
    for (int i = 0; i < WT; ++i) {
        const float *M0 = mom + (0 * WT + i) * NB + base;
        const float *M1 = mom + (1 * WT + i) * NB + base;
        float acc = mom[(2 * WT + i) * NB + base + F] + mom[(3 * WT + i) * NB + base - F - 1];
#pragma unroll
        for (int k = -(F - 1); k <= F; ++k) {
            const float a = 1.f - (float)(k < 0 ? -k : k) * inv_r;
            acc = fmaf(a, M0[-k], acc);
            acc = fmaf(k <= 0 ? -inv_r : inv_r, M1[-k], acc);
        }
        raw[((size_t)(w0 + i) * D + d) * T + t] = acc * (inv_s ? scale * __ldg(inv_s + w0 + i) : scale);
    }
}

template <int WT, int F, typename XT, bool ELL>
inline int das_fwd_launch_t(const Plan &pl, const XT *xpm, float *raw, int W, float scale,
                            const float *inv_s, cudaStream_t st) {
    constexpr int NB = 256, TB = NB - 2 * F - 2;
    dim3 grid(div_up(pl.T, TB), pl.D, W / WT);
    const size_t smem = (size_t)4 * WT * NB * sizeof(float);
    int rc;
    if ((rc = set_smem(k_das_fwd3<WT, F, XT, ELL>, smem)) != MSOT_OK) return rc;
    KLAUNCH(k_das_fwd3<WT, F, XT, ELL><<<grid, NB, smem, st>>>(
        pl.fwd_off, ELL ? pl.fwd_ell : pl.fwd_ent, xpm, raw, pl.P, pl.D, pl.T, W, pl.frac_bits,
        pl.inv_r, pl.ce1, pl.ce2, scale, inv_s, ELL ? pl.fwd_ell_off : nullptr));
    MSOT_LAUNCH_CHECK();
    return MSOT_OK;
}

// k_das_fwd3 over the plan's instance tile wt and radius F, xpm of type XT
template <typename XT>
int das_fwd_run(const Plan &pl, const void *xpm_v, float *raw, int W, float scale,
                const float *inv_s, bool ell, int wt, cudaStream_t st) {
    const XT *xpm = reinterpret_cast<const XT *>(xpm_v);
    auto by_f = [&](auto wt_c) -> int {
        constexpr int WTc = decltype(wt_c)::value;
        auto go = [&](auto f_c) -> int {
            constexpr int Fc = decltype(f_c)::value;
            return ell ? das_fwd_launch_t<WTc, Fc, XT, true>(pl, xpm, raw, W, scale, inv_s, st)
                       : das_fwd_launch_t<WTc, Fc, XT, false>(pl, xpm, raw, W, scale, inv_s, st);
        };
        switch (pl.F) {
            case 0: return go(std::integral_constant<int, 0>{});
            case 1: return go(std::integral_constant<int, 1>{});
            case 2: return go(std::integral_constant<int, 2>{});
            case 3: return go(std::integral_constant<int, 3>{});
            case 4: return go(std::integral_constant<int, 4>{});
            case 5: return go(std::integral_constant<int, 5>{});
            case 6: return go(std::integral_constant<int, 6>{});
            case 7: return go(std::integral_constant<int, 7>{});
            case 8: return go(std::integral_constant<int, 8>{});
            default:
                set_error("DAS forward: interpolation radius %g above 9 samples is not supported",
                          pl.radius);
                return MSOT_EINVAL;
        }
    };
    switch (wt) {
        case 16: return by_f(std::integral_constant<int, 16>{});
        case 8: return by_f(std::integral_constant<int, 8>{});
        case 4: return by_f(std::integral_constant<int, 4>{});
        case 2: return by_f(std::integral_constant<int, 2>{});
        default: return by_f(std::integral_constant<int, 1>{});
    }
}

}  // namespace msot
