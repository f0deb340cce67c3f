// das_fwd_staged.cu -- the DAS interpolation forward operator
// (forwardDelayAndSumMex.cpp:72-103) with each CTA's image values staged in
// shared memory.
//
// The bucket decomposition of operator.cu is kept: for tau = b + f the taps
// b-F+1 .. b+F of a (pixel, detector) pair are linear in f and only taps b-F
// and b+F+1 need the clamp, so a bucket b = floor(tau) reduces four moments
// (sum x, sum f x, sum e1 x, sum e2 x) over its pixels and each output sample
// is a (2F+2)-tap filter over the moments.  What changes is where the image
// values come from.  k_das_fwd3 gathers x[p][w] from L2 for every (pixel,
// detector) pair, P*D*W*4 bytes per apply.  Here a CTA owns a time tile of
// TT output samples for a group of G adjacent detectors.  The pixels whose
// travel time to any detector of the group falls in the tile's buckets form
// a union U, listed once per CTA at plan creation; the CTA copies x[U][w]
// into shared memory once (16-byte cp.async) and every detector of the group
// reads it there.  Adjacent detectors see nearly the same band of pixels, so
// the union is little larger than one detector's band and the L2 traffic
// drops by about G.  Each thread reduces the moments of one (detector,
// bucket) from shared memory, two instances per packed FP32 instruction
// (fma.rn.f32x2); the filter runs four outputs per thread from one register
// window of moments, and the output tile leaves through shared memory.
//
// Per CTA the plan stores (concatenated):
//   st_info  {u_off, nU, e_off, n_ent}
//   st_u     the union's pixel indices, ascending
//   st_off   [G][NBK + 1] offsets of the CTA's entries per (detector, bucket)
//   st_ent   entries (tau fraction << ib) | index in U, bucket-sorted, pixels
//            ascending within a bucket (the order of k_das_fwd3's walk, so the
//            two kernels give identical sums)
// with NBK = TT + 2F + 1 buckets spanning [k TT - F - 1, k TT + TT + F).  TT
// and G are powers of two.  The entries and offsets are read through L1.
#include <algorithm>
#include <atomic>
#include <vector>

#include "common.cuh"
#include "ptx.cuh"

namespace msot {

// image values of entry q (index in the union in its low bits) as instance
// pairs
template <int WT>
__device__ __forceinline__ void load_x(const float *s_x, uint32_t q, uint32_t umask,
                                       float2 (&xv)[WT >= 2 ? WT / 2 : 1]) {
    const float *xp = s_x + (size_t)(q & umask) * WT;
    if constexpr (WT >= 4) {
#pragma unroll
        for (int c = 0; c < WT / 4; ++c) {
            const float4 v = *reinterpret_cast<const float4 *>(xp + 4 * c);
            xv[2 * c] = make_float2(v.x, v.y);
            xv[2 * c + 1] = make_float2(v.z, v.w);
        }
    } else if constexpr (WT == 2) {
        xv[0] = *reinterpret_cast<const float2 *>(xp);
    } else {
        xv[0] = make_float2(xp[0], 0.f);
    }
}

// the four bucket moments of one entry: sum x, sum f x, sum e1 x, sum e2 x,
// instance pairs through the packed FP32 unit (fma.rn.f32x2)
template <int WT>
__device__ __forceinline__ void accumulate(float2 (&acc)[4][WT >= 2 ? WT / 2 : 1], uint32_t q,
                                           const float2 (&xv)[WT >= 2 ? WT / 2 : 1], int ib,
                                           float step, float inv_r, float ce1, float ce2) {
    constexpr int WP = WT >= 2 ? WT / 2 : 1;
    const float f = (float)(q >> ib) * step;
    const float e1 = fmaxf(0.f, fmaf(-f, inv_r, ce1));
    const float e2 = fmaxf(0.f, fmaf(f, inv_r, -ce2));
    if constexpr (WT >= 2) {
        const float2 f2 = make_float2(f, f), e12 = make_float2(e1, e1), e22 = make_float2(e2, e2);
#pragma unroll
        for (int w = 0; w < WP; ++w) {
            acc[0][w] = fadd2(acc[0][w], xv[w]);
            acc[1][w] = ffma2(f2, xv[w], acc[1][w]);
            acc[2][w] = ffma2(e12, xv[w], acc[2][w]);
            acc[3][w] = ffma2(e22, xv[w], acc[3][w]);
        }
    } else {
        acc[0][0].x += xv[0].x;
        acc[1][0].x = fmaf(f, xv[0].x, acc[1][0].x);
        acc[2][0].x = fmaf(e1, xv[0].x, acc[2][0].x);
        acc[3][0].x = fmaf(e2, xv[0].x, acc[3][0].x);
    }
}

// TT = 1 << lg_tt output samples and G = 1 << lg_g detectors per CTA; the
// shared memory holds the union's image values [nU][WT] (x_words floats,
// later the moments) and the output tile [G][WT][TT + 1].
template <int WT, int F>
__global__ void __launch_bounds__(384, WT >= 16 ? 1 : 2) k_das_fwd_st(
    const int4 *__restrict__ info, const int32_t *__restrict__ ulist,
    const int32_t *__restrict__ offs, const uint32_t *__restrict__ ents,
    const float *__restrict__ xt, float *__restrict__ raw, int P, int D, int T, int lg_g,
    int lg_tt, int n_tiles, int off_stride, int x_words, int ib, int fb, float inv_r, float ce1,
    float ce2, float scale) {
    constexpr int WP = WT >= 2 ? WT / 2 : 1;  // instance pairs (WT = 1: one scalar)
    const int G = 1 << lg_g, TT = 1 << lg_tt;
    const int NBK = TT + 2 * F + 1;
    const int NBKp = NBK | 1;  // odd row stride of the moments: conflict-free 8-byte loads
    extern __shared__ __align__(16) float st_smem[];
    float *s_x = st_smem;                        // [nU][WT], then the moments
    float *s_out = st_smem + x_words;            // [G][WT][TT + 1]
    const int cta = blockIdx.x, g = cta / n_tiles, k = cta - g * n_tiles;
    const int d0 = g << lg_g, t0 = k << lg_tt, w0 = blockIdx.y * WT;
    const int tid = threadIdx.x, nthr = blockDim.x;
    const int lane = tid & 31, warp = tid >> 5, nwarp = nthr >> 5;
    const int4 inf = __ldg(info + cta);  // u_off, nU, e_off, n_ent
    if (inf.w == 0) {
        // no pixel of the group falls in the tile: zero rows, lanes along t
        for (int rw = warp; rw < G * WT; rw += nwarp) {
            const int d = d0 + rw / WT, w = rw % WT;
            if (d >= D) continue;
            float *row = raw + ((size_t)(w0 + w) * D + d) * T;
            for (int tl = lane; tl < TT; tl += 32)
                if (t0 + tl < T) row[t0 + tl] = 0.f;
        }
        return;
    }
    // the union's image values, WT instances per pixel ([W/WT][P][WT] layout)
    {
        const float *xsrc = xt + (size_t)blockIdx.y * P * WT;
        const int32_t *U = ulist + inf.x;
        for (int i = tid; i < inf.y; i += nthr) {
            const float *src = xsrc + (size_t)__ldg(U + i) * WT;
            const uint32_t dst = smem_u32(s_x + (size_t)i * WT);
            if constexpr (WT >= 4) {
#pragma unroll
                for (int c = 0; c < WT / 4; ++c) cp_async16(dst + 16 * c, src + 4 * c);
            } else if constexpr (WT == 2) {
                cp_async8(dst, src);
            } else {
                cp_async4(dst, src);
            }
        }
    }
    // this thread's (detector, bucket) and the bounds of its entries (read
    // through L1 while the image values are in flight)
    const int j = tid / NBK, i = tid - j * NBK;
    const bool active = j < G;
    int lo = 0, hi = 0;
    if (active) {
        const int32_t *o = offs + (size_t)cta * off_stride + j * (NBK + 1) + i;
        lo = __ldg(o);
        hi = __ldg(o + 1);
    }
    cp_async_wait_all();
    __syncthreads();

    // phase 1: the thread's bucket moments, two entries per step
    const uint32_t umask = (1u << ib) - 1u;
    const float step = __int_as_float((127 - fb) << 23);  // 2^-fb
    float2 acc[4][WP];
#pragma unroll
    for (int m = 0; m < 4; ++m)
#pragma unroll
        for (int w = 0; w < WP; ++w) acc[m][w] = make_float2(0.f, 0.f);
    {
        const uint32_t *E = ents + inf.z;
        int e = lo;
        for (; e + 1 < hi; e += 2) {
            const uint32_t qa = __ldg(E + e), qb = __ldg(E + e + 1);
            float2 xa[WP], xb[WP];
            load_x<WT>(s_x, qa, umask, xa);
            load_x<WT>(s_x, qb, umask, xb);
            accumulate<WT>(acc, qa, xa, ib, step, inv_r, ce1, ce2);
            accumulate<WT>(acc, qb, xb, ib, step, inv_r, ce1, ce2);
        }
        if (e < hi) {
            const uint32_t qa = __ldg(E + e);
            float2 xa[WP];
            load_x<WT>(s_x, qa, umask, xa);
            accumulate<WT>(acc, qa, xa, ib, step, inv_r, ce1, ce2);
        }
    }
    __syncthreads();  // every thread is done with the staged image values
    float2 *M2v = reinterpret_cast<float2 *>(s_x);  // moments [G][4][WP][NBKp] (pairs)
    float *M1s = s_x;                              // WT = 1: [G][4][NBKp]
    if (active) {
#pragma unroll
        for (int m = 0; m < 4; ++m)
#pragma unroll
            for (int w = 0; w < WP; ++w) {
                if constexpr (WT >= 2)
                    M2v[((j * 4 + m) * WP + w) * NBKp + i] = acc[m][w];
                else
                    M1s[(j * 4 + m) * NBKp + i] = acc[m][0].x;
            }
    }
    __syncthreads();

    // phase 2: output t (local tl) reads buckets t - F - 1 .. t + F, i.e.
    // local indices tl .. tl + 2F + 1.  A thread filters FB = 4 consecutive
    // outputs of one (detector, instance pair) from one window of 2F + 3
    // moments: outputs tl0 + u read M0 / M1 at tl0 + 1 + (u + F - k).
    // Consecutive threads take consecutive (detector, pair) rows (odd row
    // stride: distinct banks); the tile goes through shared memory so that
    // the global stores run along t.
    constexpr int FB = 4;
    const int TTp = TT + 1;
    const int lg_nrow = lg_g + (WP == 8 ? 3 : WP == 4 ? 2 : WP == 2 ? 1 : 0);
    const int n_items = (G * WP) * (TT / FB);
    for (int it = tid; it < n_items; it += nthr) {
        const int r = it & ((1 << lg_nrow) - 1), tb = it >> lg_nrow;
        const int wp = r % WP, jj = r / WP;
        const int tl0 = tb * FB;
        float2 v0[2 * F + 3], v1[2 * F + 3], a2[FB], a3[FB];
        if constexpr (WT >= 2) {
            const float2 *B0 = M2v + ((jj * 4 + 0) * WP + wp) * NBKp + tl0 + 1;
            const float2 *B1 = M2v + ((jj * 4 + 1) * WP + wp) * NBKp + tl0 + 1;
            const float2 *B2 = M2v + ((jj * 4 + 2) * WP + wp) * NBKp + tl0 + 2 * F + 1;
            const float2 *B3 = M2v + ((jj * 4 + 3) * WP + wp) * NBKp + tl0;
#pragma unroll
            for (int c = 0; c < 2 * F + 3; ++c) v0[c] = B0[c], v1[c] = B1[c];
#pragma unroll
            for (int u = 0; u < FB; ++u) a2[u] = B2[u], a3[u] = B3[u];
        } else {
            const float *B0 = M1s + (jj * 4 + 0) * NBKp + tl0 + 1;
            const float *B1 = M1s + (jj * 4 + 1) * NBKp + tl0 + 1;
            const float *B2 = M1s + (jj * 4 + 2) * NBKp + tl0 + 2 * F + 1;
            const float *B3 = M1s + (jj * 4 + 3) * NBKp + tl0;
#pragma unroll
            for (int c = 0; c < 2 * F + 3; ++c)
                v0[c] = make_float2(B0[c], 0.f), v1[c] = make_float2(B1[c], 0.f);
#pragma unroll
            for (int u = 0; u < FB; ++u)
                a2[u] = make_float2(B2[u], 0.f), a3[u] = make_float2(B3[u], 0.f);
        }
        const float2 pr = make_float2(inv_r, inv_r), nr = make_float2(-inv_r, -inv_r);
        float *o0 = s_out + (jj * WT + (WT >= 2 ? 2 * wp : 0)) * TTp + tl0;
#pragma unroll
        for (int u = 0; u < FB; ++u) {
            float2 y = fadd2(a2[u], a3[u]);
#pragma unroll
            for (int kk = -(F - 1); kk <= F; ++kk) {
                const float a = 1.f - (float)(kk < 0 ? -kk : kk) * inv_r;
                y = ffma2(make_float2(a, a), v0[u + F - kk], y);
                y = ffma2(kk <= 0 ? nr : pr, v1[u + F - kk], y);
            }
            o0[u] = y.x * scale;
            if constexpr (WT >= 2) o0[TTp + u] = y.y * scale;
        }
    }
    __syncthreads();
    // rows (detector, instance) of the tile, lanes along t
    for (int rw = warp; rw < G * WT; rw += nwarp) {
        const int d = d0 + rw / WT, w = rw % WT;
        if (d >= D) continue;
        float *row = raw + ((size_t)(w0 + w) * D + d) * T;
        for (int tl = lane; tl < TT; tl += 32)
            if (t0 + tl < T) row[t0 + tl] = s_out[rw * TTp + tl];
    }
}

// ---------------------------------------------------------------------------
// host: table construction at plan creation
// ---------------------------------------------------------------------------
// floats of the image-value / moment region at an instance tile of wt
int st_x_words(const Plan &p, int wt) {
    const int NBKp = (p.st_tt + 2 * p.F + 1) | 1;
    const size_t xs = std::max((size_t)p.st_umax * wt, (size_t)p.st_g * 4 * wt * NBKp);
    return (int)((xs + 3) & ~(size_t)3);
}

static inline int floor_div(int a, int b) { return a >= 0 ? a / b : -((-a + b - 1) / b); }

// tiles k whose bucket range [k TT - F - 1, k TT + TT + F) holds bucket b
//   k TT - F - 1 <= b      <=>  k <= floor((b + F + 1) / TT)
//   b <= k TT + TT + F - 1  <=>  k >= floor((b - TT - F) / TT) + 1
static inline void st_tile_range(int b, int TT, int F, int n_tiles, int &k0, int &k1) {
    k0 = std::max(0, floor_div(b - TT - F, TT) + 1);
    k1 = std::min(n_tiles - 1, floor_div(b + F + 1, TT));
}

size_t st_smem_bytes(const Plan &p, int wt) {
    return ((size_t)st_x_words(p, wt) + (size_t)p.st_g * wt * (p.st_tt + 1)) * 4;
}

namespace {
struct StScan {
    long long cost = 0;
    int umax = 0, emax = 0;
};

StScan st_scan(const Plan &p, const int32_t *tfx, int TT, int G, int sample_step) {
    const int F = p.F, fb = p.frac_bits;
    const int n_tiles = div_up(p.T, TT), n_groups = div_up(p.D, G);
    std::vector<int> stamp(n_tiles), nU(n_tiles), nE(n_tiles);
    StScan s;
    int sampled = 0;
    for (int g = 0; g < n_groups; g += sample_step) {
        ++sampled;
        std::fill(stamp.begin(), stamp.end(), -1);
        std::fill(nU.begin(), nU.end(), 0);
        std::fill(nE.begin(), nE.end(), 0);
        const int d0 = g * G, nd = std::min(G, p.D - d0);
        for (int q = 0; q < p.P; ++q)
            for (int j = 0; j < nd; ++j) {
                const int b = tfx[(size_t)(d0 + j) * p.P + q] >> fb;
                int k0, k1;
                st_tile_range(b, TT, F, n_tiles, k0, k1);
                for (int k = k0; k <= k1; ++k) {
                    ++nE[k];
                    if (stamp[k] != q) {
                        stamp[k] = q;
                        ++nU[k];
                    }
                }
            }
        for (int k = 0; k < n_tiles; ++k) {
            s.umax = std::max(s.umax, nU[k]);
            s.emax = std::max(s.emax, nE[k]);
            // L2 bytes of one instance tile: 32 B per staged pixel (8
            // instances), 4 B per entry plus its shared-memory work
            s.cost += 32LL * nU[k] + 24LL * nE[k];
        }
    }
    s.cost = s.cost * n_groups / std::max(1, sampled);
    return s;
}
}  // namespace

// Pure host part of the table construction (also compiled into a CPU check):
// picks the tile shape for a device with dev_smem bytes of opt-in shared
// memory per CTA and fills t; t.tt == 0 when no shape fits.
std::atomic<int> g_st_force_tt{0}, g_st_force_g{0};

int build_fwd_staged_host(const Plan &p, const int32_t *tfx, const int32_t *foff,
                          const int2 *fent, int dev_smem, StTables &t) {
    t = StTables();
    if (p.S || p.F > 8) return MSOT_OK;
    const int fb = p.frac_bits, ib = 32 - fb;
    if (ib < 8) return MSOT_OK;  // too few index bits: the plan keeps k_das_fwd3 only
    // candidates: time tile x detector group; the cheapest that fits two CTAs
    // per SM (about 110 KB each), else one; msot_tune_set can force either
    std::vector<int> tts = {64, 32, 16, 8}, gs = {16, 8, 4, 2};
    if (g_st_force_tt.load()) tts = {g_st_force_tt.load()};
    if (g_st_force_g.load()) gs = {g_st_force_g.load()};
    // exact counts for plans up to 32 M (pixel, detector) pairs, a sample of
    // the detector groups (with a margin on the maxima) above
    const bool sample = (long long)p.P * p.D > (32LL << 20);
    const int n_groups_8 = div_up(p.D, 8);
    const int step8 = sample ? std::max(1, n_groups_8 / 32) : 1;
    int best_tt = 0, best_g = 0;
    // three CTAs per SM (228 KB less 1 KB per CTA), else two, else one;
    // shapes of at least two warps first
    const size_t budgets[] = {(size_t)75 * 1024, (size_t)113 * 1024,
                              (size_t)std::max(0, dev_smem - 1024)};
    for (int min_threads : {64, 1})
        for (size_t budget : budgets) {
            if (best_tt) break;
            long long best_cost = -1;
            for (int TT : tts)
                for (int G : gs) {
                    const int NBK = TT + 2 * p.F + 1;
                    if (G * NBK > 384 || G * NBK < min_threads || G > p.D) continue;
                    const StScan s = st_scan(p, tfx, TT, G, std::max(1, step8 * 8 / G));
                    const size_t umax = sample ? (size_t)s.umax * 5 / 4 : (size_t)s.umax;
                    const size_t emax = sample ? (size_t)s.emax * 5 / 4 + 64 : (size_t)s.emax;
                    if (umax >= ((size_t)1 << ib)) continue;
                    (void)emax;
                    const size_t xs = std::max(umax * 8, (size_t)G * 4 * 8 * (NBK | 1));
                    const size_t need = (xs + (size_t)G * 8 * (TT + 1)) * 4;
                    if (need > budget) continue;
                    if (best_cost < 0 || s.cost < best_cost) {
                        best_cost = s.cost;
                        best_tt = TT;
                        best_g = G;
                    }
                }
        }
    if (!best_tt) return MSOT_OK;

    const int TT = best_tt, G = best_g, F = p.F, NBK = TT + 2 * F + 1;
    const int n_tiles = div_up(p.T, TT), n_groups = div_up(p.D, G);
    const size_t n_cta = (size_t)n_tiles * n_groups;
    const int off_stride = (G * (NBK + 1) + 3) & ~3;
    t.info.resize(n_cta);
    t.offs.assign(n_cta * off_stride, 0);
    t.ulist.reserve((size_t)p.P * p.D / 4);
    t.ent.reserve((size_t)p.P * p.D * (NBK + TT - 1) / TT);
    std::vector<std::vector<int32_t>> Ul(n_tiles);
    std::vector<int> stamp(n_tiles);
    std::vector<int32_t> loc(p.P, -1);
    const uint32_t fmask = (1u << fb) - 1u;
    int umax = 0, emax = 0;
    for (int g = 0; g < n_groups; ++g) {
        for (auto &u : Ul) u.clear();
        std::fill(stamp.begin(), stamp.end(), -1);
        const int d0 = g * G, nd = std::min(G, p.D - d0);
        for (int q = 0; q < p.P; ++q)
            for (int j = 0; j < nd; ++j) {
                const int b = tfx[(size_t)(d0 + j) * p.P + q] >> fb;
                int k0, k1;
                st_tile_range(b, TT, F, n_tiles, k0, k1);
                for (int k = k0; k <= k1; ++k)
                    if (stamp[k] != q) {
                        stamp[k] = q;
                        Ul[k].push_back(q);
                    }
            }
        for (int k = 0; k < n_tiles; ++k) {
            const size_t cta = (size_t)g * n_tiles + k;
            if (t.ulist.size() > (size_t)INT32_MAX - p.P || t.ent.size() > (size_t)INT32_MAX / 2) {
                set_error("plan: staged forward tables exceed 2^31 entries");
                return MSOT_ERANGE;
            }
            const int u_off = (int)t.ulist.size(), e_off = (int)t.ent.size();
            for (size_t i = 0; i < Ul[k].size(); ++i) loc[Ul[k][i]] = (int32_t)i;
            t.ulist.insert(t.ulist.end(), Ul[k].begin(), Ul[k].end());
            int32_t *o = t.offs.data() + cta * off_stride;
            int cnt = 0;
            for (int j = 0; j < G; ++j) {
                const int d = d0 + j;
                for (int i = 0; i < NBK; ++i) {
                    o[j * (NBK + 1) + i] = cnt;
                    const int b = k * TT - F - 1 + i;
                    if (j >= nd || b < 0 || b >= p.T) continue;
                    const int32_t *fo = foff + (size_t)d * (p.T + 1);
                    const int2 *fe = fent + (size_t)d * p.P;
                    for (int e = fo[b]; e < fo[b + 1]; ++e) {
                        t.ent.push_back(((uint32_t)fe[e].x & fmask) << ib |
                                        (uint32_t)loc[fe[e].y]);
                        ++cnt;
                    }
                }
                o[j * (NBK + 1) + NBK] = cnt;
            }
            while (t.ent.size() & 3) t.ent.push_back(0u);  // 16-byte aligned segments
            t.info[cta] = make_int4(u_off, (int)Ul[k].size(), e_off, cnt);
            umax = std::max(umax, (int)Ul[k].size());
            emax = std::max(emax, cnt);
        }
    }
    // the union must be well below one gather per (pixel, detector) pair for
    // the staging to pay (k_das_fwd3 gathers every pair from L2)
    if (t.ulist.size() * 2 > (size_t)p.P * p.D) {
        t = StTables();
        return MSOT_OK;
    }
    if (t.ulist.empty()) t.ulist.push_back(0);
    t.tt = TT;
    t.g = G;
    t.ntiles = n_tiles;
    t.ngroups = n_groups;
    t.ib = ib;
    t.umax = umax;
    t.ent_cap = (emax + 3) & ~3;
    t.off_stride = off_stride;
    t.threads = std::min(384, (G * NBK + 31) / 32 * 32);
    return MSOT_OK;
}

int build_fwd_staged(Plan &p, const int32_t *tfx, const int32_t *foff, const int2 *fent,
                     size_t &bytes) {
    int dev_smem = 0;
    MSOT_CUDA_TRY(cudaDeviceGetAttribute(&dev_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin,
                                         p.device));
    StTables t;
    int rc = build_fwd_staged_host(p, tfx, foff, fent, dev_smem, t);
    if (rc != MSOT_OK || !t.tt) return rc;
    p.st_tt = t.tt;
    p.st_g = t.g;
    p.st_ntiles = t.ntiles;
    p.st_ngroups = t.ngroups;
    p.st_ib = t.ib;
    p.st_umax = t.umax;
    p.st_ent_cap = t.ent_cap;
    p.st_off_stride = t.off_stride;
    p.st_threads = t.threads;
    if (st_smem_bytes(p, 1) > (size_t)dev_smem) {  // even one instance per CTA does not fit
        p.st_tt = 0;
        return MSOT_OK;
    }
    auto up = [&](auto **dst, const auto &v) -> int {
        using T = typename std::remove_reference_t<decltype(v)>::value_type;
        cudaError_t e = cudaMalloc((void **)dst, v.size() * sizeof(T));
        if (e != cudaSuccess) {
            set_error("cudaMalloc(%zu): %s", v.size() * sizeof(T), cudaGetErrorString(e));
            return MSOT_ENOMEM;
        }
        bytes += v.size() * sizeof(T);
        MSOT_CUDA_TRY(cudaMemcpy(*dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
        return MSOT_OK;
    };
    if ((rc = up(&p.st_info, t.info)) || (rc = up(&p.st_u, t.ulist)) ||
        (rc = up(&p.st_off, t.offs)) || (rc = up(&p.st_ent, t.ent)))
        return rc;
    return MSOT_OK;
}

// ---------------------------------------------------------------------------
// host: launch
// ---------------------------------------------------------------------------
static int ilog2(int v) {
    int l = 0;
    while ((1 << (l + 1)) <= v) ++l;
    return l;
}

template <class K>
static int st_set_smem(K kern, size_t bytes) {
    if (bytes > 48 * 1024) {
        cudaError_t e = raise_max_dynamic_smem((const void *)kern, bytes);
        if (e != cudaSuccess) {
            set_error("cudaFuncSetAttribute(smem=%zu): %s", bytes, cudaGetErrorString(e));
            return MSOT_ECUDA;
        }
    }
    return MSOT_OK;
}

template <int WT, int F>
static int st_launch(const Plan &p, const float *xt, float *raw, int W, float scale,
                     cudaStream_t st) {
    const size_t smem = st_smem_bytes(p, WT);
    int rc;
    if ((rc = st_set_smem(k_das_fwd_st<WT, F>, smem)) != MSOT_OK) return rc;
    const dim3 grid((unsigned)(p.st_ntiles * p.st_ngroups), (unsigned)(W / WT));
    KLAUNCH(k_das_fwd_st<WT, F><<<grid, p.st_threads, smem, st>>>(
        p.st_info, p.st_u, p.st_off, p.st_ent, xt, raw, p.P, p.D, p.T, ilog2(p.st_g),
        ilog2(p.st_tt), p.st_ntiles, p.st_off_stride, st_x_words(p, WT), p.st_ib, p.frac_bits,
        p.inv_r, p.ce1, p.ce2, scale));
    MSOT_LAUNCH_CHECK();
    return MSOT_OK;
}

template <int WT>
static int st_launch_f(const Plan &p, const float *xt, float *raw, int W, float scale,
                       cudaStream_t st) {
    switch (p.F) {
        case 0: return st_launch<WT, 0>(p, xt, raw, W, scale, st);
        case 1: return st_launch<WT, 1>(p, xt, raw, W, scale, st);
        case 2: return st_launch<WT, 2>(p, xt, raw, W, scale, st);
        case 3: return st_launch<WT, 3>(p, xt, raw, W, scale, st);
        case 4: return st_launch<WT, 4>(p, xt, raw, W, scale, st);
        case 5: return st_launch<WT, 5>(p, xt, raw, W, scale, st);
        case 6: return st_launch<WT, 6>(p, xt, raw, W, scale, st);
        case 7: return st_launch<WT, 7>(p, xt, raw, W, scale, st);
        case 8: return st_launch<WT, 8>(p, xt, raw, W, scale, st);
        default:
            set_error("DAS forward: interpolation radius %g above 9 samples is not supported",
                      p.radius);
            return MSOT_EINVAL;
    }
}

bool fwd_staged_fits(const Plan &p, int wt) {
    if (!p.st_tt || !p.st_info) return false;
    int dev_smem = 0;
    if (cudaDeviceGetAttribute(&dev_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, p.device) !=
        cudaSuccess)
        return false;
    return st_smem_bytes(p, wt) <= (size_t)dev_smem;
}

int launch_das_forward_staged(const Plan &p, const float *xt, float *raw, int W, int wt,
                              float scale, cudaStream_t st) {
    switch (wt) {
        case 16: return st_launch_f<16>(p, xt, raw, W, scale, st);
        case 8: return st_launch_f<8>(p, xt, raw, W, scale, st);
        case 4: return st_launch_f<4>(p, xt, raw, W, scale, st);
        case 2: return st_launch_f<2>(p, xt, raw, W, scale, st);
        default: return st_launch_f<1>(p, xt, raw, W, scale, st);
    }
}

}  // namespace msot
