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
// drops by about G.
//
// Per CTA the plan stores (concatenated, each CTA's part 16-byte aligned):
//   st_info  {u_off, nU, e_off, n_ent}
//   st_u     the union's pixel indices, ascending
//   st_off   [G][NBK + 1] offsets of the CTA's entries per (detector, bucket)
//   st_ent   entries (tau fraction << ib) | index in U, bucket-sorted, pixels
//            ascending within a bucket (the order of k_das_fwd3's walk, so the
//            two kernels give identical sums)
// with NBK = TT + 2F + 1 buckets spanning [k TT - F - 1, k TT + TT + F).  The
// entries and offsets arrive by two bulk copies (TMA engine) on one mbarrier
// while the image values are in flight.
#include <algorithm>
#include <atomic>
#include <vector>

#include "common.cuh"
#include "ptx.cuh"

namespace msot {

__device__ int g_fwd_st_err = 0;  // set by a CTA whose bulk-copy wait timed out

template <int WT, int F>
__global__ void __launch_bounds__(384, 2) k_das_fwd_st(
    const int4 *__restrict__ info, const int32_t *__restrict__ ulist,
    const int32_t *__restrict__ offs, const uint32_t *__restrict__ ents,
    const float *__restrict__ xt, float *__restrict__ raw, int P, int D, int T, int G, int TT,
    int n_tiles, int off_stride, int ent_cap, int ib, int fb, float inv_r, float ce1, float ce2,
    float scale) {
    const int NBK = TT + 2 * F + 1;
    const int NBKp = NBK | 1;  // odd row stride of the moments: conflict-free 8-byte loads
    extern __shared__ __align__(16) unsigned char st_smem[];
    uint32_t *s_ent = reinterpret_cast<uint32_t *>(st_smem);            // [ent_cap]
    int32_t *s_off = reinterpret_cast<int32_t *>(s_ent + ent_cap);        // [off_stride]
    uint64_t *s_bar = reinterpret_cast<uint64_t *>(s_off + off_stride);   // mbarrier
    int *s_flag = reinterpret_cast<int *>(s_bar + 1);                     // wait failed
    float *s_x = reinterpret_cast<float *>(s_bar + 2);  // [nU][WT], then the moments
    const int cta = blockIdx.x, g = cta / n_tiles, k = cta - g * n_tiles;
    const int d0 = g * G, t0 = k * TT, w0 = blockIdx.y * WT;
    const int tid = threadIdx.x, nthr = blockDim.x;
    const int4 inf = __ldg(info + cta);  // u_off, nU, e_off, n_ent
    if (inf.w == 0) {
        // no pixel of the group falls in the tile: its outputs are zero
        for (int o = tid; o < G * WT * TT; o += nthr) {
            const int tl = o % TT, r = o / TT, w = r % WT, j = r / WT;
            const int d = d0 + j, t = t0 + tl;
            if (d < D && t < T) raw[((size_t)(w0 + w) * D + d) * T + t] = 0.f;
        }
        return;
    }
    const uint32_t bar = smem_u32(s_bar);
    if (tid == 0) {
        s_flag[0] = 0;
        mbar_init(bar, 1);
        mbar_init_fence();
    }
    __syncthreads();
    if (tid == 0) {
        const uint32_t ent_bytes = (uint32_t)((inf.w + 3) & ~3) * 4u;
        const uint32_t off_bytes = (uint32_t)off_stride * 4u;
        mbar_arrive_expect_tx(bar, ent_bytes + off_bytes);
        bulk_g2s(smem_u32(s_ent), ents + inf.z, ent_bytes, bar);
        bulk_g2s(smem_u32(s_off), offs + (size_t)cta * off_stride, off_bytes, bar);
    }
    // the union's image values, WT instances per pixel ([W/WT][P][WT] layout)
    {
        const float *xsrc = xt + (size_t)blockIdx.y * P * WT;
        const int32_t *U = ulist + inf.x;
        for (int i = tid; i < inf.y; i += nthr) {
            const float *src = xsrc + (size_t)__ldg(U + i) * WT;
            const uint32_t dst = smem_u32(s_x + (size_t)i * WT);
            if constexpr (WT == 8) {
                // the two 16-byte halves swap places on every other group of
                // four pixels, so that the 8-lane phases of a 16-byte load
                // over random pixels spread over all eight bank groups
                const int sw = (i >> 2) & 1;
                cp_async16(dst + 16 * sw, src);
                cp_async16(dst + 16 * (sw ^ 1), src + 4);
            } else if constexpr (WT == 4) {
                cp_async16(dst, src);
            } else if constexpr (WT == 2) {
                cp_async8(dst, src);
            } else {
                cp_async4(dst, src);
            }
        }
    }
    cp_async_wait_all();
    if (!mbar_wait_bounded(bar, 0)) s_flag[0] = 1;
    __syncthreads();
    if (s_flag[0]) {
        // the bulk copies did not complete within the bound: report, wait
        // once more (bounded) for the copies still landing here, skip the tile
        if (tid == 0) {
            atomicExch(&g_fwd_st_err, 1);
            mbar_wait_bounded(bar, 0);
        }
        __syncthreads();
        return;
    }

    // phase 1: each (detector, bucket) pair reduces its four moments; the
    // instances go in pairs through the packed FP32 unit (fma.rn.f32x2)
    constexpr int WP = WT >= 2 ? WT / 2 : 1;  // instance pairs (WT = 1: one scalar)
    const uint32_t umask = (1u << ib) - 1u;
    const float step = __int_as_float((127 - fb) << 23);  // 2^-fb
    float2 *M2v = reinterpret_cast<float2 *>(s_x);  // moments [G][4][WP][NBKp] (pairs)
    float *M1s = s_x;                              // WT = 1: [G][4][NBKp]
    const int npair = G * NBK;
    // a thread keeps the moments of its pair in registers until every thread
    // has stopped reading the staged image values (threads >= npair)
    constexpr int MAXP = 1;
    float2 acc[MAXP][4][WP];
    int pj[MAXP], pi[MAXP];
#pragma unroll
    for (int u = 0; u < MAXP; ++u) {
        const int pr = tid + u * nthr;
        pj[u] = pr < npair ? pr / NBK : -1;
        pi[u] = pr < npair ? pr - pj[u] * NBK : 0;
#pragma unroll
        for (int m = 0; m < 4; ++m)
#pragma unroll
            for (int w = 0; w < WP; ++w) acc[u][m][w] = make_float2(0.f, 0.f);
        if (pj[u] < 0) continue;
        const int lo = s_off[pj[u] * (NBK + 1) + pi[u]], hi = s_off[pj[u] * (NBK + 1) + pi[u] + 1];
        for (int e = lo; e < hi; ++e) {
            const uint32_t q = s_ent[e];
            const float f = (float)(q >> ib) * step;
            const float *xp = s_x + (size_t)(q & umask) * WT;
            const float e1 = fmaxf(0.f, fmaf(-f, inv_r, ce1));
            const float e2 = fmaxf(0.f, fmaf(f, inv_r, -ce2));
            if constexpr (WT >= 2) {
                float2 xv[WP];
                if constexpr (WT == 8) {
                    const int sw = (int)((q & umask) >> 2) & 1;
                    const float4 v = *reinterpret_cast<const float4 *>(xp + 4 * sw);
                    const float4 v2 = *reinterpret_cast<const float4 *>(xp + 4 * (sw ^ 1));
                    xv[0] = make_float2(v.x, v.y);
                    xv[1] = make_float2(v.z, v.w);
                    xv[2] = make_float2(v2.x, v2.y);
                    xv[3] = make_float2(v2.z, v2.w);
                } else if constexpr (WT == 4) {
                    const float4 v = *reinterpret_cast<const float4 *>(xp);
                    xv[0] = make_float2(v.x, v.y);
                    xv[1] = make_float2(v.z, v.w);
                } else {
                    xv[0] = *reinterpret_cast<const float2 *>(xp);
                }
                const float2 f2 = make_float2(f, f), e12 = make_float2(e1, e1),
                             e22 = make_float2(e2, e2);
#pragma unroll
                for (int w = 0; w < WP; ++w) {
                    acc[u][0][w] = fadd2(acc[u][0][w], xv[w]);
                    acc[u][1][w] = ffma2(f2, xv[w], acc[u][1][w]);
                    acc[u][2][w] = ffma2(e12, xv[w], acc[u][2][w]);
                    acc[u][3][w] = ffma2(e22, xv[w], acc[u][3][w]);
                }
            } else {
                const float xv = xp[0];
                acc[u][0][0].x += xv;
                acc[u][1][0].x = fmaf(f, xv, acc[u][1][0].x);
                acc[u][2][0].x = fmaf(e1, xv, acc[u][2][0].x);
                acc[u][3][0].x = fmaf(e2, xv, acc[u][3][0].x);
            }
        }
    }
    __syncthreads();  // every thread is done with the staged image values
#pragma unroll
    for (int u = 0; u < MAXP; ++u) {
        if (pj[u] < 0) continue;
#pragma unroll
        for (int m = 0; m < 4; ++m)
#pragma unroll
            for (int w = 0; w < WP; ++w) {
                if constexpr (WT >= 2)
                    M2v[((pj[u] * 4 + m) * WP + w) * NBKp + pi[u]] = acc[u][m][w];
                else
                    M1s[(pj[u] * 4 + m) * NBKp + pi[u]] = acc[u][m][0].x;
            }
    }
    __syncthreads();

    // phase 2: output t (local tl) reads buckets t - F - 1 .. t + F, i.e.
    // local indices tl .. tl + 2F + 1.  A thread filters FB = 4 consecutive
    // outputs of one (detector, instance pair) from one window of 2F + 3
    // moments: outputs tl0 + u read M0 / M1 at tl0 + 1 + (u + F - k).
    // Consecutive threads take consecutive (detector, pair) rows (odd row
    // stride: distinct banks); the tile goes through shared memory (over the
    // entries, no longer needed) so that the global stores run along t.
    constexpr int FB = 4;
    const int ntb = TT / FB, nrow = G * WP, TTp = TT + 1;
    float *s_out = reinterpret_cast<float *>(s_ent);  // [G][WT][TTp]
    for (int it = tid; it < nrow * ntb; it += nthr) {
        const int r = it % nrow, tb = it / nrow, wp = r % WP, jj = r / WP;
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
    for (int o = tid; o < G * WT * TT; o += nthr) {
        const int tl = o % TT, rw = o / TT, w = rw % WT, jj = rw / WT;
        const int d = d0 + jj, t = t0 + tl;
        if (d < D && t < T) raw[((size_t)(w0 + w) * D + d) * T + t] = s_out[rw * TTp + tl];
    }
}

// ---------------------------------------------------------------------------
// host: table construction at plan creation
// ---------------------------------------------------------------------------
// words of the entries region: the entries, then (after the moments) the
// output tile [G][wt][TT + 1]; a multiple of 4
int st_ent_region(const Plan &p, int wt) {
    const int out = p.st_g * wt * (p.st_tt + 1);
    return (std::max(p.st_ent_cap, out) + 3) & ~3;
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
    const int NBKp = (p.st_tt + 2 * p.F + 1) | 1;
    const size_t xs = std::max((size_t)p.st_umax * wt, (size_t)p.st_g * 4 * wt * NBKp);
    return (size_t)st_ent_region(p, wt) * 4 + (size_t)p.st_off_stride * 4 + 16 + xs * 4;
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
    // two CTAs per SM (228 KB less 1 KB per CTA), else one; shapes of at
    // least two warps first
    const size_t budgets[] = {(size_t)113 * 1024, (size_t)std::max(0, dev_smem - 1024)};
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
                    const size_t xs = std::max(umax * 8, (size_t)G * 4 * 8 * (NBK | 1));
                    const size_t er = std::max(emax, (size_t)G * 8 * (TT + 1));
                    const size_t need = ((er + 3) & ~(size_t)3) * 4 +
                                        (size_t)((G * (NBK + 1) + 3) & ~3) * 4 + 16 + xs * 4;
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
        p.st_info, p.st_u, p.st_off, p.st_ent, xt, raw, p.P, p.D, p.T, p.st_g, p.st_tt,
        p.st_ntiles, p.st_off_stride, st_ent_region(p, WT), p.st_ib, p.frac_bits, p.inv_r, p.ce1,
        p.ce2, scale));
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
        case 8: return st_launch_f<8>(p, xt, raw, W, scale, st);
        case 4: return st_launch_f<4>(p, xt, raw, W, scale, st);
        case 2: return st_launch_f<2>(p, xt, raw, W, scale, st);
        default: return st_launch_f<1>(p, xt, raw, W, scale, st);
    }
}

int fwd_staged_error(int clear) {
    int v = 0;
    if (cudaMemcpyFromSymbol(&v, g_fwd_st_err, sizeof v) != cudaSuccess) return -1;
    if (clear && v) {
        const int z = 0;
        cudaMemcpyToSymbol(g_fwd_st_err, &z, sizeof z);
    }
    return v;
}

}  // namespace msot
