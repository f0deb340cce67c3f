// plan.cu -- plan creation: validates the model tables of one MSOTmodel and
// lays them out in HBM for the sm_103a kernels (layout in common.cuh).
//
// Replaces the per-call inputs of the reference MEX functions
// (forwardDelayAndSumMex.cpp:17-55, forwardMex.cpp:18-73) and the model
// fields built by MSOTmodel.m:31-47 with one device-resident object.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdlib>
#include <cstring>
#include <vector>

#include <map>
#include <mutex>
#include <set>
#include <utility>

#include "common.cuh"

namespace msot {

static thread_local char g_err[512] = "";

const char *set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
    return g_err;
}

int check_plan_device(const Plan &pl, const char *who) {
    int dev = -1;
    MSOT_CUDA_TRY(cudaGetDevice(&dev));
    if (dev != pl.device) {
        set_error("%s: the plan was created on device %d but device %d is current", who,
                  pl.device, dev);
        return MSOT_EINVAL;
    }
    return MSOT_OK;
}

int sm_count() {
    static std::atomic<int> cached[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return 1;
    if (dev < 64) {
        const int c = cached[dev].load(std::memory_order_relaxed);
        if (c > 0) return c;
    }
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
        return 1;
    if (dev < 64) cached[dev].store(n, std::memory_order_relaxed);
    return n;
}

cudaError_t raise_max_dynamic_smem(const void *func, size_t bytes) {
    static std::mutex mu;
    static std::map<std::pair<int, const void *>, size_t> current;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(mu);
    size_t &c = current[{dev, func}];
    if (bytes <= c) return cudaSuccess;
    e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess) c = bytes;
    return e;
}

template <class T>
static int upload(T **dst, const T *src, size_t n, size_t &bytes) {
    if (n == 0) {
        *dst = nullptr;
        return MSOT_OK;
    }
    cudaError_t e = cudaMalloc((void **)dst, n * sizeof(T));
    if (e != cudaSuccess) {
        set_error("cudaMalloc(%zu): %s", n * sizeof(T), cudaGetErrorString(e));
        return MSOT_ENOMEM;
    }
    bytes += n * sizeof(T);
    if (src) MSOT_CUDA_TRY(cudaMemcpy(*dst, src, n * sizeof(T), cudaMemcpyHostToDevice));
    return MSOT_OK;
}

template <class T>
static int alloc(T **dst, size_t n, size_t &bytes) {
    return upload<T>(dst, nullptr, n, bytes);
}

static void free_plan(Plan &p) {
    solver_cache_free(p);
    void *ptrs[] = {p.tau_tiles, p.tau_pi, p.perm, p.ir_fwd, p.ir_adj, p.pre_x, p.pre_z,
                    p.sir, p.sir_se, p.sir_tiles, p.sir_pi, p.scr_img0, p.scr_img1,
                    p.scr_sino, p.fwd_off, p.fwd_ent, p.blk_tau, p.blk_span,
                    p.scr_part, p.fft_tw, p.fft_hf, p.fft_ha, p.fft_twb, p.fft_twn,
                    p.fft_hfb, p.fft_hab, p.st_info, p.st_u, p.st_off, p.st_ent,
                    p.h16_sc, p.fwd_ell, p.fwd_ell_off};
    for (void *q : ptrs)
        if (q) cudaFree(q);
    p = Plan();
}

// Fixed-point travel time: tau_fx = rint(tau * 2^fb).  The device computes
// the tap range of a (pixel, detector) pair as [ceil((tau_fx - r_fx) / 2^fb),
// floor((tau_fx + r_fx) / 2^fb)], i.e. {t : |t - tau| <= r} in fixed point.
static inline int32_t to_fx(double v, int fb) { return (int32_t)std::nearbyint(std::ldexp(v, fb)); }
static inline int tap_lo(int32_t tau, int32_t r, int fb) { return -((r - tau) >> fb); }
static inline int tap_hi(int32_t tau, int32_t r, int fb) { return (tau + r) >> fb; }

static int build(const msot_plan_desc *d, Plan &p) {
    if (!d || d->nx <= 0 || d->nz <= 0 || d->n_det <= 0 || d->n_t <= 1 || !d->travel) {
        set_error("plan: bad grid / detector / sample counts or missing travel table");
        return MSOT_EINVAL;
    }
    if (!(d->radius > 0) || !std::isfinite(d->radius)) {
        set_error("plan: interpolation radius must be positive");
        return MSOT_EINVAL;
    }
    const bool has_sir = d->sir_len > 0;
    if (has_sir && (!d->sir || !d->sir_start_end || !d->sir_idx || d->n_sir <= 0)) {
        set_error("plan: SIR tables incomplete");
        return MSOT_EINVAL;
    }
    if (d->ir_len < 0 || (d->ir_len > 0 && (d->ir_len % 2 == 0 || !d->ir))) {
        set_error("plan: IR length must be odd (got %d)", d->ir_len);
        return MSOT_EINVAL;
    }
    if ((long)d->nx * d->nz > (1L << 28) || (long)d->n_det * d->nx * d->nz > (1L << 34)) {
        set_error("plan: grid too large");
        return MSOT_EINVAL;
    }
    MSOT_CUDA_TRY(cudaGetDevice(&p.device));
    p.nx = d->nx;
    p.nz = d->nz;
    p.P = d->nx * d->nz;
    p.D = d->n_det;
    p.T = d->n_t;
    p.radius = d->radius;
    p.max_batch = d->max_batch > 0 ? d->max_batch : 1;
    const long PD = (long)p.P * p.D;

    // --- fixed-point format ---------------------------------------------------
    double tmax = 0;
    for (long i = 0; i < PD; ++i) {
        double t = d->travel[i];
        if (!std::isfinite(t)) {
            set_error("plan: non-finite travel time at %ld", i);
            return MSOT_ENONFINITE;
        }
        tmax = std::max(tmax, std::fabs(t));
    }
    double span = std::max(tmax, (double)p.T) + d->radius + 4.0;
    int ib = (int)std::ceil(std::log2(span));       // integer bits needed
    int fb = std::min(30 - ib, 23 - (int)std::ceil(std::log2(d->radius + 2.0)));
    fb = std::min(fb, 20);
    if (fb < 8) {
        set_error("plan: travel times (%g) or radius (%g) too large for fixed point", tmax,
                  d->radius);
        return MSOT_ERANGE;
    }
    p.frac_bits = fb;
    p.r_fx = to_fx(d->radius, fb);
    p.c1 = (float)(std::ldexp(1.0, -fb) / d->radius);
    p.n_tap = (int)std::floor(2.0 * d->radius) + 2;
    p.F = (int)std::floor(d->radius);
    p.inv_r = (float)(1.0 / d->radius);
    p.ce1 = (float)((d->radius - p.F) / d->radius);
    p.ce2 = (float)((p.F + 1 - d->radius) / d->radius);
    if (!has_sir && p.F > 8) {
        set_error("plan: interpolation radius %g too large (at most 9 samples without SIR)",
                  d->radius);
        return MSOT_EINVAL;
    }

    std::vector<int32_t> tfx(PD);
    for (long i = 0; i < PD; ++i) tfx[i] = to_fx(d->travel[i], fb);
    if (!has_sir) {
        // The DAS MEX has no bounds check (forwardDelayAndSumMex.cpp:80); its
        // precondition -- every tap inside [0, T) -- is checked here instead.
        for (long i = 0; i < PD; ++i) {
            if (tap_lo(tfx[i], p.r_fx, fb) < 0 || tap_hi(tfx[i], p.r_fx, fb) >= p.T) {
                set_error("plan: travel time %g (pixel %ld, detector %ld) puts taps outside "
                          "[0, %d)",
                          d->travel[i], i % p.P, i / p.P, p.T);
                return MSOT_ERANGE;
            }
        }
    }

    // --- forward table: pixels of each detector bucketed by floor(tau) ---------------
    std::vector<int32_t> foff;
    std::vector<int2> fent;
    if (!has_sir) {
        foff.assign((size_t)p.D * (p.T + 1), 0);
        fent.resize(PD);
        for (int det = 0; det < p.D; ++det) {
            int32_t *o = foff.data() + (size_t)det * (p.T + 1);
            const int32_t *tf = tfx.data() + (size_t)det * p.P;
            for (int q = 0; q < p.P; ++q) ++o[(tf[q] >> fb) + 1];
            for (int b = 0; b < p.T; ++b) o[b + 1] += o[b];
            std::vector<int32_t> fill(o, o + p.T);
            int2 *e = fent.data() + (size_t)det * p.P;
            for (int q = 0; q < p.P; ++q) e[fill[tf[q] >> fb]++] = make_int2(tf[q], q);
        }
    }
    // interleaved (ELL) copy of the forward table per (detector, time tile of
    // k_das_fwd3: 256 buckets from tile * (256 - 2F - 2) - F - 1, warp)
    std::vector<int2> fell;
    std::vector<int32_t> felloff;
    if (!has_sir && p.F <= 8) {
        const int TB = 256 - 2 * p.F - 2;
        p.fwd_ell_tiles = div_up(p.T, TB);
        felloff.reserve((size_t)p.D * p.fwd_ell_tiles * 8 + 1);
        fell.reserve((size_t)PD + PD / 2);
        const int nblk = p.fwd_ell_tiles * 8;
        std::vector<int> Ks(nblk);
        for (int det = 0; det < p.D; ++det) {
            const int32_t *o = foff.data() + (size_t)det * (p.T + 1);
            const int2 *e = fent.data() + (size_t)det * p.P;
            size_t add = 0;
            for (int i = 0; i < nblk; ++i) {
                const int b0 = (i / 8) * TB - p.F - 1 + 32 * (i % 8);
                int K = 0;
                for (int l = 0; l < 32; ++l) {
                    const int b = b0 + l;
                    if (b >= 0 && b < p.T) K = std::max(K, o[b + 1] - o[b]);
                }
                Ks[i] = K;
                add += (size_t)K * 32;
            }
            if (fell.size() + add > (size_t)INT32_MAX) {
                set_error("plan: interleaved forward table above 2^31 entries");
                return MSOT_EINVAL;
            }
            for (int i = 0; i < nblk; ++i) {
                felloff.push_back((int32_t)fell.size());
                const int b0 = (i / 8) * TB - p.F - 1 + 32 * (i % 8);
                for (int k = 0; k < Ks[i]; ++k)
                    for (int l = 0; l < 32; ++l) {
                        const int b = b0 + l;
                        const bool in = b >= 0 && b < p.T && k < o[b + 1] - o[b];
                        fell.push_back(in ? e[o[b] + k] : make_int2(0, -1));
                    }
            }
        }
        felloff.push_back((int32_t)fell.size());
    }

    // --- adjoint blocks: 64x64 pixels, travel times and bucket span per detector --------
    std::vector<int32_t> btau;
    std::vector<int2> bspan;
    if (!has_sir) {
        p.n_blk_x = div_up(p.nx, BLK_X);
        p.n_blk_z = div_up(p.nz, BLK_Z);
        p.n_blk = p.n_blk_x * p.n_blk_z;
        btau.assign((size_t)p.n_blk * p.D * BLK, TAU_PAD);
        bspan.assign((size_t)p.n_blk * p.D, make_int2(0, -1));
        for (int bz = 0; bz < p.n_blk_z; ++bz)
            for (int bx = 0; bx < p.n_blk_x; ++bx) {
                const int blk = bz * p.n_blk_x + bx;
                for (int det = 0; det < p.D; ++det) {
                    int bmin = INT32_MAX, bmax = INT32_MIN;
                    int32_t *dst = btau.data() + ((size_t)blk * p.D + det) * BLK;
                    for (int k = 0; k < BLK_PPT; ++k)
                        for (int t = 0; t < BLK_THREADS; ++t) {
                            const int iz = bz * BLK_Z + t % BLK_Z;
                            const int ix = bx * BLK_X + t / BLK_Z + (BLK_THREADS / BLK_Z) * k;
                            if (ix >= p.nx || iz >= p.nz) continue;
                            const int32_t v = tfx[(size_t)det * p.P + (size_t)ix * p.nz + iz];
                            dst[k * BLK_THREADS + t] = v;
                            bmin = std::min(bmin, v >> fb);
                            bmax = std::max(bmax, v >> fb);
                        }
                    if (bmax >= bmin) {
                        bspan[(size_t)blk * p.D + det] = make_int2(bmin, bmax);
                        p.blk_span_max = std::max(p.blk_span_max, bmax - bmin + 1);
                    }
                }
            }
    }

    // --- gather table: 8x8 pixel patches -----------------------------------------
    p.n_patch_x = div_up(p.nx, PATCH_X);
    p.n_patch_z = div_up(p.nz, PATCH_Z);
    p.n_patch = p.n_patch_x * p.n_patch_z;
    size_t ntile = has_sir ? (size_t)p.n_patch * p.D * PATCH : 0;  // SIR gather only
    std::vector<int32_t> tiles(ntile, TAU_PAD);
    std::vector<int32_t> stiles;
    if (has_sir) stiles.assign(ntile, 0);
    for (int pz = 0; pz < p.n_patch_z; ++pz)
        for (int px = 0; px < p.n_patch_x; ++px) {
            int patch = pz * p.n_patch_x + px;
            for (int q = 0; q < PATCH; ++q) {
                int ix = px * PATCH_X + q / PATCH_Z, iz = pz * PATCH_Z + q % PATCH_Z;
                if (ix >= p.nx || iz >= p.nz) continue;
                long pix = (long)ix * p.nz + iz;
                for (int det = 0; det < p.D && has_sir; ++det) {
                    size_t o = ((size_t)patch * p.D + det) * PATCH + q;
                    tiles[o] = tfx[(size_t)det * p.P + pix];
                    if (has_sir) stiles[o] = d->sir_idx[(size_t)det * p.P + pix] - 1;
                }
            }
        }

    // --- scatter table: pixels in a fixed pseudo-random order ------------------------
    // Lanes of a warp then work on pixels far apart in the image, so their
    // taps land on different samples of the shared-memory sinogram column.
    std::vector<int32_t> perm(p.P);
    for (int i = 0; i < p.P; ++i) perm[i] = i;
    uint64_t s = 0x9E3779B97F4A7C15ull;
    for (int i = p.P - 1; i > 0; --i) {
        s = s * 6364136223846793005ull + 1442695040888963407ull;
        int j = (int)((s >> 33) % (uint64_t)(i + 1));
        std::swap(perm[i], perm[j]);
    }
    std::vector<int32_t> tpi(has_sir ? PD : 0);
    std::vector<int32_t> spi;
    if (has_sir) spi.resize(PD);
    for (int det = 0; det < p.D && has_sir; ++det)
        for (int j = 0; j < p.P; ++j) {
            tpi[(size_t)det * p.P + j] = tfx[(size_t)det * p.P + perm[j]];
            if (has_sir) spi[(size_t)det * p.P + j] = d->sir_idx[(size_t)det * p.P + perm[j]] - 1;
        }

    // --- SIR ----------------------------------------------------------------------
    std::vector<float> sirf;
    std::vector<int2> se;
    if (has_sir) {
        p.S = d->sir_len;
        p.NS = d->n_sir;
        for (long i = 0; i < PD; ++i)
            if (d->sir_idx[i] < 1 || d->sir_idx[i] > p.NS) {
                set_error("plan: sirIndices[%ld] = %d outside [1, %d]", i, d->sir_idx[i], p.NS);
                return MSOT_ERANGE;
            }
        se.resize(p.NS);
        int maxlen = 0;
        for (int k = 0; k < p.NS; ++k) {
            int a = d->sir_start_end[2 * k] - 1, b = d->sir_start_end[2 * k + 1] - 1;
            if (a < 0 || b >= p.S) {
                set_error("plan: sirTimestepsStartAndEnd of column %d outside [1, %d]", k + 1,
                          p.S);
                return MSOT_ERANGE;
            }
            se[k] = make_int2(a, b);
            maxlen = std::max(maxlen, b - a + 1);
        }
        sirf.resize((size_t)p.NS * p.S);
        for (size_t i = 0; i < sirf.size(); ++i) sirf[i] = (float)d->sir[i];
        (void)maxlen;
    }

    // --- IR, prefilter, normalisation ----------------------------------------------
    p.norm = d->norm > 0 ? d->norm : 1.0;
    p.scale = (float)(1.0 / p.norm);
    std::vector<float> irf, ira;
    if (d->ir_len > 0) {
        p.L = d->ir_len;
        p.Lh = p.L / 2;
        irf.resize(p.L);
        ira.resize(p.L);
        for (int k = 0; k < p.L; ++k) {
            irf[k] = (float)(d->ir[k] / p.norm);
            ira[k] = (float)(d->ir[p.L - 1 - k] / p.norm);
        }
    }
    // FFT convolution tables (FP64 on the host, rounded once to FP32)
    std::vector<float2> ftw, fhf, fha;
    if (p.L > 0 && p.L <= 2049) {
        p.fft_log4n = p.L <= 513 ? 5 : 6;
        const int N = 1 << (2 * p.fft_log4n);
        ftw.resize(N);
        fhf.resize(N);
        fha.resize(N);
        const double two_pi = 6.283185307179586476925286766559;
        for (int t = 0; t < N; ++t)
            ftw[t] = make_float2((float)std::cos(two_pi * t / N), (float)-std::sin(two_pi * t / N));
        // direct DFT of the short tap vectors: H[f] = sum_k h[k] e^{-2 pi i f k / N} / N
        for (int f = 0; f < N; ++f) {
            double fr = 0, fi = 0, ar = 0, ai = 0;
            for (int k = 0; k < p.L; ++k) {
                const double ang = -two_pi * (double)(((long)f * k) % N) / N;
                const double c = std::cos(ang), sn = std::sin(ang);
                const double hf = d->ir[k] / p.norm, ha = d->ir[p.L - 1 - k] / p.norm;
                fr += hf * c; fi += hf * sn;
                ar += ha * c; ai += ha * sn;
            }
            fhf[f] = make_float2((float)(fr / N), (float)(fi / N));
            fha[f] = make_float2((float)(ar / N), (float)(ai / N));
        }
    }
    std::vector<float4> ftwb, ftwn, fhfb, fhab;
    if (p.fft_log4n == 5) {
        auto brev5 = [](int i) {
            return ((i & 1) << 4) | ((i & 2) << 2) | (i & 4) | ((i & 8) >> 2) | ((i & 16) >> 4);
        };
        ftwb.resize(512);
        ftwn.resize(512);
        fhfb.resize(512);
        fhab.resize(512);
        for (int m = 0; m < 16; ++m)
            for (int lane = 0; lane < 32; ++lane) {
                const int i = m * 32 + lane, ka = brev5(2 * m), kb = brev5(2 * m + 1);
                const float2 a = ftw[lane * ka], b = ftw[lane * kb];
                ftwb[i] = make_float4(a.x, b.x, a.y, b.y);
                const float2 c = ftw[lane * 2 * m], d = ftw[lane * (2 * m + 1)];
                ftwn[i] = make_float4(c.x, d.x, -c.y, -d.y);
                const float2 hf = fhf[lane + 32 * ka], hg = fhf[lane + 32 * kb];
                fhfb[i] = make_float4(hf.x, hg.x, hf.y, hg.y);
                const float2 ha = fha[lane + 32 * ka], hb = fha[lane + 32 * kb];
                fhab[i] = make_float4(ha.x, hb.x, ha.y, hb.y);
            }
    }
    std::vector<float> px, pz;
    if (d->pre_len_x > 0) {
        if (d->pre_len_x % 2 == 0 || !d->pre_x || d->pre_len_x > 2 * p.nx - 1) {
            set_error("plan: bad prefilter length along x");
            return MSOT_EINVAL;
        }
        p.Kx = d->pre_len_x / 2;
        px.assign(d->pre_x, d->pre_x + d->pre_len_x);
    }
    if (d->pre_len_z > 0) {
        if (d->pre_len_z % 2 == 0 || !d->pre_z || d->pre_len_z > 2 * p.nz - 1) {
            set_error("plan: bad prefilter length along z");
            return MSOT_EINVAL;
        }
        p.Kz = d->pre_len_z / 2;
        pz.assign(d->pre_z, d->pre_z + d->pre_len_z);
    }

    // --- upload -------------------------------------------------------------------
    size_t &B = p.device_bytes;
    int rc;
#define UP(dst, vec)                                                                       \
    if ((rc = upload(&(dst), (vec).data(), (vec).size(), B)) != MSOT_OK) return rc;
    UP(p.tau_tiles, tiles);
    UP(p.tau_pi, tpi);
    UP(p.perm, perm);
    if (!has_sir) {
        if ((rc = build_fwd_staged(p, tfx.data(), foff.data(), fent.data(), B)) != MSOT_OK)
            return rc;
        UP(p.fwd_off, foff);
        UP(p.fwd_ent, fent);
        UP(p.fwd_ell, fell);
        UP(p.fwd_ell_off, felloff);
        UP(p.blk_tau, btau);
        UP(p.blk_span, bspan);
    }
    if (has_sir) {
        UP(p.sir, sirf);
        UP(p.sir_se, se);
        UP(p.sir_tiles, stiles);
        UP(p.sir_pi, spi);
    }
    if (p.L) {
        UP(p.ir_fwd, irf);
        UP(p.ir_adj, ira);
    }
    if (p.fft_log4n) {
        UP(p.fft_tw, ftw);
        UP(p.fft_hf, fhf);
        UP(p.fft_ha, fha);
    }
    if (p.fft_log4n == 5) {
        UP(p.fft_twb, ftwb);
        UP(p.fft_twn, ftwn);
        UP(p.fft_hfb, fhfb);
        UP(p.fft_hab, fhab);
    }
    if (p.Kx >= 0) {
        std::vector<float> v(px.begin(), px.end());
        UP(p.pre_x, v);
    }
    if (p.Kz >= 0) {
        std::vector<float> v(pz.begin(), pz.end());
        UP(p.pre_z, v);
    }
#undef UP
    const size_t W = (size_t)p.max_batch;
    if ((rc = alloc(&p.scr_img0, W * p.P, B)) != MSOT_OK) return rc;
    if ((rc = alloc(&p.scr_img1, W * p.P, B)) != MSOT_OK) return rc;
    if ((rc = alloc(&p.scr_sino, W * p.D * p.T, B)) != MSOT_OK) return rc;
    if ((rc = alloc(&p.h16_sc, 2 * W, B)) != MSOT_OK) return rc;
    p.pre_gain_x = p.pre_gain_z = 1.f;  // bounds of |prefiltered| / max |input|
    if (!px.empty()) {
        double g = 0;
        for (float t : px) g += std::fabs((double)t);
        p.pre_gain_x = (float)g;
    }
    if (!pz.empty()) {
        double g = 0;
        for (float t : pz) g += std::fabs((double)t);
        p.pre_gain_z = (float)g;
    }
    if (!has_sir) {
        // detector groups of the adjoint: enough CTAs to fill the GPU twice,
        // at most 512 partial images in flight
        p.adj_groups_max = std::max(1, std::min(p.D, (int)std::min<size_t>(32, 512 / W)));
        if ((rc = alloc(&p.scr_part, (size_t)p.adj_groups_max * W * p.P, B)) != MSOT_OK)
            return rc;
    }

    return MSOT_OK;
}

}  // namespace msot

using namespace msot;

extern "C" {

const char *msot_last_error(void) { return g_err; }
int msot_version(void) { return 1; }

static std::mutex g_live_mu;
static std::set<const msot_plan *> g_live;  // plans created and not yet destroyed

int msot_plan_valid(msot_plan_t plan) {
    std::lock_guard<std::mutex> g(g_live_mu);
    return plan && g_live.count(plan) ? 1 : 0;
}

int msot_plan_create(const msot_plan_desc *desc, msot_plan_t *out) {
    if (!out) {
        set_error("plan: null output handle");
        return MSOT_EINVAL;
    }
    *out = nullptr;
    msot_plan *h = new (std::nothrow) msot_plan;
    if (!h) return MSOT_ENOMEM;
    int rc = build(desc, h->p);
    if (rc != MSOT_OK) {
        free_plan(h->p);
        delete h;
        return rc;
    }
    {
        std::lock_guard<std::mutex> g(g_live_mu);
        g_live.insert(h);
    }
    *out = h;
    return MSOT_OK;
}

int msot_plan_destroy(msot_plan_t plan) {
    if (!plan) return MSOT_OK;
    {
        std::lock_guard<std::mutex> g(g_live_mu);
        g_live.erase(plan);
    }
    free_plan(plan->p);
    delete plan;
    return MSOT_OK;
}

size_t msot_plan_device_bytes(msot_plan_t plan) { return plan ? plan->p.device_bytes : 0; }

}  // extern "C"
