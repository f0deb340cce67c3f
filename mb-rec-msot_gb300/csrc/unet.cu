// unet.cu -- the learned warm start: a U-Net on the project's own kernels.
//
// No counterpart in the reference.  Architecture (levels L, base channels
// c0, channels c_l = c0 2^l, square images of side S divisible by 2^(L-1)):
//   encoder l = 0..L-1:  conv3x3 + ReLU, conv3x3 + ReLU (-> e_l), 2x2 average
//                        pool (l < L-1)
//   decoder l = L-2..0:  nearest 2x upsampling of d_{l+1} (d_{L-1} = e_{L-1}),
//                        concat [up, e_l], conv3x3 + ReLU, conv3x3 + ReLU (-> d_l)
//   output:              conv1x1 c0 -> 1
// Activations NCHW FP32; weights kept in FP32 (Adam) and used as BF16 in the
// forward and data-gradient convolutions, FP32 accumulation everywhere.
// Parameter layout (flat): per conv in the order enc (a, b) l = 0..L-1, dec
// (c, d) l = L-2..0, output: weight [Co][Ci][k][k], then bias [Co].
#include <cuda_bf16.h>

#include <atomic>
#include <cmath>
#include <cstdint>
#include <random>
#include <vector>

#include "common.cuh"

namespace msot {

constexpr int CT = 16;   // spatial tile
constexpr int COT = 8;   // output channels per CTA
constexpr int CIT = 8;   // input channels per shared-memory stage

// 3x3 "same" convolution, out[n][o][y][x] = bias[o] + sum_i sum_k w(o, i, k)
// in[n][i][y + ky - 1][x + kx - 1]; TRANS reads the data-gradient weights
// w(o, i, k) = W[i][o][8 - k] of a layer W[Co'][Ci'][9] (Ci' = Co here).
template <bool TRANS>
__global__ void __launch_bounds__(256) k_conv3(const float *__restrict__ in, int Ci,
                                               const __nv_bfloat16 *__restrict__ w,
                                               const float *__restrict__ bias,
                                               float *__restrict__ out, int Co, int H, int Wd,
                                               int relu, int tiles_x) {
    __shared__ float s_in[CIT][CT + 2][CT + 3];
    __shared__ float s_w[COT][CIT][9];
    const int tile = blockIdx.x, ty0 = (tile / tiles_x) * CT, tx0 = (tile % tiles_x) * CT;
    const int co0 = blockIdx.y * COT, n = blockIdx.z;
    const int tx = threadIdx.x % CT, ty = threadIdx.x / CT;
    const float *inn = in + (size_t)n * Ci * H * Wd;
    float acc[COT];
#pragma unroll
    for (int c = 0; c < COT; ++c) acc[c] = 0.f;
    for (int ci0 = 0; ci0 < Ci; ci0 += CIT) {
        for (int i = threadIdx.x; i < CIT * (CT + 2) * (CT + 2); i += 256) {
            const int c = i / ((CT + 2) * (CT + 2)), r = i % ((CT + 2) * (CT + 2));
            const int yy = r / (CT + 2), xx = r % (CT + 2);
            const int y = ty0 + yy - 1, x = tx0 + xx - 1;
            float v = 0.f;
            if (ci0 + c < Ci && y >= 0 && y < H && x >= 0 && x < Wd)
                v = inn[((size_t)(ci0 + c) * H + y) * Wd + x];
            s_in[c][yy][xx] = v;
        }
        for (int i = threadIdx.x; i < COT * CIT * 9; i += 256) {
            const int o = i / (CIT * 9), r = i % (CIT * 9), c = r / 9, k = r % 9;
            float v = 0.f;
            if (co0 + o < Co && ci0 + c < Ci) {
                const size_t idx = TRANS ? ((size_t)(ci0 + c) * Co + (co0 + o)) * 9 + (8 - k)
                                         : ((size_t)(co0 + o) * Ci + (ci0 + c)) * 9 + k;
                v = __bfloat162float(w[idx]);
            }
            s_w[o][c][k] = v;
        }
        __syncthreads();
#pragma unroll
        for (int c = 0; c < CIT; ++c)
#pragma unroll
            for (int k = 0; k < 9; ++k) {
                const float v = s_in[c][ty + k / 3][tx + k % 3];
#pragma unroll
                for (int o = 0; o < COT; ++o) acc[o] = fmaf(s_w[o][c][k], v, acc[o]);
            }
        __syncthreads();
    }
    const int y = ty0 + ty, x = tx0 + tx;
    if (y >= H || x >= Wd) return;
#pragma unroll
    for (int o = 0; o < COT; ++o) {
        if (co0 + o >= Co) break;
        float v = acc[o] + (bias ? bias[co0 + o] : 0.f);
        if (relu) v = fmaxf(v, 0.f);
        out[(((size_t)n * Co + co0 + o) * H + y) * Wd + x] = v;
    }
}

// ---------------------------------------------------------------------------
// Tensor-core 3x3 convolution (tcgen05.mma kind::tf32, accumulator in TMEM).
//
// Implicit GEMM per CTA: D[m][o] (m = pixel of an 8 x 16 tile, o = NT output
// channels) += sum over taps k and input channels i of A_k[m][i] B_k[i][o],
// A_k the input shifted by tap k, B_k[i][o] = w(o, i, k).  Input channels
// go through shared memory TC_CK at a time; each MMA consumes K = 8 channels.
// Both operands are K-major in the canonical no-swizzle layout: core
// matrices of 8 rows x 16 bytes (4 channels), 128 contiguous bytes; LBO =
// distance of the core matrices adjacent in K, SBO = in M (or N).
//   A: three copies kx = 0..2 of the 10 x 16 halo window starting at column
//      kx (core matrix (halo row, 8-column group)), so tap (ky, kx) is copy
//      kx from halo row ky: rows of D map to pixel (m / 16, m % 16).
//   B: [tap][channel group][o / 8][o % 8][channel % 4].
// Activations are rounded to TF32 (cvt.rna) when staged; BF16 weights are
// exact in TF32.  Every wait is bounded: on a timeout the CTA sets *err,
// skips its stores and still frees its TMEM.
// ---------------------------------------------------------------------------
constexpr int TC_TY = 8, TC_TX = 16;              // pixel tile (M = 128)
constexpr int TC_CK = 32;                         // input channels per stage
constexpr int TC_HY = TC_TY + 2;                  // halo rows
constexpr int TC_LBO_A = TC_HY * 2 * 128;         // 2560 B: next 4 channels
constexpr int TC_ACOPY = (TC_CK / 4) * TC_LBO_A;  // 20480 B per kx copy
constexpr int TC_THREADS = 256;

__host__ __device__ constexpr size_t tc_smem_bytes(int NT) {
    return 3 * (size_t)TC_ACOPY + 9 * (size_t)NT * 128;
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ uint64_t tc_mdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    // start (16 B units) | LBO << 16 | SBO << 32 | descriptor version 1 at bit
    // 46; base offset 0, no swizzle
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}
// instruction descriptor: D F32 (bits 4-5 = 1), A and B TF32 (bits 7-9,
// 10-12 = 2), both K-major, N >> 3 at bit 17, M >> 4 at bit 24
__host__ __device__ constexpr uint32_t tc_idesc_tf32(int M, int N) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) |
           ((uint32_t)(M >> 4) << 24);
}
__device__ __forceinline__ float tc_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}
__device__ __forceinline__ bool tc_mbar_test(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.b32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
// bounded wait for phase `parity` of the barrier (about a second)
__device__ __forceinline__ bool tc_mbar_wait(uint32_t bar, uint32_t parity) {
    const long long t0 = clock64();
    while (!tc_mbar_test(bar, parity))
        if (clock64() - t0 > 2000000000ll) return false;
    return true;
}

__device__ int g_unet_tc_err = 0;  // set by a tensor-core CTA whose wait timed out
std::atomic<int> g_unet_tc{1};     // tensor-core convolutions on (msot_tune_set)

__device__ __forceinline__ void tc_bulk_load(uint32_t dst, const void *src, uint32_t bytes,
                                             uint32_t bar) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
                 : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            dst),
        "l"(src), "r"(bytes), "r"(bar)
        : "memory");
}

// Input channels ci0 .. ci0 + 31 of the tile's halo window, staged in two
// steps so that the loads of one stage are all in flight together (and can
// overlap the previous stage's MMAs): tc_load_input fills registers, task t
// (< 1440) = 4 channels of halo pixel (row hy, column hx), hx fastest, and
// tc_store_input writes them as one 16-byte vector into each kx copy that
// holds the pixel.  Eight consecutive lanes write eight consecutive pixels
// (the eight 16-byte rows of a core matrix): no bank conflicts.
constexpr int TC_HX = TC_TX + 2;
constexpr int TC_NT_IN = (TC_CK / 4) * TC_HY * TC_HX;  // 1440 tasks
constexpr int TC_IN_PER = (TC_NT_IN + TC_THREADS - 1) / TC_THREADS;
struct TcIn {
    float4 q[TC_IN_PER];
};
__device__ __forceinline__ void tc_load_input(TcIn &R, const float *inn, int Ci, int ci0, int H,
                                              int Wd, int ty0, int tx0, bool) {
    const size_t plane = (size_t)H * Wd;
#pragma unroll
    for (int u = 0; u < TC_IN_PER; ++u) {
        const int t = threadIdx.x + u * TC_THREADS;
        const int hx = t % TC_HX, hy = (t / TC_HX) % TC_HY, cq = t / (TC_HX * TC_HY);
        const int y = ty0 + hy - 1, x = tx0 + hx - 1, c = ci0 + 4 * cq;
        float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
        if (t < TC_NT_IN && y >= 0 && y < H && x >= 0 && x < Wd) {
            const float *p0 = inn + (size_t)c * plane + (size_t)y * Wd + x;
            q.x = c < Ci ? p0[0] : 0.f;
            q.y = c + 1 < Ci ? p0[plane] : 0.f;
            q.z = c + 2 < Ci ? p0[2 * plane] : 0.f;
            q.w = c + 3 < Ci ? p0[3 * plane] : 0.f;
        }
        R.q[u] = q;
    }
}
__device__ __forceinline__ void tc_store_input(const TcIn &R, float *sA) {
#pragma unroll
    for (int u = 0; u < TC_IN_PER; ++u) {
        const int t = threadIdx.x + u * TC_THREADS;
        if (t >= TC_NT_IN) break;
        const int hx = t % TC_HX, hy = (t / TC_HX) % TC_HY, cq = t / (TC_HX * TC_HY);
        const float4 v = make_float4(tc_tf32(R.q[u].x), tc_tf32(R.q[u].y), tc_tf32(R.q[u].z),
                                     tc_tf32(R.q[u].w));
        float *base = sA + cq * (TC_LBO_A / 4) + hy * 64;
#pragma unroll
        for (int kx = 0; kx < 3; ++kx) {
            const int xx = hx - kx;
            if (xx >= 0 && xx < TC_TX)
                *reinterpret_cast<float4 *>(base + kx * (TC_ACOPY / 4) + (xx >> 3) * 32 +
                                            (xx & 7) * 4) = v;
        }
    }
}

// wpk: the layer's weights packed per (output tile, channel stage) in the
// shared-memory B layout (NT * 288 floats each, TF32-exact), see
// k_pack_weights; bias may be null (data gradient)
template <int NT>
__global__ void __launch_bounds__(TC_THREADS) k_conv3_tc(const float *__restrict__ in, int Ci,
                                                         const float *__restrict__ wpk,
                                                         const float *__restrict__ bias,
                                                         float *__restrict__ out, int Co, int H,
                                                         int Wd, int relu, int tiles_x, int vec) {
    static_assert(NT == 32 || NT == 64, "N tile");
    extern __shared__ __align__(1024) uint8_t tc_smem[];
    float *sA = reinterpret_cast<float *>(tc_smem);
    float *sB = reinterpret_cast<float *>(tc_smem + 3 * TC_ACOPY);
    __shared__ __align__(8) uint64_t mbar[2];  // [0] MMAs done, [1] weights landed
    __shared__ uint32_t tmem_slot;
    const int ty0 = (blockIdx.x / tiles_x) * TC_TY, tx0 = (blockIdx.x % tiles_x) * TC_TX;
    const int co0 = blockIdx.y * NT, n = blockIdx.z;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t bar = smem_u32(&mbar[0]), bar_w = smem_u32(&mbar[1]);
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(&tmem_slot)),
                     "r"((uint32_t)NT));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (threadIdx.x == 32) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_w));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tm = tmem_slot;
    const float *inn = in + (size_t)n * Ci * H * Wd;
    const int nstage = (Ci + TC_CK - 1) / TC_CK;
    const float *wt = wpk + (size_t)blockIdx.y * nstage * (NT * 288);
    constexpr uint32_t WBYTES = NT * 288 * 4;
    bool ok = true;
    int issued = 0;
    TcIn R;
    tc_load_input(R, inn, Ci, 0, H, Wd, ty0, tx0, vec != 0);
    for (int s = 0; s < nstage; ++s) {
        if (s > 0) {  // the previous stage's MMAs must be done with shared memory
            const bool mine = tc_mbar_wait(bar, (uint32_t)(s - 1) & 1u);
            ok = !__syncthreads_or(!mine);
            if (!ok) break;
        }
        if (threadIdx.x == 0) tc_bulk_load(smem_u32(sB), wt + (size_t)s * NT * 288, WBYTES, bar_w);
        tc_store_input(R, sA);
        // generic-proxy stores -> visible to the tensor core (async proxy)
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        // the next stage's loads go out first (warp 0 included) and overlap
        // this stage's MMAs
        if (s + 1 < nstage) tc_load_input(R, inn, Ci, (s + 1) * TC_CK, H, Wd, ty0, tx0, vec != 0);
        if (threadIdx.x == 0) {
            if (!tc_mbar_wait(bar_w, (uint32_t)s & 1u)) atomicExch(&g_unet_tc_err, 1);
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t a0 = smem_u32(sA), b0 = smem_u32(sB);
            constexpr uint32_t idesc = tc_idesc_tf32(128, NT);
#pragma unroll 1
            for (int k = 0; k < 9; ++k) {
                const int ky = k / 3, kx = k % 3;
#pragma unroll
                for (int q = 0; q < TC_CK / 8; ++q) {
                    const uint64_t da = tc_mdesc(
                        a0 + kx * TC_ACOPY + ky * 256 + q * 2 * TC_LBO_A, TC_LBO_A, 128);
                    const uint64_t db =
                        tc_mdesc(b0 + k * NT * 128 + q * 2 * (NT * 16), NT * 16, 128);
                    const uint32_t acc = (s | k | q) != 0;
                    asm volatile(
                        "{\n\t.reg .pred p;\n\t"
                        "setp.ne.b32 p, %4, 0;\n\t"
                        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tm),
                        "l"(da), "l"(db), "r"(idesc), "r"(acc));
                }
            }
            asm volatile(
                "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                    bar)
                : "memory");
        }
        issued = s + 1;
    }
    if (ok) {
        const bool mine = tc_mbar_wait(bar, (uint32_t)(nstage - 1) & 1u);
        ok = !__syncthreads_or(!mine);
    }
    if (!ok) {
        if (threadIdx.x == 0) atomicExch(&g_unet_tc_err, 1);
        // give the MMAs and the weight copy in flight a second bounded chance
        // before the TMEM and the shared memory are released
        if (issued > 0) tc_mbar_wait(bar, (uint32_t)(issued - 1) & 1u);
        if (threadIdx.x == 0 && issued < nstage) tc_mbar_wait(bar_w, (uint32_t)issued & 1u);
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    // epilogue: warp w reads TMEM lanes 32 (w % 4) .. + 31 (= pixels), columns
    // (w / 4) NT / 2 .. + NT / 2 (= output channels)
    const int m = (warp & 3) * 32 + lane;
    const int y = ty0 + m / TC_TX, x = tx0 + m % TC_TX;
    const bool inside = ok && y < H && x < Wd;
#pragma unroll
    for (int j0 = (warp >> 2) * (NT / 2); j0 < (warp >> 2) * (NT / 2) + NT / 2; j0 += 16) {
        uint32_t r[16];
        const uint32_t ta = tm + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)j0;
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, "
            "%10, %11, %12, %13, %14, %15}, [%16];"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),
              "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]),
              "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
            : "r"(ta));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        if (inside) {
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const int o = co0 + j0 + j;
                if (o < Co) {
                    float v = __uint_as_float(r[j]) + (bias ? bias[o] : 0.f);
                    if (relu) v = fmaxf(v, 0.f);
                    out[(((size_t)n * Co + o) * H + y) * Wd + x] = v;
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tm),
                     "r"((uint32_t)NT));
}

// Packs the BF16 weights of every tensor-core convolution into the
// shared-memory B layout of k_conv3_tc: for entry e (one layer, forward or
// data gradient) and element j of [Co / NT][stage][tap k][channel group]
// [o / 8][o % 8][c % 4]: w(o, c, k) = W[o][c][k] (forward) or W[c][o][8 - k]
// (data gradient: o runs over the layer's inputs, c over its outputs), 0
// outside the channel ranges.
struct PackEntry {
    size_t dst;        // offset in the packed buffer
    size_t src;        // weight offset in the BF16 parameter array
    int Ci, Co;        // channels of the convolution as launched
    int Wci, Wco;      // dimensions of the stored weights W[Wco][Wci][9]
    int NT, nstage, trans;
    size_t count;      // Co / NT * nstage * NT * 288
};
__global__ void k_pack_weights(const __nv_bfloat16 *__restrict__ wb, float *__restrict__ wpk,
                               const PackEntry *__restrict__ ent, int n_ent, size_t total) {
    for (size_t g = (size_t)blockIdx.x * blockDim.x + threadIdx.x; g < total;
         g += (size_t)gridDim.x * blockDim.x) {
        int e = 0;
        while (e + 1 < n_ent && g >= ent[e + 1].dst) ++e;
        const PackEntry E = ent[e];
        const size_t j = g - E.dst;
        const int per = E.NT * 288;
        const int blk = (int)(j / per), r = (int)(j % per);
        const int cot = blk / E.nstage, stg = blk % E.nstage;
        const int k = r / (E.NT * 32), r2 = r % (E.NT * 32);
        const int cg = r2 / (E.NT * 4), r3 = r2 % (E.NT * 4);
        const int o = cot * E.NT + (r3 / 32) * 8 + (r3 % 32) / 4;
        const int c = stg * TC_CK + cg * 4 + r3 % 4;
        float v = 0.f;
        if (o < E.Co && c < E.Ci) {
            const size_t idx = E.trans ? ((size_t)c * E.Wci + o) * 9 + (8 - k)
                                       : ((size_t)o * E.Wci + c) * 9 + k;
            v = __bfloat162float(wb[E.src + idx]);
        }
        wpk[g] = v;
    }
}

// Tensor-core weight gradient: dW[o][i][k] += sum over pixels p of
// dy[o][p] x[i][p + off_k].  Per CTA: M = 128 output channels (rows beyond
// Co are never read back), N = 32 input channels, all 9 taps accumulated in
// TMEM (columns k * 32 + i); K = the pixels of the (image, 8 x 16 tile)
// stages this CTA takes (split over blockIdx.z), 8 per MMA.
//   A (dy):  [o / 8][pixel / 4][o % 8][pixel % 4], pixel = r * 16 + x.
//   B (x):   three copies kx of the halo window starting at column kx,
//            [i / 8][halo row][x / 4][i % 8][x % 4].
// Then each CTA adds its 128 x 288 partial sums to dW with float atomics.
constexpr int DW_LBO = 128;                      // K-adjacent core matrices
constexpr int DW_SBO_A = 32 * 128;               // next 8 output channels
constexpr int DW_SBO_B = TC_HY * 4 * 128;        // next 8 input channels (5120 B)
constexpr int DW_ABYTES = 16 * DW_SBO_A;         // 65536
constexpr int DW_BCOPY = 4 * DW_SBO_B;           // 20480 per kx copy
constexpr size_t DW_SMEM = (size_t)DW_ABYTES + 3 * DW_BCOPY;

// One stage of k_conv3_dw_tc in registers.  Lane mappings put the 8 rows
// of a core matrix (output / input channel mod 8) on 8 consecutive lanes, so
// every 16-byte shared store of an 8-lane phase fills one 128-byte core
// matrix (no bank conflicts), and each channel row's 16 pixels are 64
// contiguous bytes of 4 lanes' float4 loads.
//   a[u]: task t = tid + 256 u < 256 ceil(rows / 8): o = 8 (t >> 8) + (t & 7)
//         (zero for o >= rows), pixel quad (t >> 3) & 3 of tile row (t >> 5) & 7.
//   b[u]: task t < 1280: channel 8 (t / 320) + (t & 7), quad (t >> 3) & 3 of
//         halo row (t >> 5) % 10; l[u] / r[u] the pixels left of and right of
//         the quad, so the shifted copies 0 and 2 are vectors too.
struct DwIn {
    float4 a[16];
    float4 b[5];
    float l[5], r[5];
};
__device__ __forceinline__ float4 dw_row4(const float *row, int x0, int Wd, bool vec) {
    if (vec && x0 + 3 < Wd) return *reinterpret_cast<const float4 *>(row + x0);
    return make_float4(x0 < Wd ? row[x0] : 0.f, x0 + 1 < Wd ? row[x0 + 1] : 0.f,
                       x0 + 2 < Wd ? row[x0 + 2] : 0.f, x0 + 3 < Wd ? row[x0 + 3] : 0.f);
}
__device__ __forceinline__ void dw_load(DwIn &R, const float *x, int Ci, int ci0, const float *dy,
                                        int Co, int co0, int rows, int H, int Wd, int n, int tile,
                                        int tiles_x, bool vec) {
    const int ty0 = (tile / tiles_x) * TC_TY, tx0 = (tile % tiles_x) * TC_TX;
    const float *dyn = dy + ((size_t)n * Co + co0) * H * Wd;
#pragma unroll
    for (int u = 0; u < 16; ++u) {
        const int t = threadIdx.x + u * TC_THREADS;
        const int o = 8 * (t >> 8) + (t & 7), xq = (t >> 3) & 3, r = (t >> 5) & 7;
        const int y = ty0 + r;
        R.a[u] = (t < ((rows + 7) >> 3) * 256 && o < rows && y < H)
                     ? dw_row4(dyn + ((size_t)o * H + y) * Wd, tx0 + 4 * xq, Wd, vec)
                     : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    const float *xn = x + ((size_t)n * Ci + ci0) * H * Wd;
#pragma unroll
    for (int u = 0; u < 5; ++u) {
        const int t = threadIdx.x + u * TC_THREADS;
        const int c = 8 * (t / 320) + (t & 7), xq = (t >> 3) & 3, hy = (t >> 5) % TC_HY;
        const int y = ty0 + hy - 1, x0 = tx0 + 4 * xq;
        const bool live = t < 32 * TC_HY * 4 && ci0 + c < Ci && y >= 0 && y < H;
        const float *row = xn + ((size_t)c * H + y) * Wd;
        R.b[u] = live ? dw_row4(row, x0, Wd, vec) : make_float4(0.f, 0.f, 0.f, 0.f);
        R.l[u] = live && x0 >= 1 && x0 - 1 < Wd ? row[x0 - 1] : 0.f;
        R.r[u] = live && x0 + 4 < Wd ? row[x0 + 4] : 0.f;
    }
}
// layouts: see k_conv3_dw_tc; copy kx, column xx holds input column
// tx0 + xx + kx - 1, so for quad g copy 1 is the loaded float4, copy 0 is
// (left, x, y, z) and copy 2 is (y, z, w, right)
__device__ __forceinline__ void dw_store(const DwIn &R, float *sA, float *sB, int rows) {
#pragma unroll
    for (int u = 0; u < 16; ++u) {
        const int t = threadIdx.x + u * TC_THREADS;
        if (t >= ((rows + 7) >> 3) * 256) break;
        const int o = 8 * (t >> 8) + (t & 7), xq = (t >> 3) & 3, r = (t >> 5) & 7;
        const float4 v = R.a[u];
        *reinterpret_cast<float4 *>(sA + (o >> 3) * (DW_SBO_A / 4) + (r * 4 + xq) * 32 +
                                    (o & 7) * 4) =
            make_float4(tc_tf32(v.x), tc_tf32(v.y), tc_tf32(v.z), tc_tf32(v.w));
    }
#pragma unroll
    for (int u = 0; u < 5; ++u) {
        const int t = threadIdx.x + u * TC_THREADS;
        if (t >= 32 * TC_HY * 4) break;
        const int c = 8 * (t / 320) + (t & 7), xq = (t >> 3) & 3, hy = (t >> 5) % TC_HY;
        const float4 v = R.b[u];
        const float e0 = tc_tf32(v.x), e1 = tc_tf32(v.y), e2 = tc_tf32(v.z), e3 = tc_tf32(v.w);
        float *dst = sB + (c >> 3) * (DW_SBO_B / 4) + hy * 128 + xq * 32 + (c & 7) * 4;
        *reinterpret_cast<float4 *>(dst) = make_float4(tc_tf32(R.l[u]), e0, e1, e2);
        *reinterpret_cast<float4 *>(dst + DW_BCOPY / 4) = make_float4(e0, e1, e2, e3);
        *reinterpret_cast<float4 *>(dst + 2 * (DW_BCOPY / 4)) =
            make_float4(e1, e2, e3, tc_tf32(R.r[u]));
    }
}

__global__ void __launch_bounds__(TC_THREADS) k_conv3_dw_tc(const float *__restrict__ x, int Ci,
                                                            const float *__restrict__ dy, int Co,
                                                            float *__restrict__ dw, int H, int Wd,
                                                            int N, int tiles_x, int tiles_img,
                                                            int splits, int vec) {
    extern __shared__ __align__(1024) uint8_t tc_smem[];
    float *sA = reinterpret_cast<float *>(tc_smem);
    float *sB = reinterpret_cast<float *>(tc_smem + DW_ABYTES);
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_slot;
    const int co0 = blockIdx.x * 128, ci0 = blockIdx.y * 32;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t bar = smem_u32(&mbar);
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(&tmem_slot)),
                     "r"(512u));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (threadIdx.x == 32) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tm = tmem_slot;
    const int rows = min(128, Co - co0);
    bool ok = true;
    int issued = 0;
    const int total = N * tiles_img;
    DwIn R;
    if ((int)blockIdx.z < total)
        dw_load(R, x, Ci, ci0, dy, Co, co0, rows, H, Wd, blockIdx.z / tiles_img,
                blockIdx.z % tiles_img, tiles_x, vec != 0);
    for (int tt = blockIdx.z; tt < total; tt += splits) {
        if (issued > 0) {
            const bool mine = tc_mbar_wait(bar, (uint32_t)(issued - 1) & 1u);
            ok = !__syncthreads_or(!mine);
            if (!ok) break;
        }
        dw_store(R, sA, sB, rows);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        // the next stage's loads go out first (warp 0 included) and overlap
        // this stage's MMAs
        const int nt = tt + splits;
        if (nt < total)
            dw_load(R, x, Ci, ci0, dy, Co, co0, rows, H, Wd, nt / tiles_img, nt % tiles_img,
                    tiles_x, vec != 0);
        if (threadIdx.x == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t a0 = smem_u32(sA), b0 = smem_u32(sB);
            constexpr uint32_t idesc = tc_idesc_tf32(128, 32);
#pragma unroll 1
            for (int k = 0; k < 9; ++k) {
                const int ky = k / 3, kx = k % 3;
#pragma unroll 4
                for (int j = 0; j < 16; ++j) {
                    const uint64_t da = tc_mdesc(a0 + j * 256, DW_LBO, DW_SBO_A);
                    const uint64_t db = tc_mdesc(
                        b0 + kx * DW_BCOPY + (((j >> 1) + ky) * 4 + (j & 1) * 2) * 128, DW_LBO,
                        DW_SBO_B);
                    const uint32_t acc = (issued | j) != 0;
                    asm volatile(
                        "{\n\t.reg .pred p;\n\t"
                        "setp.ne.b32 p, %4, 0;\n\t"
                        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(
                            tm + (uint32_t)(k * 32)),
                        "l"(da), "l"(db), "r"(idesc), "r"(acc));
                }
            }
            asm volatile(
                "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                    bar)
                : "memory");
        }
        ++issued;
    }
    if (ok && issued > 0) {
        const bool mine = tc_mbar_wait(bar, (uint32_t)(issued - 1) & 1u);
        ok = !__syncthreads_or(!mine);
    }
    if (!ok) {
        if (threadIdx.x == 0) atomicExch(&g_unet_tc_err, 1);
        if (issued > 0) tc_mbar_wait(bar, (uint32_t)(issued - 1) & 1u);
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    // epilogue: warp w reads lanes 32 (w % 4) + lane (= output channel) of the
    // taps k = w / 4, w / 4 + 2, ... (32 columns each)
    const int o = co0 + (warp & 3) * 32 + lane;
    const bool live = ok && issued > 0 && (warp & 3) * 32 + lane < rows;
    for (int k = warp >> 2; k < 9; k += 2) {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            uint32_t r[16];
            const uint32_t ta = tm + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)(k * 32 + h * 16);
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, "
                "%10, %11, %12, %13, %14, %15}, [%16];"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),
                  "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]),
                  "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                : "r"(ta));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (live) {
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const int c = ci0 + h * 16 + j;
                    if (c < Ci) atomicAdd(&dw[((size_t)o * Ci + c) * 9 + k], __uint_as_float(r[j]));
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tm), "r"(512u));
}

// dW[o][i][k] += sum over (n, y, x) of dy[n][o][y][x] x[n][i][y + ky - 1][x + kx - 1]
// CTA = (8 output channels, 8 input channels, split of the (n, tile) range)
__global__ void __launch_bounds__(256) k_conv3_dw(const float *__restrict__ x, int Ci,
                                                  const float *__restrict__ dy, int Co,
                                                  float *__restrict__ dw, int H, int Wd, int N,
                                                  int tiles_x, int tiles_img, int splits) {
    __shared__ float s_x[CIT][CT + 2][CT + 3];
    __shared__ float s_dy[COT][CT][CT + 1];
    const int co0 = blockIdx.x * COT, ci0 = blockIdx.y * CIT;
    constexpr int NOUT = COT * CIT * 9;  // 576
    float acc[3] = {0.f, 0.f, 0.f};
    int oo[3], ii[3], kk[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        const int t = threadIdx.x + j * 256;
        oo[j] = t / (CIT * 9);
        ii[j] = (t / 9) % CIT;
        kk[j] = t % 9;
    }
    const int total = N * tiles_img;
    for (int tt = blockIdx.z; tt < total; tt += splits) {
        const int n = tt / tiles_img, tile = tt % tiles_img;
        const int ty0 = (tile / tiles_x) * CT, tx0 = (tile % tiles_x) * CT;
        __syncthreads();
        for (int i = threadIdx.x; i < CIT * (CT + 2) * (CT + 2); i += 256) {
            const int c = i / ((CT + 2) * (CT + 2)), r = i % ((CT + 2) * (CT + 2));
            const int yy = r / (CT + 2), xx = r % (CT + 2);
            const int y = ty0 + yy - 1, xq = tx0 + xx - 1;
            float v = 0.f;
            if (ci0 + c < Ci && y >= 0 && y < H && xq >= 0 && xq < Wd)
                v = x[(((size_t)n * Ci + ci0 + c) * H + y) * Wd + xq];
            s_x[c][yy][xx] = v;
        }
        for (int i = threadIdx.x; i < COT * CT * CT; i += 256) {
            const int o = i / (CT * CT), r = i % (CT * CT), yy = r / CT, xx = r % CT;
            const int y = ty0 + yy, xq = tx0 + xx;
            float v = 0.f;
            if (co0 + o < Co && y < H && xq < Wd)
                v = dy[(((size_t)n * Co + co0 + o) * H + y) * Wd + xq];
            s_dy[o][yy][xx] = v;
        }
        __syncthreads();
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            if (threadIdx.x + j * 256 >= NOUT) break;
            const int o = oo[j], c = ii[j], ky = kk[j] / 3, kx = kk[j] % 3;
            float a = acc[j];
            for (int yy = 0; yy < CT; ++yy)
#pragma unroll
                for (int xx = 0; xx < CT; ++xx)
                    a = fmaf(s_dy[o][yy][xx], s_x[c][yy + ky][xx + kx], a);
            acc[j] = a;
        }
    }
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        if (threadIdx.x + j * 256 >= NOUT) break;
        const int o = co0 + oo[j], c = ci0 + ii[j];
        if (o < Co && c < Ci) atomicAdd(&dw[((size_t)o * Ci + c) * 9 + kk[j]], acc[j]);
    }
}

// db[o] += sum over (n, p) dy[n][o][p]; one CTA per (o, n)
__global__ void k_bias_grad(const float *__restrict__ dy, int Co, int HW, float *db) {
    __shared__ float sh[32];
    const int o = blockIdx.x, n = blockIdx.y;
    const float *p = dy + ((size_t)n * Co + o) * HW;
    float a = 0.f;
    for (int i = threadIdx.x; i < HW; i += blockDim.x) a += p[i];
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) a += __shfl_down_sync(0xffffffffu, a, s);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = a;
    __syncthreads();
    if (threadIdx.x < 32) {
        a = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.f;
#pragma unroll
        for (int s = 16; s > 0; s >>= 1) a += __shfl_down_sync(0xffffffffu, a, s);
        if (threadIdx.x == 0) atomicAdd(&db[o], a);
    }
}

// dy_pre = dy_post * (y_post > 0)
__global__ void k_relu_bwd(const float *__restrict__ y, const float *__restrict__ dy,
                           float *__restrict__ out, size_t n) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
        out[i] = y[i] > 0.f ? dy[i] : 0.f;
}

// 2x2 average pool of [NC][H][W] -> [NC][H/2][W/2], and its adjoint
__global__ void k_pool(const float *__restrict__ in, float *__restrict__ out, int NC, int H,
                       int Wd) {
    const int h = H / 2, w = Wd / 2;
    const size_t n = (size_t)NC * h * w;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        const size_t c = i / ((size_t)h * w);
        const int r = (int)(i % ((size_t)h * w)), y = r / w, x = r % w;
        const float *p = in + (c * H + 2 * y) * Wd + 2 * x;
        out[i] = 0.25f * (p[0] + p[1] + p[Wd] + p[Wd + 1]);
    }
}
__global__ void k_pool_bwd(const float *__restrict__ dout, float *__restrict__ din, int NC,
                           int H, int Wd, int accumulate) {
    const size_t n = (size_t)NC * H * Wd;
    const int w = Wd / 2, h = H / 2;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        const size_t c = i / ((size_t)H * Wd);
        const int r = (int)(i % ((size_t)H * Wd)), y = r / Wd, x = r % Wd;
        const float g = 0.25f * dout[(c * h + y / 2) * w + x / 2];
        din[i] = accumulate ? din[i] + g : g;
    }
}
// nearest 2x upsampling of [N][C][h][w] into channels [0, C) of [N][Ctot][2h][2w]
__global__ void k_up_into(const float *__restrict__ in, float *__restrict__ out, int N, int C,
                          int Ctot, int h, int w) {
    const int H = 2 * h, Wd = 2 * w;
    const size_t n = (size_t)N * C * H * Wd;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        const size_t nc = i / ((size_t)H * Wd);
        const int r = (int)(i % ((size_t)H * Wd)), y = r / Wd, x = r % Wd;
        const int b = (int)(nc / C), c = (int)(nc % C);
        out[(((size_t)b * Ctot + c) * H + y) * Wd + x] = in[(nc * h + y / 2) * w + x / 2];
    }
}
// adjoint: dsmall[n][c][y][x] = sum of the 2x2 block of channel c of dbig [N][Ctot][2h][2w]
__global__ void k_up_bwd(const float *__restrict__ dbig, float *__restrict__ dsmall, int N,
                         int C, int Ctot, int h, int w) {
    const size_t n = (size_t)N * C * h * w;
    const int Wd = 2 * w, H = 2 * h;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        const size_t nc = i / ((size_t)h * w);
        const int r = (int)(i % ((size_t)h * w)), y = r / w, x = r % w;
        const int b = (int)(nc / C), c = (int)(nc % C);
        const float *p = dbig + (((size_t)b * Ctot + c) * H + 2 * y) * Wd + 2 * x;
        dsmall[i] = p[0] + p[1] + p[Wd] + p[Wd + 1];
    }
}
// copy [N][C][HW] into channels [c0, c0 + C) of [N][Ctot][HW] (or back, adding when acc)
__global__ void k_chan_copy(const float *__restrict__ src, int Cs, int cs0, float *__restrict__ dst,
                            int Cd, int cd0, int N, int C, int HW, int acc) {
    const size_t n = (size_t)N * C * HW;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        const int p = (int)(i % HW);
        const size_t nc = i / HW;
        const int b = (int)(nc / C), c = (int)(nc % C);
        const float v = src[((size_t)b * Cs + cs0 + c) * HW + p];
        float &d = dst[((size_t)b * Cd + cd0 + c) * HW + p];
        d = acc ? d + v : v;
    }
}
// 1x1 output conv c0 -> 1 and its gradients
__global__ void k_conv1(const float *__restrict__ in, int C, const float *__restrict__ w,
                        const float *__restrict__ b, float *__restrict__ out, int N, int HW) {
    const size_t n = (size_t)N * HW;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        const int bi = (int)(i / HW), p = (int)(i % HW);
        float a = b[0];
        for (int c = 0; c < C; ++c) a = fmaf(w[c], in[((size_t)bi * C + c) * HW + p], a);
        out[i] = a;
    }
}
__global__ void k_conv1_bwd_data(const float *__restrict__ dout, const float *__restrict__ w,
                                 float *__restrict__ din, int C, int N, int HW) {
    const size_t n = (size_t)N * C * HW;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        const int p = (int)(i % HW);
        const size_t nc = i / HW;
        const int bi = (int)(nc / C), c = (int)(nc % C);
        din[i] = w[c] * dout[(size_t)bi * HW + p];
    }
}
// dw[c] += sum dout * in[c]; one CTA per (c, n)
__global__ void k_conv1_dw(const float *__restrict__ dout, const float *__restrict__ in,
                           float *dw, int C, int HW) {
    __shared__ float sh[32];
    const int c = blockIdx.x, n = blockIdx.y;
    const float *a = dout + (size_t)n * HW, *x = in + ((size_t)n * C + c) * HW;
    float s = 0.f;
    for (int i = threadIdx.x; i < HW; i += blockDim.x) s = fmaf(a[i], x[i], s);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (threadIdx.x == 0) atomicAdd(&dw[c], s);
    }
}
// loss = mean (out - t)^2 (partial sums in FP64 per CTA), dout = 2 (out - t) / n
__global__ void k_mse(const float *__restrict__ out, const float *__restrict__ t,
                      float *__restrict__ dout, size_t n, double *loss) {
    __shared__ double sh[32];
    double s = 0.0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        const float d = out[i] - t[i];
        s += (double)d * d;
        dout[i] = 2.f * d / (float)n;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (threadIdx.x == 0) atomicAdd(loss, s / (double)n);
    }
}
// Adam (Kingma & Ba) with bias correction; refreshes the BF16 copy
__global__ void k_adam(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m,
                       float *__restrict__ v, __nv_bfloat16 *__restrict__ pb, size_t n, float lr,
                       float b1, float b2, float eps, float c1, float c2) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float pi = p[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        p[i] = pi;
        pb[i] = __float2bfloat16_rn(pi);
    }
}
__global__ void k_to_bf16(const float *__restrict__ p, __nv_bfloat16 *__restrict__ pb, size_t n) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
        pb[i] = __float2bfloat16_rn(p[i]);
}

}  // namespace msot

using namespace msot;

constexpr size_t NO_PACK = ~(size_t)0;

struct ConvL {
    int Ci, Co, S;        // channels and spatial side
    size_t w_off, b_off;  // in the flat parameter array
    size_t pk_fwd = NO_PACK, pk_bwd = NO_PACK;  // packed tensor-core weights (k_pack_weights)
};

struct msot_unet {
    int L = 0, c0 = 0, S = 0, max_n = 0;
    std::vector<int> ch, side;
    std::vector<ConvL> enc_a, enc_b, dec_c, dec_d;
    size_t out_w = 0, out_b = 0, n_par = 0;
    float *par = nullptr, *grad = nullptr, *m = nullptr, *v = nullptr;
    __nv_bfloat16 *parb = nullptr;
    float *wpk = nullptr;  // tensor-core weights in the shared-memory operand layout
    PackEntry *pk_ent = nullptr;
    int n_pk = 0;
    size_t pk_total = 0;
    // forward activations (post-ReLU) per level
    std::vector<float *> ea, e, pool, cat, da, d;
    // gradient buffers per level: Ga (concat-sized), Gb, Gc, Gd, Gs (c_l channels)
    std::vector<float *> Ga, Gb, Gc, Gd, Gs;
    float *outb = nullptr, *dout = nullptr;
    double *loss = nullptr;
    std::vector<void *> all;
    ~msot_unet() {
        for (void *q : all) cudaFree(q);
    }
};

namespace {

inline unsigned nblk(size_t n) { return (unsigned)std::min<size_t>((n + 255) / 256, 65535); }

template <class T>
T *dalloc(msot_unet *u, size_t n) {
    void *p = nullptr;
    if (cudaMalloc(&p, (n ? n : 1) * sizeof(T)) != cudaSuccess) return nullptr;
    u->all.push_back(p);
    return static_cast<T *>(p);
}

inline bool tc_shape(int Ci, int Co) { return Ci >= 8 && Co % 32 == 0; }
inline int tc_nt(int Co) { return Co % 64 == 0 ? 64 : 32; }

template <int NT>
int conv3_tc(const float *in, int Ci, const float *wpk, const float *bias, float *out, int Co,
             int S, int N, int relu, cudaStream_t st) {
    const size_t smem = tc_smem_bytes(NT);
    MSOT_CUDA_TRY(raise_max_dynamic_smem((const void *)k_conv3_tc<NT>, smem));
    const int tx = (S + TC_TX - 1) / TC_TX, ty = (S + TC_TY - 1) / TC_TY;
    const int vec = (S % 4 == 0) && ((uintptr_t)in % 16 == 0);
    dim3 grid(tx * ty, Co / NT, N);
    KLAUNCH(k_conv3_tc<NT><<<grid, TC_THREADS, smem, st>>>(in, Ci, wpk, bias, out, Co, S, S, relu,
                                                          tx, vec));
    MSOT_LAUNCH_CHECK();
    return MSOT_OK;
}

// 3x3 "same" convolution of [N][Ci][S][S] into [N][Co][S][S]: on the tensor
// cores when the layer's weights were packed for this direction (Ci >= 8,
// Co a multiple of 32: every layer but the network's first), else the
// CUDA-core kernel on the BF16 weights
template <bool TRANS>
int conv3(const float *in, int Ci, const __nv_bfloat16 *w, const float *wpk, const float *bias,
          float *out, int Co, int S, int N, int relu, cudaStream_t st) {
    if (g_unet_tc.load() && wpk)
        return tc_nt(Co) == 64 ? conv3_tc<64>(in, Ci, wpk, bias, out, Co, S, N, relu, st)
                               : conv3_tc<32>(in, Ci, wpk, bias, out, Co, S, N, relu, st);
    const int tx = (S + CT - 1) / CT;
    dim3 grid(tx * tx, (Co + COT - 1) / COT, N);
    KLAUNCH(k_conv3<TRANS><<<grid, 256, 0, st>>>(in, Ci, w, bias, out, Co, S, S, relu, tx));
    MSOT_LAUNCH_CHECK();
    return MSOT_OK;
}

int conv_fwd(msot_unet *u, const ConvL &c, const float *in, float *out, int N, cudaStream_t st) {
    return conv3<false>(in, c.Ci, u->parb + c.w_off,
                        c.pk_fwd == NO_PACK ? nullptr : u->wpk + c.pk_fwd, u->par + c.b_off, out,
                        c.Co, c.S, N, 1, st);
}

int pack_weights(msot_unet *u, cudaStream_t st) {
    if (!u->pk_total) return MSOT_OK;
    KLAUNCH(k_pack_weights<<<nblk(u->pk_total), 256, 0, st>>>(u->parb, u->wpk, u->pk_ent,
                                                              u->n_pk, u->pk_total));
    MSOT_LAUNCH_CHECK();
    return MSOT_OK;
}

// conv c with input x and ReLU output y; dy_post = d loss / d y.  Adds dW, db;
// writes dy_pre (scratch) and dx (if non-null).  No two pointers alias.
int conv_bwd(msot_unet *u, const ConvL &c, const float *x, const float *y, const float *dy_post,
             float *dy_pre, float *dx, int N, cudaStream_t st) {
    const size_t ny = (size_t)N * c.Co * c.S * c.S;
    KLAUNCH(k_relu_bwd<<<nblk(ny), 256, 0, st>>>(y, dy_post, dy_pre, ny));
    if (g_unet_tc.load() && c.Ci >= 8) {
        const int tx = (c.S + TC_TX - 1) / TC_TX, ty = (c.S + TC_TY - 1) / TC_TY;
        const int tiles = tx * ty, cog = (c.Co + 127) / 128, cig = (c.Ci + 31) / 32;
        const int splits = std::max(1, std::min(N * tiles, (sm_count() - 4) / (cog * cig)));
        MSOT_CUDA_TRY(raise_max_dynamic_smem((const void *)k_conv3_dw_tc, DW_SMEM));
        const int vec = (c.S % 4 == 0) && ((uintptr_t)x % 16 == 0) && ((uintptr_t)dy_pre % 16 == 0);
        KLAUNCH(k_conv3_dw_tc<<<dim3(cog, cig, splits), TC_THREADS, DW_SMEM, st>>>(
            x, c.Ci, dy_pre, c.Co, u->grad + c.w_off, c.S, c.S, N, tx, tiles, splits, vec));
    } else {
        const int tx = (c.S + CT - 1) / CT, tiles = tx * tx;
        const int cog = (c.Co + COT - 1) / COT, cig = (c.Ci + CIT - 1) / CIT;
        const int splits =
            std::max(1, std::min(N * tiles, (4 * sm_count() + cog * cig - 1) / (cog * cig)));
        KLAUNCH(k_conv3_dw<<<dim3(cog, cig, splits), 256, 0, st>>>(
            x, c.Ci, dy_pre, c.Co, u->grad + c.w_off, c.S, c.S, N, tx, tiles, splits));
    }
    KLAUNCH(k_bias_grad<<<dim3(c.Co, N), 256, 0, st>>>(dy_pre, c.Co, c.S * c.S,
                                                        u->grad + c.b_off));
    MSOT_LAUNCH_CHECK();
    if (dx)
        return conv3<true>(dy_pre, c.Co, u->parb + c.w_off,
                           c.pk_bwd == NO_PACK ? nullptr : u->wpk + c.pk_bwd, nullptr, dx, c.Ci,
                           c.S, N, 0, st);
    return MSOT_OK;
}

int forward(msot_unet *u, const float *in, int N, cudaStream_t st) {
    int rc;
    const int L = u->L;
    const float *x = in;
    for (int l = 0; l < L; ++l) {
        if ((rc = conv_fwd(u, u->enc_a[l], x, u->ea[l], N, st))) return rc;
        if ((rc = conv_fwd(u, u->enc_b[l], u->ea[l], u->e[l], N, st))) return rc;
        if (l + 1 < L) {
            const int S = u->side[l];
            const size_t n = (size_t)N * u->ch[l] * (S / 2) * (S / 2);
            KLAUNCH(k_pool<<<nblk(n), 256, 0, st>>>(u->e[l], u->pool[l], N * u->ch[l], S, S));
            x = u->pool[l];
        }
    }
    const float *dn = u->e[L - 1];
    for (int l = L - 2; l >= 0; --l) {
        const int S = u->side[l], Cu = u->ch[l + 1], Ce = u->ch[l], Ct = Cu + Ce;
        KLAUNCH(k_up_into<<<nblk((size_t)N * Cu * S * S), 256, 0, st>>>(dn, u->cat[l], N, Cu, Ct,
                                                                         S / 2, S / 2));
        KLAUNCH(k_chan_copy<<<nblk((size_t)N * Ce * S * S), 256, 0, st>>>(
            u->e[l], Ce, 0, u->cat[l], Ct, Cu, N, Ce, S * S, 0));
        if ((rc = conv_fwd(u, u->dec_c[l], u->cat[l], u->da[l], N, st))) return rc;
        if ((rc = conv_fwd(u, u->dec_d[l], u->da[l], u->d[l], N, st))) return rc;
        dn = u->d[l];
    }
    const int HW = u->S * u->S;
    KLAUNCH(k_conv1<<<nblk((size_t)N * HW), 256, 0, st>>>(dn, u->c0, u->par + u->out_w,
                                                          u->par + u->out_b, u->outb, N, HW));
    MSOT_LAUNCH_CHECK();
    return MSOT_OK;
}

// gradients of mean (out - target)^2 after forward(); loss in u->loss
int backward(msot_unet *u, const float *in, const float *target, int N, cudaStream_t st) {
    int rc;
    const int HW = u->S * u->S, L = u->L;
    MSOT_CUDA_TRY(cudaMemsetAsync(u->grad, 0, u->n_par * sizeof(float), st));
    MSOT_CUDA_TRY(cudaMemsetAsync(u->loss, 0, sizeof(double), st));
    KLAUNCH(k_mse<<<nblk((size_t)N * HW), 256, 0, st>>>(u->outb, target, u->dout,
                                                       (size_t)N * HW, u->loss));
    const float *top = L >= 2 ? u->d[0] : u->e[0];
    KLAUNCH(k_conv1_dw<<<dim3(u->c0, N), 256, 0, st>>>(u->dout, top, u->grad + u->out_w, u->c0,
                                                       HW));
    KLAUNCH(k_bias_grad<<<dim3(1, N), 256, 0, st>>>(u->dout, 1, HW, u->grad + u->out_b));
    KLAUNCH(k_conv1_bwd_data<<<nblk((size_t)N * u->c0 * HW), 256, 0, st>>>(
        u->dout, u->par + u->out_w, u->Gb[0], u->c0, N, HW));
    MSOT_LAUNCH_CHECK();
    // decoder, shallow to deep: Gb[l] = d loss / d d_l on entry
    for (int l = 0; l + 1 < L; ++l) {
        const int S = u->side[l], Cu = u->ch[l + 1], Ce = u->ch[l], Ct = Cu + Ce;
        if ((rc = conv_bwd(u, u->dec_d[l], u->da[l], u->d[l], u->Gb[l], u->Gc[l], u->Gd[l], N,
                           st)))
            return rc;
        if ((rc = conv_bwd(u, u->dec_c[l], u->cat[l], u->da[l], u->Gd[l], u->Gc[l], u->Ga[l], N,
                           st)))
            return rc;
        KLAUNCH(k_chan_copy<<<nblk((size_t)N * Ce * S * S), 256, 0, st>>>(
            u->Ga[l], Ct, Cu, u->Gs[l], Ce, 0, N, Ce, S * S, 0));
        const int h = S / 2;
        KLAUNCH(k_up_bwd<<<nblk((size_t)N * Cu * h * h), 256, 0, st>>>(u->Ga[l], u->Gb[l + 1], N,
                                                                        Cu, Ct, h, h));
        MSOT_LAUNCH_CHECK();
    }
    // encoder, deep to shallow: Gb[l] = d loss / d e_l from above
    for (int l = L - 1; l >= 0; --l) {
        const int S = u->side[l];
        if (l + 1 < L) {
            const size_t n = (size_t)N * u->ch[l] * S * S;
            KLAUNCH(k_chan_copy<<<nblk(n), 256, 0, st>>>(u->Gs[l], u->ch[l], 0, u->Gb[l],
                                                         u->ch[l], 0, N, u->ch[l], S * S, 1));
        }
        if ((rc = conv_bwd(u, u->enc_b[l], u->ea[l], u->e[l], u->Gb[l], u->Gc[l], u->Gd[l], N,
                           st)))
            return rc;
        const float *xin = l == 0 ? in : u->pool[l - 1];
        if ((rc = conv_bwd(u, u->enc_a[l], xin, u->ea[l], u->Gd[l], u->Gc[l],
                           l > 0 ? u->Ga[l] : nullptr, N, st)))
            return rc;
        if (l > 0) {
            const int Sp = u->side[l - 1];
            const size_t n = (size_t)N * u->ch[l - 1] * Sp * Sp;
            KLAUNCH(k_pool_bwd<<<nblk(n), 256, 0, st>>>(u->Ga[l], u->Gb[l - 1], N * u->ch[l - 1],
                                                        Sp, Sp, 0));
            MSOT_LAUNCH_CHECK();
        }
    }
    return MSOT_OK;
}

int check_net(msot_unet_t u, int N, const void *a, const void *b) {
    if (!u || N <= 0 || N > u->max_n || !a || !b) {
        set_error("unet: bad arguments (batch %d, max %d)", N, u ? u->max_n : 0);
        return MSOT_EINVAL;
    }
    return MSOT_OK;
}

}  // namespace

extern "C" {

int msot_unet_create(int levels, int base_channels, int side, int max_batch, uint64_t seed,
                     msot_unet_t *out) {
    return msot_unet_create_ch(levels, base_channels, 1, side, max_batch, seed, out);
}

int msot_unet_create_ch(int levels, int base_channels, int in_channels, int side, int max_batch,
                        uint64_t seed, msot_unet_t *out) {
    if (!out || levels < 1 || levels > 6 || base_channels < 1 || base_channels > 256 ||
        in_channels < 1 || in_channels > 8 || max_batch < 1 || side < 1 ||
        side % (1 << (levels - 1)) != 0) {
        set_error("unet_create: bad arguments (side must be divisible by 2^(levels-1), "
                  "1 .. 8 input channels)");
        return MSOT_EINVAL;
    }
    auto *u = new msot_unet();
    u->L = levels;
    u->c0 = base_channels;
    u->S = side;
    u->max_n = max_batch;
    size_t off = 0;
    auto add = [&](std::vector<ConvL> &vec, int Ci, int Co, int S) {
        ConvL c{Ci, Co, S, off, off + (size_t)Co * Ci * 9};
        off = c.b_off + Co;
        vec.push_back(c);
    };
    for (int l = 0; l < levels; ++l) {
        u->ch.push_back(base_channels << l);
        u->side.push_back(side >> l);
    }
    u->dec_c.resize(levels);
    u->dec_d.resize(levels);
    for (int l = 0; l < levels; ++l) {
        add(u->enc_a, l == 0 ? in_channels : u->ch[l - 1], u->ch[l], u->side[l]);
        add(u->enc_b, u->ch[l], u->ch[l], u->side[l]);
    }
    for (int l = levels - 2; l >= 0; --l) {
        std::vector<ConvL> tmp;
        add(tmp, u->ch[l + 1] + u->ch[l], u->ch[l], u->side[l]);
        add(tmp, u->ch[l], u->ch[l], u->side[l]);
        u->dec_c[l] = tmp[0];
        u->dec_d[l] = tmp[1];
    }
    u->out_w = off;
    u->out_b = off + base_channels;
    u->n_par = u->out_b + 1;
    // tensor-core packing of every eligible layer and direction
    std::vector<PackEntry> ents;
    auto pack = [&](ConvL &c) {
        if (tc_shape(c.Ci, c.Co)) {
            PackEntry e{u->pk_total, c.w_off, c.Ci, c.Co, c.Ci, c.Co, tc_nt(c.Co),
                        (c.Ci + TC_CK - 1) / TC_CK, 0, 0};
            e.count = (size_t)(c.Co / e.NT) * e.nstage * e.NT * 288;
            c.pk_fwd = u->pk_total;
            u->pk_total += e.count;
            ents.push_back(e);
        }
        if (tc_shape(c.Co, c.Ci)) {
            PackEntry e{u->pk_total, c.w_off, c.Co, c.Ci, c.Ci, c.Co, tc_nt(c.Ci),
                        (c.Co + TC_CK - 1) / TC_CK, 1, 0};
            e.count = (size_t)(c.Ci / e.NT) * e.nstage * e.NT * 288;
            c.pk_bwd = u->pk_total;
            u->pk_total += e.count;
            ents.push_back(e);
        }
    };
    for (auto &c : u->enc_a) pack(c);
    for (auto &c : u->enc_b) pack(c);
    for (int l = 0; l + 1 < levels; ++l) {
        pack(u->dec_c[l]);
        pack(u->dec_d[l]);
    }
    u->n_pk = (int)ents.size();
    // He-normal weights (fan-in), zero biases
    std::vector<float> h(u->n_par, 0.f);
    std::mt19937_64 rng(seed);
    std::normal_distribution<float> nd(0.f, 1.f);
    auto init = [&](const ConvL &c) {
        const float sd = std::sqrt(2.f / (float)(c.Ci * 9));
        for (size_t i = 0; i < (size_t)c.Co * c.Ci * 9; ++i) h[c.w_off + i] = sd * nd(rng);
    };
    for (auto &c : u->enc_a) init(c);
    for (auto &c : u->enc_b) init(c);
    for (int l = 0; l + 1 < levels; ++l) {
        init(u->dec_c[l]);
        init(u->dec_d[l]);
    }
    for (int c = 0; c < base_channels; ++c) h[u->out_w + c] = std::sqrt(1.f / base_channels) * nd(rng);
    bool ok = true;
    auto F = [&](size_t n) {
        float *p = dalloc<float>(u, n);
        ok = ok && p;
        return p;
    };
    u->par = F(u->n_par);
    u->grad = F(u->n_par);
    u->m = F(u->n_par);
    u->v = F(u->n_par);
    u->parb = dalloc<__nv_bfloat16>(u, u->n_par);
    ok = ok && u->parb;
    if (u->pk_total) {
        u->wpk = F(u->pk_total);
        u->pk_ent = dalloc<PackEntry>(u, ents.size());
        ok = ok && u->pk_ent;
    }
    const size_t N = max_batch;
    for (int l = 0; l < levels; ++l) {
        const size_t S2 = (size_t)u->side[l] * u->side[l], c = u->ch[l];
        const size_t ct = l + 1 < levels ? (size_t)u->ch[l + 1] + c : c;
        u->ea.push_back(F(N * c * S2));
        u->e.push_back(F(N * c * S2));
        u->pool.push_back(l + 1 < levels ? F(N * c * S2 / 4) : nullptr);
        u->cat.push_back(l + 1 < levels ? F(N * ct * S2) : nullptr);
        u->da.push_back(l + 1 < levels ? F(N * c * S2) : nullptr);
        u->d.push_back(l + 1 < levels ? F(N * c * S2) : nullptr);
        u->Ga.push_back(F(N * ct * S2));
        u->Gb.push_back(F(N * c * S2));
        u->Gc.push_back(F(N * c * S2));
        u->Gd.push_back(F(N * c * S2));
        u->Gs.push_back(F(N * c * S2));
    }
    u->outb = F(N * side * side);
    u->dout = F(N * side * side);
    u->loss = dalloc<double>(u, 1);
    ok = ok && u->loss;
    if (!ok) {
        delete u;
        set_error("unet_create: device allocation failed");
        return MSOT_ENOMEM;
    }
    cudaError_t e = cudaMemcpy(u->par, h.data(), sizeof(float) * u->n_par, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && u->n_pk)
        e = cudaMemcpy(u->pk_ent, ents.data(), sizeof(PackEntry) * ents.size(),
                       cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(u->m, 0, sizeof(float) * u->n_par);
    if (e == cudaSuccess) e = cudaMemset(u->v, 0, sizeof(float) * u->n_par);
    if (e != cudaSuccess) {
        delete u;
        set_error("unet_create: %s", cudaGetErrorString(e));
        return MSOT_ECUDA;
    }
    KLAUNCH(k_to_bf16<<<nblk(u->n_par), 256>>>(u->par, u->parb, u->n_par));
    if (int rc = pack_weights(u, 0)) {
        delete u;
        return rc;
    }
    *out = u;
    return MSOT_OK;
}

int msot_unet_destroy(msot_unet_t u) {
    delete u;
    return MSOT_OK;
}

int msot_unet_param_count(msot_unet_t u, size_t *n) {
    if (!u || !n) {
        set_error("unet_param_count: null argument");
        return MSOT_EINVAL;
    }
    *n = u->n_par;
    return MSOT_OK;
}

int msot_unet_get_params(msot_unet_t u, float *host) {
    if (!u || !host) {
        set_error("unet_get_params: null argument");
        return MSOT_EINVAL;
    }
    MSOT_CUDA_TRY(cudaMemcpy(host, u->par, sizeof(float) * u->n_par, cudaMemcpyDeviceToHost));
    return MSOT_OK;
}

int msot_unet_set_params(msot_unet_t u, const float *host) {
    if (!u || !host) {
        set_error("unet_set_params: null argument");
        return MSOT_EINVAL;
    }
    MSOT_CUDA_TRY(cudaMemcpy(u->par, host, sizeof(float) * u->n_par, cudaMemcpyHostToDevice));
    KLAUNCH(k_to_bf16<<<nblk(u->n_par), 256>>>(u->par, u->parb, u->n_par));
    MSOT_LAUNCH_CHECK();
    if (int rc = pack_weights(u, 0)) return rc;
    MSOT_CUDA_TRY(cudaDeviceSynchronize());
    return MSOT_OK;
}

int msot_unet_forward(msot_unet_t u, const float *d_in, float *d_out, int n, void *stream) {
    int rc = check_net(u, n, d_in, d_out);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    if ((rc = forward(u, d_in, n, st))) return rc;
    MSOT_CUDA_TRY(cudaMemcpyAsync(d_out, u->outb, sizeof(float) * n * u->S * u->S,
                                  cudaMemcpyDeviceToDevice, st));
    return MSOT_OK;
}

int msot_unet_gradients(msot_unet_t u, const float *d_in, const float *d_target, int n,
                        double *loss, float *host_grad, void *stream) {
    int rc = check_net(u, n, d_in, d_target);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    if ((rc = forward(u, d_in, n, st))) return rc;
    if ((rc = backward(u, d_in, d_target, n, st))) return rc;
    if (loss)
        MSOT_CUDA_TRY(cudaMemcpyAsync(loss, u->loss, sizeof(double), cudaMemcpyDeviceToHost, st));
    if (host_grad)
        MSOT_CUDA_TRY(cudaMemcpyAsync(host_grad, u->grad, sizeof(float) * u->n_par,
                                      cudaMemcpyDeviceToHost, st));
    MSOT_CUDA_TRY(cudaStreamSynchronize(st));
    return MSOT_OK;
}

int msot_unet_check(msot_unet_t u) {
    if (!u) {
        set_error("unet_check: null net");
        return MSOT_EINVAL;
    }
    MSOT_CUDA_TRY(cudaDeviceSynchronize());
    int flag = 0;
    MSOT_CUDA_TRY(cudaMemcpyFromSymbol(&flag, g_unet_tc_err, sizeof(int)));
    if (flag) {
        const int zero = 0;
        MSOT_CUDA_TRY(cudaMemcpyToSymbol(g_unet_tc_err, &zero, sizeof(int)));
        set_error("unet: a tensor-core convolution timed out waiting for its MMAs");
        return MSOT_ECUDA;
    }
    return MSOT_OK;
}

int msot_unet_adam_step(msot_unet_t u, double lr, int step, void *stream) {
    if (!u || step < 1 || !(lr > 0)) {
        set_error("unet_adam_step: bad arguments");
        return MSOT_EINVAL;
    }
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - std::pow(b1, (float)step), c2 = 1.f - std::pow(b2, (float)step);
    KLAUNCH(k_adam<<<nblk(u->n_par), 256, 0, (cudaStream_t)stream>>>(
        u->par, u->grad, u->m, u->v, u->parb, u->n_par, (float)lr, b1, b2, 1e-8f, c1, c2));
    MSOT_LAUNCH_CHECK();
    return pack_weights(u, (cudaStream_t)stream);
}

}  // extern "C"
