// gemm_tc.cu -- FP32-accurate GEMM on the sm_103a tensor cores:
//   C (M x N) = alpha * A (M x K) * B (K x N), all column-major FP32.
// Used for the dense products of backproject_waveeq.m:33 (K(t, t') times the
// radial integrals) and of the pre-processing's zero-phase filter (the T x T
// circulant of ifft(|H|^2), filter_butter_zero_phase.m:42-48).
//
// Precision: each operand is split into a TF32 head and a TF32 tail
// (x = hi + lo, hi = tf32(x), lo = tf32(x - hi)) and the product is
// hi*hi + hi*lo + lo*hi, three tcgen05.mma kind::tf32 per K step with FP32
// accumulation in TMEM: about 2^-21 relative per product, the order of a
// plain FP32 GEMM.
//
// CTA = one 128 x 128 tile of C, 256 threads.  K runs in stages of 32: the
// threads load the A and B panels of the next stage into registers while the
// tensor cores work on the current one, split them and store the four
// panels (A hi / lo, B hi / lo) in shared memory in the canonical K-major,
// no-swizzle layout (8-row x 16-byte core matrices; the 16 core matrices of
// a 4-wide K group are contiguous, K groups 2048 bytes apart).  Two buffers
// of 64 KB alternate; thread 0 issues the 12 MMAs of a stage and commits
// them to the buffer's mbarrier, which the stage two later waits for before
// it overwrites the buffer.  Every wait is bounded; a timeout sets an error
// flag (tc_sgemm_check), writes the tile as NaN and still frees the TMEM.
#include <atomic>

#include "common.cuh"
#include "ptx.cuh"

namespace msot {

namespace {

constexpr int GT = 128;          // tile rows (M) and columns (N)
constexpr int GK = 32;           // K per stage
constexpr int G_THREADS = 256;
constexpr int G_KGROUP = 2048;   // bytes between 4-wide K groups of one panel
constexpr int G_PANEL = (GK / 4) * G_KGROUP;  // 16 KB: one 128 x 32 panel
constexpr int G_STAGE = 4 * G_PANEL;          // A hi, A lo, B hi, B lo
constexpr size_t G_SMEM = 2 * (size_t)G_STAGE;

__device__ int g_gemm_err = 0;

__device__ __forceinline__ uint64_t g_mdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    // start (16 B units) | LBO << 16 | SBO << 32 | descriptor version 1 at
    // bit 46; base offset 0, no swizzle
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}
// instruction descriptor: D F32, A and B TF32, both K-major, N >> 3 at bit
// 17, M >> 4 at bit 24
__host__ __device__ constexpr uint32_t g_idesc(int M, int N) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) |
           ((uint32_t)(M >> 4) << 24);
}
__device__ __forceinline__ float g_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

// registers of one stage: A rows m = tid % 128, K groups tid / 128 + 2 j;
// B column n = g_bcol(tid), K groups 4 g_bhalf(tid) + j.  Eight consecutive
// threads take eight consecutive columns of the same K group, so that each
// 8-thread phase of a 16-byte shared store fills one 128-byte core matrix
// (no bank conflicts).
struct GRegs {
    float4 a[4], b[4];
};
__device__ __forceinline__ int g_bcol(int tid) { return (tid & 7) | ((tid >> 4) << 3); }
__device__ __forceinline__ int g_bhalf(int tid) { return (tid >> 3) & 1; }

__device__ __forceinline__ void g_load(GRegs &R, const float *A, int lda, const float *B, int ldb,
                                       int M, int N, int K, int m0, int n0, int k0, bool bvec) {
    const int tid = threadIdx.x;
    {
        const int m = m0 + tid % GT;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int k = k0 + 4 * (tid / GT + 2 * j);
            float v[4];
#pragma unroll
            for (int c = 0; c < 4; ++c)
                v[c] = (m < M && k + c < K) ? __ldg(A + (size_t)(k + c) * lda + m) : 0.f;
            R.a[j] = make_float4(v[0], v[1], v[2], v[3]);
        }
    }
    {
        const int n = n0 + g_bcol(tid);
        const float *col = B + (size_t)n * ldb;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int k = k0 + 4 * (4 * g_bhalf(tid) + j);
            if (n < N && bvec && k + 3 < K) {
                R.b[j] = __ldg(reinterpret_cast<const float4 *>(col + k));
            } else {
                float v[4];
#pragma unroll
                for (int c = 0; c < 4; ++c) v[c] = (n < N && k + c < K) ? __ldg(col + k + c) : 0.f;
                R.b[j] = make_float4(v[0], v[1], v[2], v[3]);
            }
        }
    }
}

__device__ __forceinline__ void g_split_store(const float4 &v, uint8_t *hi, uint8_t *lo,
                                              uint32_t off) {
    const float4 h = make_float4(g_tf32(v.x), g_tf32(v.y), g_tf32(v.z), g_tf32(v.w));
    const float4 l = make_float4(g_tf32(v.x - h.x), g_tf32(v.y - h.y), g_tf32(v.z - h.z),
                                 g_tf32(v.w - h.w));
    *reinterpret_cast<float4 *>(hi + off) = h;
    *reinterpret_cast<float4 *>(lo + off) = l;
}

// element (row r, K group g) of a panel: core matrix (r / 8, g), row r % 8
__device__ __forceinline__ uint32_t g_off(int r, int g) {
    return (uint32_t)(g * G_KGROUP + (r >> 3) * 128 + (r & 7) * 16);
}

__device__ __forceinline__ void g_store(const GRegs &R, uint8_t *stage) {
    const int tid = threadIdx.x;
    uint8_t *ahi = stage, *alo = stage + G_PANEL, *bhi = stage + 2 * G_PANEL,
            *blo = stage + 3 * G_PANEL;
#pragma unroll
    for (int j = 0; j < 4; ++j) g_split_store(R.a[j], ahi, alo, g_off(tid % GT, tid / GT + 2 * j));
#pragma unroll
    for (int j = 0; j < 4; ++j)
        g_split_store(R.b[j], bhi, blo, g_off(g_bcol(tid), 4 * g_bhalf(tid) + j));
}

__global__ void __launch_bounds__(G_THREADS, 1) k_gemm_3xtf32(
    int M, int N, int K, float alpha, const float *__restrict__ A, int lda,
    const float *__restrict__ B, int ldb, float *__restrict__ C, int ldc, int bvec) {
    extern __shared__ __align__(1024) uint8_t g_smem[];
    __shared__ __align__(8) uint64_t mbar[2];  // MMAs of buffer 0 / 1 done
    __shared__ uint32_t tmem_slot;
    const int m0 = blockIdx.x * GT, n0 = blockIdx.y * GT;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(&tmem_slot)),
                     "r"((uint32_t)GT));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (threadIdx.x == 32) {
        mbar_init(smem_u32(&mbar[0]), 1);
        mbar_init(smem_u32(&mbar[1]), 1);
        mbar_init_fence();
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tm = tmem_slot;
    const int ns = (K + GK - 1) / GK;
    bool ok = true;
    int issued = 0;  // stages whose MMAs were committed
    GRegs R;
    g_load(R, A, lda, B, ldb, M, N, K, m0, n0, 0, bvec != 0);
    for (int s = 0; s < ns; ++s) {
        const int buf = s & 1;
        uint8_t *stage = g_smem + buf * G_STAGE;
        if (s >= 2) {  // the MMAs of stage s - 2 must be done with this buffer
            const bool mine = mbar_wait_bounded(smem_u32(&mbar[buf]), (uint32_t)((s - 2) >> 1) & 1u);
            ok = !__syncthreads_or(!mine);
            if (!ok) break;
        }
        g_store(R, stage);
        // generic-proxy stores -> visible to the tensor core (async proxy)
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (s + 1 < ns) g_load(R, A, lda, B, ldb, M, N, K, m0, n0, (s + 1) * GK, bvec != 0);
        if (threadIdx.x == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t base = smem_u32(stage);
            constexpr uint32_t idesc = g_idesc(GT, GT);
#pragma unroll
            for (int kk = 0; kk < GK / 8; ++kk) {
                const uint32_t koff = (uint32_t)(2 * kk * G_KGROUP);
                const uint64_t ahi = g_mdesc(base + koff, G_KGROUP, 128);
                const uint64_t alo = g_mdesc(base + G_PANEL + koff, G_KGROUP, 128);
                const uint64_t bhi = g_mdesc(base + 2 * G_PANEL + koff, G_KGROUP, 128);
                const uint64_t blo = g_mdesc(base + 3 * G_PANEL + koff, G_KGROUP, 128);
                const uint64_t da[3] = {ahi, ahi, alo}, db[3] = {bhi, blo, bhi};
#pragma unroll
                for (int p = 0; p < 3; ++p) {
                    const uint32_t acc = (s | kk | p) != 0;
                    asm volatile(
                        "{\n\t.reg .pred q;\n\t"
                        "setp.ne.b32 q, %4, 0;\n\t"
                        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, q;\n\t}\n" ::"r"(tm),
                        "l"(da[p]), "l"(db[p]), "r"(idesc), "r"(acc));
                }
            }
            asm volatile(
                "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                    smem_u32(&mbar[buf]))
                : "memory");
        }
        issued = s + 1;
    }
    // the last commit covers every MMA issued before it
    if (ok && issued > 0) {
        const bool mine = mbar_wait_bounded(smem_u32(&mbar[(issued - 1) & 1]),
                                            (uint32_t)((issued - 1) >> 1) & 1u);
        ok = !__syncthreads_or(!mine);
    }
    if (!ok) {
        if (threadIdx.x == 0) atomicExch(&g_gemm_err, 1);
        // one more bounded wait for the MMAs in flight before the TMEM and
        // the shared memory are released
        if (issued > 0)
            mbar_wait_bounded(smem_u32(&mbar[(issued - 1) & 1]), (uint32_t)((issued - 1) >> 1) & 1u);
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    // epilogue: warp w reads TMEM lanes 32 (w % 4) .. + 31 (rows m) and
    // columns 64 (w / 4) .. + 63 (n); lanes run along m (coalesced stores)
    const int m = m0 + (warp & 3) * 32 + lane;
#pragma unroll 1
    for (int j0 = (warp >> 2) * 64; j0 < (warp >> 2) * 64 + 64; j0 += 16) {
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
        if (m < M) {
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const int n = n0 + j0 + j;
                // a tile whose MMAs timed out is written as NaN, never as
                // a plausible value
                if (n < N)
                    C[(size_t)n * ldc + m] =
                        ok ? alpha * __uint_as_float(r[j]) : __int_as_float(0x7fc00000);
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tm),
                     "r"((uint32_t)GT));
}

}  // namespace

int tc_sgemm(int M, int N, int K, float alpha, const float *A, int lda, const float *B, int ldb,
             float *C, int ldc, cudaStream_t st) {
    if (M <= 0 || N <= 0 || K <= 0 || !A || !B || !C || lda < M || ldb < K || ldc < M) {
        set_error("tc_sgemm: bad arguments");
        return MSOT_EINVAL;
    }
    const cudaError_t e = raise_max_dynamic_smem((const void *)k_gemm_3xtf32, G_SMEM);
    if (e != cudaSuccess) {
        set_error("tc_sgemm: cudaFuncSetAttribute: %s", cudaGetErrorString(e));
        return MSOT_ECUDA;
    }
    // 16-byte B column loads when every column starts 16-byte aligned
    const int bvec = ((reinterpret_cast<uintptr_t>(B) & 15) == 0 && ldb % 4 == 0) ? 1 : 0;
    const dim3 grid((unsigned)div_up(M, GT), (unsigned)div_up(N, GT));
    if (grid.y > 65535u) {
        set_error("tc_sgemm: N = %d too large for one launch", N);
        return MSOT_EINVAL;
    }
    KLAUNCH(k_gemm_3xtf32<<<grid, G_THREADS, G_SMEM, st>>>(M, N, K, alpha, A, lda, B, ldb, C, ldc,
                                                           bvec));
    MSOT_LAUNCH_CHECK();
    return MSOT_OK;
}

int tc_sgemm_check() {
    int v = 0;
    MSOT_CUDA_TRY(cudaMemcpyFromSymbol(&v, g_gemm_err, sizeof v));
    if (v) {
        const int z = 0;
        cudaMemcpyToSymbol(g_gemm_err, &z, sizeof z);
        set_error("tc_sgemm: a bounded wait for the tensor cores ran out");
        return MSOT_ETIMEOUT;
    }
    return MSOT_OK;
}

}  // namespace msot
