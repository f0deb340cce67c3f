// common.cuh -- shared definitions of the sm_103a MSOT operator library.
//
// Device-side data layout (all device memory, built once per plan):
//   tau_tiles  int32 [n_patch][n_det][PATCH]   travel time of pixel q of patch
//              (8x8 pixels) to detector d, fixed point Q(frac_bits); padding
//              pixels hold TAU_PAD.  Read by the gather kernels (transpose).
//   tau_pi     int32 [n_det][P]                travel times with the pixels in a
//              fixed pseudo-random order perm[] (scatter kernels).
//   ir_fwd/ir_adj float [L]                    IR taps (and flipped) times 1/norm.
//   pre_x/pre_z float [2K+1]                   circular prefilter taps.
//   sir        float [n_sir][S], sir_se int2 [n_sir] (0-based inclusive),
//   sir_tiles  int32 [n_patch][n_det][PATCH]   SIR column per (pixel, detector),
//   sir_pi     int32 [n_det][P]                the same in scatter order.
// Batched vectors are instance-major FP32: image [W][nx][nz], sinogram
// [W][n_det][n_t].
#pragma once

#include <atomic>
#include <cstdint>
#include <cstdio>
#include <cuda_runtime.h>
#include <vector>

#include "../../include/msot_gpu.h"

namespace msot {

constexpr int PATCH_X = 8;           // patch width (x columns)
constexpr int PATCH_Z = 8;           // patch height (z rows)
constexpr int PATCH = PATCH_X * PATCH_Z;
constexpr int32_t TAU_PAD = INT32_MIN;  // marks a padding pixel in tau_tiles
constexpr int BLK_X = 64, BLK_Z = 64, BLK = BLK_X * BLK_Z;  // adjoint pixel block
constexpr int BLK_THREADS = 256, BLK_PPT = BLK / BLK_THREADS;  // 16 pixels per thread

struct Plan {
    int device = -1;   // CUDA device the plan's tables live on (current at creation)
    int nx, nz, P, D, T;
    double radius;
    int frac_bits;     // fixed-point fraction bits of tau
    int32_t r_fx;      // radius in fixed point
    float c1;          // 2^-frac_bits / radius
    int n_tap;         // upper bound of taps per (pixel, detector): floor(2r) + 2
    int n_patch_x, n_patch_z, n_patch;
    // tables
    int32_t *tau_tiles = nullptr;  // [n_patch][D][PATCH] (gather kernels)
    int32_t *tau_pi = nullptr;     // [D][P] pixels in scatter order perm[] (SIR)
    int32_t *perm = nullptr;       // [P] scatter order -> pixel index (SIR)
    // bucket decomposition of the tri interpolation (no SIR): for tau = b + f
    // (b integer, 0 <= f < 1) the weights of taps b-F+1 .. b+F are exactly
    // linear in f and only taps b-F and b+F+1 need the clamp at zero.
    int F = 0;                     // floor(radius)
    float inv_r = 0.f;             // 1 / radius
    float ce1 = 0.f, ce2 = 0.f;    // (r - F)/r and (F + 1 - r)/r
    int32_t *fwd_off = nullptr;    // [D][T+1] CSR offsets of bucket b = floor(tau)
    int2 *fwd_ent = nullptr;       // [D][P] (tau fixed point, pixel) sorted by bucket
    // the same entries per (detector, time tile of the forward, warp of 32
    // buckets), interleaved: row k holds the k-th entry of each of the warp's
    // buckets ((0, -1) past a bucket's end), so that a warp's entry load is
    // 256 contiguous bytes; fwd_ell_off[(d * ntiles + tile) * 8 + warp] is a
    // block's first entry (the next block's start ends it)
    int2 *fwd_ell = nullptr;
    int32_t *fwd_ell_off = nullptr;
    int fwd_ell_tiles = 0;
    // staged forward (das_fwd_staged.cu): CTA = (time tile of st_tt samples,
    // group of st_g detectors); st_tt == 0 when the plan has no such tables
    int st_tt = 0, st_g = 0, st_ntiles = 0, st_ngroups = 0, st_ib = 0;
    int st_umax = 0;               // largest pixel union of a CTA
    int st_ent_cap = 0;            // largest entry count of a CTA, rounded up to 4
    int st_off_stride = 0;         // ints per CTA in st_off
    int st_threads = 0;            // threads per CTA
    int4 *st_info = nullptr;       // [n_cta] {u_off, nU, e_off, n_ent}
    int32_t *st_u = nullptr;       // pixel unions, ascending per CTA
    int32_t *st_off = nullptr;     // [n_cta][st_off_stride] entry offsets per (detector, bucket)
    uint32_t *st_ent = nullptr;    // entries (tau fraction << st_ib) | index in the union
    // adjoint pixel blocks of BLK_Z x BLK_X pixels; thread t of a CTA owns
    // the pixels (iz = t % BLK_Z, ix = t / BLK_Z + 4k), k < BLK_PPT
    int n_blk_x = 0, n_blk_z = 0, n_blk = 0;
    int32_t *blk_tau = nullptr;    // [n_blk][D][BLK_PPT][BLK_THREADS] (TAU_PAD outside)
    int2 *blk_span = nullptr;      // [n_blk][D] first / last bucket of the block
    int blk_span_max = 0;          // largest last - first + 1
    int adj_groups_max = 0;        // detector groups the partial buffer is sized for
    float *scr_part = nullptr;     // [adj_groups_max][max_batch][P] adjoint partial sums
    struct SolverCache *solver = nullptr;  // solver workspace and captured CUDA graphs
    // variants chosen by msot_autotune for this plan (0 = the built-in choice)
    int tune_fwd_wt = 0;      // instances per CTA of the DAS forward (8, 4, 2)
    int tune_adj_wt = 0;      // instances per CTA of the DAS adjoint (2, 1)
    int tune_conv_mb = 0;     // register cap of the IR convolution (1, 3, 4)
    int tune_tv_cluster = 0;  // CTAs per image of the SB_ITV2 cluster kernel
    int tune_fwd_staged = 0;  // DAS forward kernel: 1 staged, 2 k_das_fwd3 (CSR), 4 k_das_fwd3 (ELL), 0 = knobs
    // reduced storage (msot_plan_set_storage): the interpolation input of the
    // DAS forward in BF16 (1) or FP16 with a power-of-two scale per instance
    // (2), FP32 accumulation; mutable so that a solver can run its
    // full-precision refinement iterations with it off
    mutable int image_fmt = 0;   // in effect now: 0 FP32, 1 BF16, 2 FP16
    int storage_fmt = 0;         // requested
    int refine_every = 0;        // L1 solver: every refine_every-th outer iteration in FP32
    float *h16_sc = nullptr;     // FP16: [max_batch] scales s, then [max_batch] 1 / s
    float pre_gain_x = 1.f, pre_gain_z = 1.f;  // sum |taps| of the prefilter axes
    // IR
    int L = 0, Lh = 0;
    float *ir_fwd = nullptr, *ir_adj = nullptr;
    // overlap-save FFT convolution: N-point complex FFTs (N = 4^log4n), two real
    // columns per transform; spectra of the (flipped) taps scaled by 1/(N norm)
    int fft_log4n = 0;
    float2 *fft_tw = nullptr;    // [N] exp(-2 pi i t / N)
    float2 *fft_hf = nullptr;    // [N] spectrum of ir_fwd / N
    float2 *fft_ha = nullptr;    // [N] spectrum of ir_adj / N
    // the same for the split-complex 1024-point kernel (N = 1024 only): per
    // register pair m and lane, (re a, re b, im a, im b) of w^(lane k1) for
    // k1 = brev5(2m), brev5(2m + 1); conj w^(lane n) for n = 2m, 2m + 1; and
    // H[lane + 32 k2] for k2 = brev5(2m), brev5(2m + 1)  ([16][32] each)
    float4 *fft_twb = nullptr, *fft_twn = nullptr, *fft_hfb = nullptr, *fft_hab = nullptr;
    // prefilter
    int Kx = -1, Kz = -1;   // -1: no prefilter along that axis
    float *pre_x = nullptr, *pre_z = nullptr;
    double norm = 1.0;
    float scale = 1.f;      // 1/norm
    // SIR
    int S = 0, NS = 0;
    float *sir = nullptr;
    int2 *sir_se = nullptr;        // [NS] 0-based inclusive start/end
    int32_t *sir_tiles = nullptr;  // [n_patch][D][PATCH] 0-based SIR column
    int32_t *sir_pi = nullptr;     // [D][P] SIR column in scatter order
    // scratch for the operator chains
    int max_batch = 0;
    float *scr_img0 = nullptr, *scr_img1 = nullptr;  // [max_batch][P]
    float *scr_sino = nullptr;                       // [max_batch][D][T]
    size_t device_bytes = 0;
};

const char *set_error(const char *fmt, ...);
// Raises a kernel's maximum dynamic shared memory to `bytes` if it is below
// (never lowers it): the attribute is process-wide per function, so plans of
// different sizes used from several threads must not shrink it between
// another thread's setting and launch.  Thread-safe.  plan.cu
cudaError_t raise_max_dynamic_smem(const void *func, size_t bytes);
// a kernel's dynamic shared memory limit raised to `bytes` where above 48 KB
template <class K>
inline int set_smem(K kern, size_t bytes) {
    if (bytes > 48 * 1024) {
        cudaError_t e = raise_max_dynamic_smem((const void *)kern, bytes);
        if (e != cudaSuccess) {
            set_error("cudaFuncSetAttribute(smem=%zu): %s", bytes, cudaGetErrorString(e));
            return MSOT_ECUDA;
        }
    }
    return MSOT_OK;
}
// k_das_fwd3 launches per storage format of the interpolation input (xpm of
// FP32, BF16 or FP16 values; inv_s: the FP16 inverse scales, else null)
int das_fwd_run_f32(const Plan &pl, const void *xpm, float *raw, int W, float scale,
                    const float *inv_s, bool ell, int wt, cudaStream_t st);
int das_fwd_run_bf16(const Plan &pl, const void *xpm, float *raw, int W, float scale,
                     const float *inv_s, bool ell, int wt, cudaStream_t st);
int das_fwd_run_f16(const Plan &pl, const void *xpm, float *raw, int W, float scale,
                    const float *inv_s, bool ell, int wt, cudaStream_t st);


// tensor-core convolutions of the warm-start U-Net on (1) or off (0); unet.cu
extern std::atomic<int> g_unet_tc;
// register cap (minimum resident CTAs per SM) of the IR convolution; operator.cu
// DAS forward on the interleaved entry table for plans not autotuned; operator.cu
extern std::atomic<int> g_fwd_ell;
extern std::atomic<int> g_conv_min_blocks;
// next-detector register prefetch of the DAS adjoint on (1) or off (0); operator.cu
extern std::atomic<int> g_adj_prefetch;

// launch counter (every kernel launch of the library goes through KLAUNCH)
extern std::atomic<long long> g_launch_count;
#define KLAUNCH(...) (++::msot::g_launch_count, __VA_ARGS__)

// kernel families timed by TimedScope when profiling is enabled
enum KernelId {
    KID_PREFILTER = 0,
    KID_INTERP_FWD = 1,
    KID_INTERP_ADJ = 2,
    KID_CONV = 3,
    KID_VECTOR = 4,
    KID_PERMUTE = 5,
    KID_TV_PROX = 6,
    KID_COUNT = 7
};

// Records a CUDA event pair around the launches in its scope (on stream st)
// when profiling is enabled (msot_profile_enable); otherwise does nothing.
class TimedScope {
  public:
    TimedScope(int kid, cudaStream_t st);
    ~TimedScope();
    TimedScope(const TimedScope &) = delete;
    TimedScope &operator=(const TimedScope &) = delete;

  private:
    int kid_;
    cudaStream_t st_;
    long slot_;
};

#define MSOT_CUDA_TRY(expr)                                                            \
    do {                                                                               \
        cudaError_t e_ = (expr);                                                       \
        if (e_ != cudaSuccess) {                                                       \
            ::msot::set_error("%s:%d %s: %s", __FILE__, __LINE__, #expr,               \
                              cudaGetErrorString(e_));                                 \
            return MSOT_ECUDA;                                                         \
        }                                                                              \
    } while (0)

#define MSOT_LAUNCH_CHECK()                                                            \
    do {                                                                               \
        cudaError_t e_ = cudaGetLastError();                                           \
        if (e_ != cudaSuccess) {                                                       \
            ::msot::set_error("%s:%d launch: %s", __FILE__, __LINE__,                  \
                              cudaGetErrorString(e_));                                 \
            return MSOT_ECUDA;                                                         \
        }                                                                              \
    } while (0)

// operator chains (operator.cu)
int launch_prefilter(const Plan &pl, const float *in, float *out, int W, bool transpose,
                     bool along_x, float scale, int out_mode, cudaStream_t st);
int launch_to_pixmajor(const Plan &pl, const float *in, float *out, int W, cudaStream_t st);
int launch_permute(const Plan &pl, const float *in, float *out, int W, cudaStream_t st);
int launch_das_forward(const Plan &pl, const float *x_pi, float *raw, int W, float scale,
                       cudaStream_t st);
int launch_das_adjoint(const Plan &pl, const float *raw, float *x, int W, float scale,
                       cudaStream_t st);
int launch_conv(const Plan &pl, const float *in, float *out, int W, bool transpose,
                cudaStream_t st);
int launch_sir_forward(const Plan &pl, const float *x_pi, float *raw, int W, float scale,
                       cudaStream_t st);
int launch_sir_adjoint(const Plan &pl, const float *raw, float *x, int W, float scale,
                       cudaStream_t st);
int interp_forward(const Plan &pl, const float *x_pi, float *raw, int W, float scale,
                   cudaStream_t st);
int interp_adjoint(const Plan &pl, const float *raw, float *x, int W, float scale,
                   cudaStream_t st);
int apply_forward(const Plan &pl, const float *img, float *sino, int W, cudaStream_t st);

// Per-group scalars of the Krylov solvers (one group = one instance, or the
// whole batch when coupled).
struct Scal {
    double alpha, beta, c, s, phibar, normr, normrmin, normb;
    double rho, thet, phi, gamma;  // gamma = alpha / beta_prev
    double rho_cg, rho1_cg, alpha_cg;
    int done, improved, pad0, pad1;
};

// Forward operator with the LSQR sinogram update fused into the EIR
// convolution's epilogue (y = A img never stored):
//   mode 0: u = sl*b - sl*y ; mode 1: u = sl*y - gamma*u (u kept where done)
// and per-block partial sums of u^2 in part[w * nparts + slot].  Returns 1
// (nothing launched) when the plan's convolution path cannot fuse it.
int apply_forward_update(const Plan &pl, const float *img, float *u, const float *b, int W,
                         int mode, float sl, const Scal *sc, int coupled, double *part,
                         int *nparts, cudaStream_t st);
bool forward_update_fusable(const Plan &pl, int W);
void solver_cache_free(Plan &pl);  // solver.cu
void solver_cache_invalidate(Plan &pl);  // drops the captured solver graphs (solver.cu)
bool profiling_enabled();          // timing.cu
int apply_transpose(const Plan &pl, const float *sino, float *img, int W, cudaStream_t st);

inline int div_up(int a, int b) { return (a + b - 1) / b; }

// MSOT_OK when the current device is the one the plan was created on, else
// MSOT_EINVAL with a message naming `who`: every kernel of a call reads the
// plan's tables, which live on that device only.  plan.cu
int check_plan_device(const Plan &pl, const char *who);

// time tile / detector group forced on the staged forward tables of plans
// created from now on (0 = chosen by the plan); das_fwd_staged.cu
extern std::atomic<int> g_st_force_tt, g_st_force_g;
// staged DAS forward (das_fwd_staged.cu): builds the plan's st_* tables
// from the fixed-point travel times tfx [D][P] and the per-detector bucket
// CSR (foff [D][T+1], fent [D][P]); leaves st_tt = 0 when no tile shape fits
int build_fwd_staged(Plan &p, const int32_t *tfx, const int32_t *foff, const int2 *fent,
                     size_t &bytes);
// the host-side tables of the staged forward before upload
struct StTables {
    int tt = 0, g = 0, ntiles = 0, ngroups = 0, ib = 0, umax = 0, ent_cap = 0, off_stride = 0,
        threads = 0;
    std::vector<int4> info;
    std::vector<int32_t> ulist, offs;
    std::vector<uint32_t> ent;
};
int build_fwd_staged_host(const Plan &p, const int32_t *tfx, const int32_t *foff,
                          const int2 *fent, int dev_smem, StTables &t);
size_t st_smem_bytes(const Plan &p, int wt);
int st_x_words(const Plan &p, int wt);
bool fwd_staged_fits(const Plan &p, int wt);
// xt in the [W/wt][P][wt] layout of das_fwd_wt
int launch_das_forward_staged(const Plan &p, const float *xt, float *raw, int W, int wt,
                              float scale, cudaStream_t st);
// staged forward on (1, default) or off (0); operator.cu
extern std::atomic<int> g_fwd_staged;
// instances per CTA of the DAS forward at batch W: the interpolation input is
// laid out [W/wt][P][wt] (pixel-major within an instance tile).  operator.cu
int das_fwd_wt(const Plan &pl, int W);

// C (M x N) = alpha A (M x K) B (K x N), column-major FP32, on the tensor
// cores with a 3 x TF32 split (FP32-level accuracy); gemm_tc.cu
int tc_sgemm(int M, int N, int K, float alpha, const float *A, int lda, const float *B, int ldb,
             float *C, int ldc, cudaStream_t st);
// MSOT_ETIMEOUT (and clears the flag) when a tc_sgemm tile's bounded wait ran
// out since the last check; synchronises the device
int tc_sgemm_check();

// Streaming multiprocessors of the current device (queried once per device,
// cached; 1 if the query fails).  Launch heuristics size grids by it.  plan.cu
int sm_count();

}  // namespace msot

struct msot_plan {
    msot::Plan p;
};
