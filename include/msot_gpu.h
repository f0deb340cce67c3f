/*
 * msot_gpu.h -- C ABI of the GB300 (sm_103a) implementation of the
 * model-based MSOT operator A, its transpose, the non-negative solvers that
 * call them, and the two analytic reconstructors.
 *
 * Conventions
 *   - Every function returns an int status: MSOT_OK (0) or a negative
 *     MSOT_E* code; msot_last_error() gives a message for the calling thread.
 *     No C++ exception crosses this boundary.
 *   - Device pointers are CUDA device memory of the current device; `stream`
 *     is a cudaStream_t passed as void* (NULL = legacy default stream).
 *   - A plan belongs to the device that was current when it was created;
 *     a call on it with another device current returns MSOT_EINVAL.
 *   - Batched layouts are instance-major and FP32:
 *       image     [batch][nx][nz]       (pixel p = ix*nz + iz, MATLAB Nz x Nx)
 *       sinogram  [batch][n_det][n_t]   (MATLAB T x D x W)
 *     so one instance is one contiguous MATLAB image / sinogram.
 *   - Host-buffer entry points (msot_mex_*) take FP64 arrays in exactly the
 *     column-major layouts of the reference MEX functions and do all device
 *     transfers themselves.
 *   - A plan's tables are immutable after creation and the plan may be used
 *     from several host threads on different streams, except for the
 *     functions documented as using the plan's scratch (msot_forward,
 *     msot_transpose, msot_interp_transpose and the solvers, which also keep
 *     their captured graphs in the plan), which must not overlap on the GPU
 *     for one plan, and msot_autotune, which changes the plan's kernel
 *     choices and runs alone on it.
 */
#ifndef MSOT_GPU_H
#define MSOT_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MSOT_OK 0
#define MSOT_EINVAL -1     /* bad argument / shape / class */
#define MSOT_ERANGE -2     /* travel time or index out of the representable range */
#define MSOT_ECUDA -3      /* CUDA runtime error */
#define MSOT_ENOMEM -4     /* allocation failed */
#define MSOT_ENONFINITE -5 /* NaN/Inf in an input or a solver scalar */
#define MSOT_ETIMEOUT -6   /* a bounded device-side wait gave up */

typedef struct msot_plan *msot_plan_t;

/* Geometry and model tables of one MSOTmodel (MSOTmodel.m:18-48).
 * Replaces the model struct fields absoluteTravelTimeIndices,
 * circularInterpolationRadiusInSamples, IRHat/IRFlippedHat (as taps), the
 * Discretization prefilter (as separable circular taps), the normalisation
 * factor (MSOTmodel.m:271-287) and, when include_sir, SPMR / SPMRIndices /
 * SPMRTimestepIndexStartAndEnd (MSOTmodel.m:463-480). */
typedef struct msot_plan_desc {
    int nx, nz;               /* pixel grid: nx columns (x), nz rows (z) */
    int n_det, n_t;           /* detectors, time samples per detector */
    double radius;            /* interpolation radius in samples */
    const double *travel;     /* host [n_det][nx*nz] fractional sample indices (MATLAB P x D) */
    int ir_len;               /* odd; 0 = no IR convolution */
    const double *ir;         /* host IR taps (MSOTmodel.m:338-342) */
    int pre_len_x, pre_len_z; /* odd; 0 = no prefilter along that axis */
    const double *pre_x;      /* host circular kernel along x, centred */
    const double *pre_z;      /* host circular kernel along z, centred */
    double norm;              /* model normalisation factor; <= 0 means 1 */
    /* spatial impulse response (forwardMex.cpp:18-27); sir_len == 0 = none */
    int sir_len, n_sir;
    const double *sir;            /* host [n_sir][sir_len] (MATLAB S x NS) */
    const int32_t *sir_start_end; /* host [n_sir][2], 1-based inclusive */
    const int32_t *sir_idx;       /* host [n_det][nx*nz], 1-based */
    int max_batch;            /* largest batch the plan's scratch is sized for */
} msot_plan_desc;

const char *msot_last_error(void);
int msot_version(void);

int msot_plan_create(const msot_plan_desc *desc, msot_plan_t *plan);
int msot_plan_destroy(msot_plan_t plan);
/* Bytes of device memory the plan holds (tables + scratch). */
size_t msot_plan_device_bytes(msot_plan_t plan);

/* model.Funcs.applyForward (MSOTmodel.m:285 -> forwardWithoutSIR :208-222 or
 * forward :189-206): prefilter, interpolation (+SIR), IR convolution, 1/norm.
 * d_img [batch][nx][nz] -> d_sino [batch][n_det][n_t].  Uses plan scratch. */
int msot_forward(msot_plan_t plan, const float *d_img, float *d_sino, int batch, void *stream);

/* model.Funcs.applyTranspose (MSOTmodel.m:286 -> transposeWithoutSIR
 * :243-257 or transpose :224-241).  d_sino -> d_img.  Uses plan scratch. */
int msot_transpose(msot_plan_t plan, const float *d_sino, float *d_img, int batch, void *stream);

/* The bare interpolation operators, i.e. the MEX kernels on device FP32
 * data in the instance-major layouts above (no prefilter, IR or norm):
 *   forwardDelayAndSumMex.cpp:15 / forwardMex.cpp:16 (when the plan has SIR)
 *   transposeDelayAndSumMex.cpp:15 / transposeMex.cpp:16 */
int msot_interp_forward(msot_plan_t plan, const float *d_coeffs, float *d_raw, int batch,
                        void *stream);
int msot_interp_transpose(msot_plan_t plan, const float *d_raw, float *d_coeffs, int batch,
                          void *stream);

/* Reduced-precision storage (the mixed-precision configuration of the
 * reference's L1 solve; no counterpart in the reference, which is FP64
 * throughout).  The interpolation input of the DAS forward (the prefiltered
 * image the forwardDelayAndSumMex.cpp:80-100 loop reads per (pixel,
 * detector) pair) is stored in 16 bits and widened to FP32 for the FP32
 * accumulation, which halves the bytes the forward gathers:
 * image_format = 1: BF16, round to nearest; 2: FP16, round to nearest, of
 * the values times a power-of-two scale per instance (from the instance's
 * largest magnitude and the prefilter's gain, so that the stored values
 * stay below 2^14; the forward's output is multiplied back by the inverse,
 * exactly); 0: FP32 (default).  refine_every = k > 0: the L1 solver runs
 * every k-th outer iteration with the FP32 input (the other solvers use the
 * setting as is).  The FP32 default meets the operators' 1e-5 bar; 16-bit
 * storage is for solves held to their 1e-3 bar against the FP64 oracle.
 * Plans without SIR only; drops the plan's captured solver graphs. */
int msot_plan_set_storage(msot_plan_t plan, int image_format, int refine_every);

/* Allocation-free form of msot_interp_transpose for plans without SIR; no
 * counterpart in the reference.  It is for callers that are not allowed to
 * allocate device memory, e.g. a host application whose device memory is
 * owned by another allocator or that runs under a fixed memory budget.  Its
 * partial sums live in a 16 MiB array inside the library instead of the
 * plan's scratch, so the call performs no cudaMalloc / cudaFree.  The array
 * belongs to the library's operator module: it is allocated when CUDA loads
 * that module on a device and held there until the process exits.  Under
 * lazy module loading (CUDA's default) that load can be the first call of
 * this function on the device, so a caller with a fixed budget makes one
 * warm-up call (or sets CUDA_MODULE_LOADING=EAGER) before its budget
 * applies.  Limit: batch * nx * nz <= 4 Mi (4194304) elements, else
 * MSOT_ERANGE.  The first call on a device looks up the array's device
 * address (cudaGetSymbolAddress) with that device current and keeps it for
 * the process: this assumes the device's primary context (the CUDA runtime's
 * own), with no cudaDeviceReset afterwards; make that first call before any
 * stream capture.  The current device must be the plan's.  All calls share
 * the one array: calls that overlap on the GPU (other streams or threads)
 * race and must be serialised by the caller.  The detector groups differ
 * from msot_interp_transpose's, so the result equals it up to the order of
 * the FP32 partial sums, not bit for bit. */
int msot_interp_transpose_noalloc(msot_plan_t plan, const float *d_raw, float *d_coeffs,
                                  int batch, void *stream);

/* Travel-time table of two speeds of sound on the GPU (FP64): the medium
 * (c_below) and the coupling medium (c_above) are separated by the membrane
 * z = sum_k membrane[k] x^k (n_coef <= 8).  A pixel with z > m(x) reaches a
 * detector along the path through (x_m, m(x_m)) minimising
 * |p - q| / c_below + |q - d| / c_above over x_m in [-radius, radius]
 * (refraction.m:8-19, fermat_principle.m:17-24, there by fminbnd; here a
 * golden-section search to the FP64 limit), other pixels straight at c_above
 * (refraction.m:20-24).  travel as msot_travel_times; x_mem (may be NULL)
 * receives x_m, NaN where the path does not cross the membrane
 * (calculate_travel_time.m's x_membrane_intersections); virt_x / virt_z
 * (both or neither NULL) the virtual sources of MSOTmodel.m:585-594: on the
 * ray from the detector through the membrane point at the distance
 * t * c_above, the pixel itself where x_m is NaN.  Host [n_det][nx*nz].
 * Synchronous. */
int msot_travel_times_dual(int n_det, double radius, double coverage_deg, const double *x, int nx,
                           const double *z, int nz, double c_below, double c_above,
                           const double *membrane, int n_coef, double fs, double delay,
                           double n_crop, double *travel, double *x_mem, double *virt_x,
                           double *virt_z);

/* Travel-time table of a single speed of sound on the GPU (FP64):
 * MSOTmodel.m:350-382 with calculate_travel_time's straight rays and the arc
 * detector positions of Probe.m:112-116.  x (nx) and z (nz) are the pixel
 * coordinate vectors (Discretization.m:34); travel receives host
 * [n_det][nx*nz] = |x_p - x_d| / c * fs - delay - n_crop, the layout
 * msot_plan_desc.travel takes.  Synchronous. */
int msot_travel_times(int n_det, double radius, double coverage_deg, const double *x, int nx,
                      const double *z, int nz, double c, double fs, double delay, double n_crop,
                      double *travel);

/* Spatial pixel model response (SPMR) tables for include_sir plans, the
 * role of calculate_polarSPMR.m:21-184 + MSOTmodel.m:463-480 (2-D, single
 * speed of sound).  The reference obtains the element's spatial impulse
 * response from Field II (not available); here it is the Rayleigh integral
 * over sub_x x sub_y point sources on the element.  The rest follows the
 * reference: N-shape pixel response and order-8 Butterworth low pass at fs/2
 * at 5 GHz, DAC-rate sampling around the travel time, 1e-4 zeroing,
 * start/end samples, common crop, and the pixel -> column index of
 * MSOTmodel.m:472-477.  Outputs match msot_plan_desc's sir / sir_start_end /
 * sir_idx. */
typedef struct msot_spmr_spec {
    int n_det;                  /* arc array (Probe.m:112-116) */
    double radius, coverage_deg;
    const double *x;            /* host pixel coordinate vectors, nx and nz entries */
    int nx;
    const double *z;
    int nz;
    double c, fs;               /* speed of sound [m/s], DAC sampling rate [Hz] */
    double pixel_sigma;         /* Gaussian pixel model sigma [m] (Discretization.m:43) */
    double elem_width, elem_height;  /* element size [m] (pitch - separation, height) */
    double elem_elev_radius;    /* elevation focus radius [m]; 0 = flat element */
    int sub_x, sub_y;           /* point sources along the width / the height */
    int half_window;            /* DAC samples each side of the travel time (45 in the reference) */
    /* dual speed of sound (MSOTmodel.m:579-596): host [n_det][nx*nz] virtual
     * source positions (msot_travel_times_dual) used for the polar mapping in
     * place of the pixels, with c the coupling medium's speed; both NULL for
     * a single speed of sound */
    const double *virt_x, *virt_z;
} msot_spmr_spec;
typedef struct msot_spmr_info {
    double d_min, d_step, a_step_deg;  /* polar grid (MSOTmodel.m:600-613) */
    int n_dist, n_angle;
    int n_sir, sir_len;         /* table columns (n_dist * n_angle) and cropped length */
} msot_spmr_info;
/* Sizes and grid of the tables (computes them once). */
int msot_spmr_query(const msot_spmr_spec *spec, msot_spmr_info *info);
/* sir: host [n_sir][sir_len]; start_end: host [n_sir][2] (1-based inclusive);
 * sir_idx: host [n_det][nx*nz] (1-based column).  MSOT_ERANGE when a column's
 * response reaches the edge of the half_window (widen it) or a pixel maps
 * outside the table. */
int msot_spmr_tables(const msot_spmr_spec *spec, double *sir, int32_t *start_end,
                     int32_t *sir_idx);

/* Estimate sigma_max of the unnormalised operator by power iteration on the
 * GPU (replaces the svds call, MSOTmodel.m:277-278); FP64 norms. */
int msot_estimate_norm(msot_plan_t plan, int iters, uint64_t seed, double *sigma_max,
                       void *stream);

/* ------------------------------------------------------------------------ */
/* Solvers.  b: d_sino [batch][n_det][n_t]; result d_rec [batch][nx][nz].
 * Each instance of the batch is an independent reconstruction (one
 * single-wavelength call of the reference); coupled = 1 instead treats the
 * whole batch as the wavelengths of ONE reference call (shared scalars).
 * d_x0 (optional, may be NULL) seeds the iterate (warm start; the reference
 * always starts from zero).  err_img/err_reg (optional host arrays of
 * `batch` doubles) receive lCurveErrImg / lCurveErrReg per instance. */

/* rec_nn_with_L2_reg.m:1 with RegL2 = identity (lambdaL2 <= 0: no reg).
 * When err_img is given and an instance's final residual ||A x - b||^2 is
 * NaN or Inf (NaN / Inf in its data or start), returns MSOT_ENONFINITE naming
 * the first such instance; the images are still written.  The same holds
 * for the _warm and _2 forms below. */
int msot_rec_nn_with_L2_reg(msot_plan_t plan, const float *d_b, float *d_rec, int batch,
                            int num_iter, double lambdaL2, const float *d_x0, int coupled,
                            double *err_img, double *err_reg, void *stream);

/* Warm start of both splitting variables of nnls_L2_less (no reference
 * counterpart: the reference starts w and v from zero, nnls_L2_less.m:28-29).
 * d_w0 seeds the image w, d_v0 the multiplier v; at the method's fixed point
 * v = (A'(A w - b) + lambdaL2 w) / beta on the zero set of w and 0 elsewhere
 * (beta = 1e-3), which is what a consistent warm start supplies. */
int msot_rec_nn_with_L2_reg_warm(msot_plan_t plan, const float *d_b, float *d_rec, int batch,
                                 int num_iter, double lambdaL2, const float *d_w0,
                                 const float *d_v0, int coupled, double *err_img,
                                 double *err_reg, void *stream);

/* The same iteration with its whole state in and out: starts from (d_w0,
 * d_v0) (both NULL: the zero start of rec_nn_with_L2_reg; d_v0 NULL with a
 * d_w0: v = 0) and writes the final image to d_rec and the final multiplier
 * v to d_v, so that num_iter = k1 followed by a call from (d_rec, d_v) with
 * k2 iterations is the k1 + k2 iteration solve.  No reference counterpart
 * (the reference keeps v inside nnls_L2_less.m). */
int msot_rec_nn_with_L2_reg_state(msot_plan_t plan, const float *d_b, float *d_rec, float *d_v,
                                  int batch, int num_iter, double lambdaL2, const float *d_w0,
                                  const float *d_v0, int coupled, double *err_img,
                                  double *err_reg, void *stream);

/* rec_nn_with_L2_reg.m:1 with both regularisers of the reference's overview
 * script (reconstruction_overview_script.m:46-54): RegL2 = identity weighted
 * by lambdaL2 and RegL2_2 = RegL2T_2 = laplacian_per_wavelength (MATLAB
 * del2 per image; the reference passes it as its own transpose) weighted by
 * lambdaL2_2 (combine_forward_and_transpose_with_two_regs.m:8-14).  As in
 * incorporate_l2_reg_into_model_functions.m:8-18 the Laplacian term enters
 * only when lambdaL2 > 0 as well.  err_reg2 (optional host, batch doubles)
 * receives lCurveErrReg_2 = ||del2(rec)||^2. */
int msot_rec_nn_with_L2_reg_2(msot_plan_t plan, const float *d_b, float *d_rec, int batch,
                              int num_iter, double lambdaL2, double lambdaL2_2, const float *d_x0,
                              int coupled, double *err_img, double *err_reg, double *err_reg2,
                              void *stream);
/* laplacian_per_wavelength.m:4-8: d_out[w] = del2(d_in[w], 1) for images
 * [batch][nx][nz] (z fastest): (second differences along x + along z) / 4,
 * the end values extrapolated linearly from the interior. */
int msot_laplacian_per_wavelength(const float *d_in, float *d_out, int batch, int nx, int nz,
                                  void *stream);

/* rec_nn_with_L1_eye_reg.m:1.  MSOT_ENONFINITE as for the L2 solver when an
 * instance's final residual is NaN or Inf (err_img given). */
int msot_rec_nn_with_L1_eye_reg(msot_plan_t plan, const float *d_b, float *d_rec, int batch,
                                int num_iter, double reg, const float *d_x0, int coupled,
                                double *err_img, double *err_reg, void *stream);

/* rec_nn_with_TV_reg.m:1 (nnls_sparsa_based_reg_matrix_less.m:31-85; prox
 * SB_ITV2.m:20-40, TV term ITV.m:5-6).  Square grids only (MSOT_EINVAL
 * otherwise, as rec_nn_with_TV_reg.m:23-25 errors).  sparsa_iter is SpaRSA's
 * MaxiterA (2 in the reference, nnls_sparsa_based_reg_matrix_less.m:64);
 * err_reg receives ITV of each reconstruction. */
int msot_rec_nn_with_TV_reg(msot_plan_t plan, const float *d_b, float *d_rec, int batch,
                            int num_iter, double reg, int sparsa_iter, const float *d_x0,
                            int coupled, double *err_img, double *err_reg, void *stream);

/* SB_ITV2.m:1-40: u = argmin 1/2 ||u - g||^2 + mu ITV(u) for `batch` n x n
 * images (device FP32, [batch][n][n] column-major per image).  Synchronous. */
int msot_sb_itv2(const float *d_g, float *d_u, int batch, int n, double mu, void *stream);

/* ITV.m:1-6: isotropic TV of `batch` n x n device images -> host itv[batch].
 * Synchronous. */
int msot_itv(const float *d_x, double *itv, int batch, int n, void *stream);

/* ------------------------------------------------------------------------ */
/* Analytic reconstructors.  d_sig: [W][D][T] device FP32 (MATLAB T x D x W);
 * x (nx) and z (nz): host FP64 pixel coordinate vectors (the meshgrid of
 * Discretization.m:34 -- fov_x varies along columns, fov_z along rows);
 * outputs [W][nx][nz] device FP32.  An index outside the sinogram returns
 * MSOT_ERANGE (the reference errors).  Synchronous. */

/* dmas_cf.m:19-107: DMAS-CF, DMAS, coherence factor and DAS images. */
int msot_dmas_cf(const float *d_sig, int W, int D, int T, const double *x, int nx,
                 const double *z, int nz, double c, double fs, double n_crop, double coverage_deg,
                 double radius, float *d_dmas_cf, float *d_dmas, float *d_cf, float *d_das,
                 void *stream);

/* backproject_waveeq.m:1-50: psf host FP64 m x n (column-major, m along T);
 * d_K device FP32 K_n x K_n column-major (bp_kernel.m of the full acquisition
 * times; the samples n_crop+1 .. n_crop+T are used). */
int msot_backproject_waveeq(const float *d_sig, int W, int D, int T, const double *x, int nx,
                            const double *z, int nz, double c, double fs, double n_crop,
                            double coverage_deg, double radius, const double *psf, int psf_m,
                            int psf_n, const float *d_K, int K_n, float *d_out, void *stream);

/* ------------------------------------------------------------------------ */
/* Learned warm start (no counterpart in the reference): a U-Net that maps an
 * image (e.g. the adjoint of the data) to an NNLS start.  levels, base
 * channels c0 (c_l = c0 2^l), square side divisible by 2^(levels-1);
 * encoder conv3x3+ReLU x2 and 2x2 average pooling, decoder nearest
 * upsampling + concat + conv3x3+ReLU x2, output conv1x1.  Weights FP32
 * (Adam) used as BF16 in the convolutions, FP32 accumulation; activations
 * [n][1][side][side] FP32 on the device.  3x3 convolutions with >= 8 input
 * and a multiple of 32 output channels (forward and data gradient) run on
 * the tensor cores (tcgen05, TF32-rounded activations).  Parameter layout: per conv (encoder
 * a, b for level 0..L-1, decoder c, d for level L-2..0, output) the weights
 * [Co][Ci][k][k] then the biases [Co]. */
typedef struct msot_unet *msot_unet_t;
int msot_unet_create(int levels, int base_channels, int side, int max_batch, uint64_t seed,
                     msot_unet_t *net);
/* The same with in_channels (1 .. 8) input channels, [n][in_channels][side]
 * [side]; msot_unet_create is in_channels = 1.  The output has one channel. */
int msot_unet_create_ch(int levels, int base_channels, int in_channels, int side, int max_batch,
                        uint64_t seed, msot_unet_t *net);
int msot_unet_destroy(msot_unet_t net);
int msot_unet_param_count(msot_unet_t net, size_t *n);
int msot_unet_get_params(msot_unet_t net, float *host_params);
int msot_unet_set_params(msot_unet_t net, const float *host_params);
int msot_unet_forward(msot_unet_t net, const float *d_in, float *d_out, int n, void *stream);
/* Forward + backward of the mean squared error against d_target; the
 * gradients stay in the net for msot_unet_adam_step and are copied to
 * host_grad when it is not NULL.  Synchronous. */
int msot_unet_gradients(msot_unet_t net, const float *d_in, const float *d_target, int n,
                        double *loss, float *host_grad, void *stream);
/* One Adam step (beta1 0.9, beta2 0.999, eps 1e-8) on the last gradients;
 * step counts from 1 for the bias correction. */
int msot_unet_adam_step(msot_unet_t net, double lr, int step, void *stream);
/* Synchronises the device and reports (then clears) a tensor-core
 * convolution whose bounded wait for its MMAs ran out (MSOT_ECUDA). */
int msot_unet_check(msot_unet_t net);

/* ------------------------------------------------------------------------ */
/* Raw-sinogram pre-processing, in the order of
 * reconstruction_example_script.m:24-26, along the time axis of every column
 * ([n_cols][T_raw] FP32 on the device, t fastest = MATLAB T x D x W):
 *   crop_first_n_signals.m:2          the first n_crop samples are dropped;
 *   apply_butterworth_window_to_sinogram.m:5-9  (window_order > 0)
 *       x = mean + (x - mean) |h|, h the order-window_order Butterworth
 *       band-pass with cut-offs [window_low, window_high] / T (in samples,
 *       T = T_raw - n_crop) evaluated at T points of [0, pi);
 *   filter_butter_zero_phase.m:16-48 with use_fft = true (fmin or fmax > 0,
 *       Hz; <= 0 switches that half off): demean when fmin > 0, then
 *       ifft(|H|^2 fft(x)) with H the order-8 low-pass at fmax times the
 *       order-2 high-pass at fmin on T whole-circle bins.
 * The plan holds the window, the T x T circulant of ifft(|H|^2) and a
 * [max_cols][T] workspace.  d_out may equal d_raw unless n_crop > 0 without
 * the filter.  The reference's filtfilt branch (use_fft = false) is not
 * provided. */
typedef struct msot_prep *msot_prep_t;
int msot_prep_create(int T_raw, int n_crop, int window_order, double window_low,
                     double window_high, double fs, double fmin, double fmax, int max_cols,
                     msot_prep_t *prep);
int msot_prep_apply(msot_prep_t prep, const float *d_raw, float *d_out, int n_cols, void *stream);
int msot_prep_destroy(msot_prep_t prep);
/* Host only: |H(e^{iw})| of the digital Butterworth filter the pre-processing
 * designs (type 0 low-pass, 1 high-pass, 2 band-pass [wn1, wn2]; cut-offs in
 * units of the Nyquist frequency), at w = pi k / n (whole = 0) or 2 pi k / n
 * (whole = 1), k = 0 .. n - 1. */
int msot_butter_response(int order, int type, double wn1, double wn2, int n, int whole,
                         double *mag);

/* ------------------------------------------------------------------------ */
/* Instrumentation (no counterpart in the reference, whose only timing is
 * tic/toc, e.g. rec_nn_with_L2_reg.m:44-49). */

/* Autotuner (no reference counterpart): times the variants of the plan's
 * hot kernels on its own geometry at `batch` instances -- the DAS forward's
 * kernel (image values staged in shared memory per time tile and detector
 * group, or gathered per detector) and instances per CTA (8, 4, 2), the DAS
 * adjoint's instances per CTA (4, 2, 1), the register cap of the
 * IR convolution (1, 3, 4 resident CTAs per SM) and, for square grids, the
 * CTAs per image of the
 * SB_ITV2 cluster kernel (automatic, 1 .. 16, or -1: 16 CTAs with the
 * vectors in a global-memory workspace) -- and keeps the fastest in
 * the plan (they change results only in float summation order).  Drops the
 * plan's captured solver graphs.  Not concurrent with other calls on the
 * plan.  out (may be NULL) receives the choices and their times. */
typedef struct msot_tuning {
    int fwd_wt, conv_min_blocks, tv_cluster;  /* 0 = the built-in choice */
    double fwd_ms, transpose_ms, tv_prox_ms;  /* per apply of the chosen variant */
    int adj_wt;                               /* instances per CTA of the DAS adjoint (4, 2, 1) */
    int fwd_staged;                           /* DAS forward: 1 staged, 2 per-detector buckets,
                                                 4 per-detector buckets, interleaved entries */
} msot_tuning;
int msot_autotune(msot_plan_t plan, int batch, void *stream, msot_tuning *out);

/* Kernel tuning knob (no reference counterpart; results change only in
 * float summation order):
 *   "tv_prox_cluster"  CTAs per image of the shared-memory SB_ITV2 kernel
 *                      (1, 2, 4, 8, 16; 0 = automatic; -1 = 16 CTAs per
 *                      image with the vectors in global memory).
 *   "fwd_ell"          1 (default) = plans not autotuned run the DAS forward on
 *                      the interleaved (per-warp) copy of its entry table;
 *                      0 = the choice "fwd_staged" makes.
 *   "fwd_staged"       with "fwd_ell" 0: 1 (default) = the DAS forward stages
 *                      each CTA's image values in shared memory where the
 *                      plan's tables fit, 0 = per-detector gathers on the CSR
 *                      table (plans autotuned keep their pick; all forms give
 *                      the same sums).
 *   "fwd_staged_tile", "fwd_staged_group"  time samples per CTA (8 .. 64) and
 *                      detectors per CTA (1 .. 16) of the staged forward's
 *                      tables in plans created afterwards; 0 (default) = the
 *                      plan picks the shape that fits shared memory.
 *   "adj_prefetch"     1 (default) = the DAS adjoint loads the next detector's
 *                      samples into registers during the current one; 0 = off.
 *   "conv_min_blocks"  register cap of the IR convolution, as resident CTAs
 *                      per SM: 4 (default), 3, or 1 (uncapped).
 *   "unet_tensor_cores" 1 (default) = U-Net 3x3 convolutions on the tensor
 *                      cores where the shape allows, 0 = CUDA cores only
 *                      (FP32 activations, no TF32 rounding). */
int msot_tune_set(const char *key, int value);
/* SB_ITV2 kernel choice: 0 (default) = the shared-memory cluster kernel
 * wherever the image fits, 1 = always the global-memory kernel. */
int msot_tv_prox_path(int path);
/* Split-Bregman sweeps and CGS steps summed over all images of all cluster-
 * kernel SB_ITV2 launches since the last call (then reset); syncs the device. */
int msot_tv_prox_stats(long long *sweeps, long long *cg_steps);
/* Number of kernels the library has launched since it was loaded. */
long long msot_launch_count(void);
/* on != 0: record a CUDA event pair around every launch of the hot kernel
 * families (reset on each call); 0 disables. */
/* Throughput (GB/s) of random 32-byte-sector loads from a device buffer of
 * buffer_bytes (1 .. 96 MiB) that stays resident in L2: the ceiling of the
 * DAS interpolation kernels, whose gathers L2 serves.  Synchronous. */
int msot_l2_gather_probe(size_t buffer_bytes, double *gbs);
int msot_profile_enable(int on);
/* Name of kernel family `kid` (0..6), NULL past the end. */
const char *msot_profile_kernel_name(int kid);
/* Launches and summed event time (ms) recorded for family `kid`; syncs the device. */
int msot_profile_read(int kid, int *launches, double *total_ms);

/* ------------------------------------------------------------------------ */
/* MATLAB-level drop-in (host buffers, FP64, MATLAB memory layouts).  The MEX
 * gateways mex/msot_model_mex.cpp, mex/rec_nn_with_L2_reg.cpp,
 * mex/rec_nn_with_L1_eye_reg.cpp and mex/rec_nn_with_TV_reg.cpp wrap these. */

/* 1 when `plan` was created and not yet destroyed (a registry of live
 * plans: MEX callers hand plans to MATLAB as integer handles), else 0. */
int msot_plan_valid(msot_plan_t plan);

/* The fields of the reference's model object a plan is built from
 * (MSOTmodel.m:18-48): Discretization.sizeOfPixelGrid = [nx nz];
 * Data.absoluteTravelTimeIndices (P x D), circularInterpolationRadiusInSamples,
 * numTimeSamplesPerTransducer; Data.IRHat (interleaved complex, n_hat
 * entries, the length-(T + L - 1) transform of the IR, MSOTmodel.m:338-346)
 * with Probe.eirLength = L; Discretization.prefilter (interleaved complex
 * nz x nx, column-major, Discretization.m:47-51); Data.SPMR /
 * SPMRTimestepIndexStartAndEnd / SPMRIndices when includeSir. */
typedef struct msot_model_fields {
    int nx, nz, n_det, n_t;
    double radius;
    const double *travel;     /* P x D */
    const double *ir_hat;     /* NULL: no IR convolution */
    int n_hat, eir_length;
    const double *prefilter;  /* NULL: no prefilter */
    int sir_len, n_sir;       /* 0: no SIR */
    const double *sir;
    const int32_t *sir_start_end, *sir_idx;
    double norm;              /* model normalisation factor; <= 0: sigma_max is
                                 estimated (power iteration, 100 steps), as the
                                 reference runs svds when none is given
                                 (MSOTmodel.m:273-279) */
    int max_batch;            /* largest wavelength stack per call */
} msot_model_fields;
/* Plan of a reference model: IR taps = the first eirLength samples of
 * ifft(IRHat) (the rest must vanish, else MSOT_EINVAL); prefilter taps = the
 * two circular factors of ifft2(prefilter), which is separable for the
 * Gaussian pixel model, truncated below 1e-13 of the centre. */
int msot_plan_create_from_model(const msot_model_fields *fields, msot_plan_t *plan);
/* The plan's normalisation factor (0 for an invalid handle). */
double msot_plan_norm(msot_plan_t plan);
/* The plan's grid, detectors, samples and largest batch (any pointer may be
 * NULL); MSOT_EINVAL for an invalid handle.  No device work. */
int msot_plan_shape(msot_plan_t plan, int *nx, int *nz, int *n_det, int *n_t, int *max_batch);

/* model.Funcs.applyForward (transpose = 0: image Nz x Nx x W -> sinogram
 * T x D x W) and applyTranspose (transpose = 1: the reverse), FP64 host
 * arrays; W <= the plan's max_batch.  Synchronous. */
int msot_host_apply(msot_plan_t plan, int transpose, const double *in, int W, double *out);

/* The solvers on a T x D x W stack data (FP64 host), one reference call:
 * the W wavelengths are solved coupled and the outputs are sums over the
 * stack; rec receives Nz x Nx x W.  rec_nn_with_L2_reg.m:1 (RegL2 the
 * identity weighted by lambdaL2 > 0, RegL2_2 laplacian_per_wavelength
 * weighted by lambdaL2_2 > 0 and used only with lambdaL2 > 0, as the
 * reference does).  err_reg (may be NULL) receives ||rec||^2 and err_reg2
 * (may be NULL) ||del2(rec)||^2 whatever the weights, as the reference
 * evaluates them whenever RegL2 / RegL2_2 are given. */
int msot_host_rec_nn_with_L2_reg(msot_plan_t plan, const double *data, int W, int num_iter,
                                 double lambdaL2, double lambdaL2_2, double *rec,
                                 double *err_img, double *err_reg, double *err_reg2);
/* rec_nn_with_L1_eye_reg.m:1 (err_reg = ||rec||_1). */
int msot_host_rec_nn_with_L1_eye_reg(msot_plan_t plan, const double *data, int W, int num_iter,
                                     double reg, double *rec, double *err_img,
                                     double *err_reg);
/* rec_nn_with_TV_reg.m:1 (square grids; err_reg = the summed ITV). */
int msot_host_rec_nn_with_TV_reg(msot_plan_t plan, const double *data, int W, int num_iter,
                                 double reg, double *rec, double *err_img, double *err_reg);

/* ------------------------------------------------------------------------ */
/* Host-buffer entry points with the reference MEX contracts (FP64 in/out,
 * column-major, MATLAB-owned inputs; output written to caller memory that
 * MATLAB allocated with mxCreate*).  Arithmetic is FP32 on the GPU. */

/* forwardDelayAndSumMex.cpp:15-104: image W x P, travelTimes P x D,
 * numTimesteps, radius -> out W x T x D. */
int msot_mex_forwardDelayAndSum(const double *image, int W, int P, const double *travel, int D,
                                int T, double radius, double *out);
/* transposeDelayAndSumMex.cpp:15-98: sigMat W x T x D -> out W x P. */
int msot_mex_transposeDelayAndSum(const double *sig, int W, int T, int D, const double *travel,
                                  int P, double radius, double *out);
/* forwardMex.cpp:16-162 */
int msot_mex_forward(const double *image, int W, int P, const int32_t *sir_idx,
                     const double *travel, int D, const double *sir, int S, int NS, int T,
                     const int32_t *start_end, double radius, double *out);
/* transposeMex.cpp:16-158 */
int msot_mex_transpose(const double *sig, int W, int T, int D, const int32_t *sir_idx,
                       const double *travel, int P, const double *sir, int S, int NS,
                       const int32_t *start_end, double radius, double *out);

#ifdef __cplusplus
}
#endif
#endif
