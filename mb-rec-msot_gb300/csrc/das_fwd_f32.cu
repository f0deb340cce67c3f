// das_fwd_f32.cu -- k_das_fwd3 on the FP32 interpolation input (das_fwd.cuh)
#include "das_fwd.cuh"

namespace msot {

int das_fwd_run_f32(const Plan &pl, const void *xpm, float *raw, int W, float scale,
                   const float *inv_s, bool ell, int wt, cudaStream_t st) {
    return das_fwd_run<float>(pl, xpm, raw, W, scale, inv_s, ell, wt, st);
}

}  // namespace msot
