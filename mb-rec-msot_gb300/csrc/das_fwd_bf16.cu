// das_fwd_bf16.cu -- k_das_fwd3 on the BF16 interpolation input (das_fwd.cuh)
#include "das_fwd.cuh"

namespace msot {

int das_fwd_run_bf16(const Plan &pl, const void *xpm, float *raw, int W, float scale,
                   const float *inv_s, bool ell, int wt, cudaStream_t st) {
    return das_fwd_run<__nv_bfloat16>(pl, xpm, raw, W, scale, inv_s, ell, wt, st);
}

}  // namespace msot
