// Per-row preparation of a vector set before the distance pass, and the
// device-side statistics the selection certificate needs.
#pragma once
#include <cuda_bf16.h>

#include "common.cuh"

namespace yg {

// statistics of one vector set, kept in device memory
struct SetStats {
  unsigned int max_norm_bits;   // max ||x|| (float bits; non-negative floats order as ints)
  unsigned int max_resid_bits;  // max ||x - bf16(x)||
  int all_exact;                // 1 iff every row is "exact class" (see row_exact below)
  int n_nan;                    // rows with a NaN/Inf coordinate
};

// A row is exact class when all coordinates are integers of magnitude <= 256
// (exactly representable in bf16) and ||x||^2 <= 2^22.  For two exact-class
// rows every product and partial sum of the distance expansion is an integer
// below 2^24, so FP32 FFMA chains and the BF16 tensor-core path (FP32
// accumulate) both give the exact value, in any summation order.
constexpr double kExactNorm2Max = 4194304.0;  // 2^22

// Per-row preparation.  One warp per row.  Writes (each optional):
//   norm64[i]   = sum x^2 in FP64 (exact up to FP64 rounding)
//   norm32[i]   = (float) norm64[i]
//   flags[i]    = 1 if exact class
//   resid[i]    = || x - bf16(x) ||   (FP64 accumulate, stored as float, rounded up)
//   packed row  = bf16(scale * x) in [Kp] columns (zero padded), when packed != null
//   normpart[i] = when base_parts: bf16 parts (hi, mid, lo) of (float)norm64 in
//                 columns 0..2, zero in 3..15; when query_ones: 1,1,1,0...
// and folds max norm / max residual / all-exact / NaN counts into *stats.
int prep_rows(const float *x, long ld, int n, int d, float scale, double *norm64,
              float *norm32, unsigned char *flags, float *resid,
              __nv_bfloat16 *packed, int Kp, __nv_bfloat16 *normpart,
              int normpart_mode, SetStats *stats, cudaStream_t st);

int stats_reset(SetStats *stats, cudaStream_t st);

}  // namespace yg
