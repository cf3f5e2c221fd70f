// Per-row preparation of a vector set before the distance pass, and the
// device-side statistics the selection certificate needs.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "common.cuh"

namespace yg {

// statistics of one vector set, kept in device memory
struct SetStats {
  unsigned int max_norm_bits;   // max ||x|| (float bits; non-negative floats order as ints)
  unsigned int max_resid_bits;  // max ||x - bf16(x)|| (fp16(x) for an fp16 packing)
  int all_exact;                // 1 iff every row is "exact class" (see row_exact below)
  int n_nan;                    // rows with a NaN/Inf coordinate
  unsigned int max_lo_bits;     // split packing: max ||lo||, lo = bf16(x - bf16(x))
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
// warps: warps per block of the row-vector form (1..8): small blocks fit on an
// SM beside a running distance pass, so packing can overlap one
// f16 = 1: the packed row and the norm parts are IEEE fp16 instead of bf16
// (same layout; resid is then the error of the fp16 packing, infinite for a
// row that fp16 cannot hold: |scale x| > 65504 or ||x||^2 >= 2^15)
// Rows translated before everything else: with mu != null, row r is taken
// as fl(x_r - mu_i) (FP32 subtraction), mu_i = mu + i * d with
// i = row_inst[r] when row_inst != null, else r / rows_per_inst.
struct RowShift {
  const float *mu = nullptr;
  const int *row_inst = nullptr;
  int rows_per_inst = 1;
};
int prep_rows(const float *x, long ld, int n, int d, float scale, double *norm64,
              float *norm32, unsigned char *flags, float *resid,
              __nv_bfloat16 *packed, int Kp, __nv_bfloat16 *normpart,
              int normpart_mode, SetStats *stats, cudaStream_t st, int warps = 8,
              int f16 = 0, RowShift shift = RowShift());

// Split ("3xBF16") packing: x = hi + lo + r with hi = bf16(x), lo = bf16(x - hi),
// written as three K segments of Kp1 = 64*ceil(d/64) columns each:
//   layout 0 (queries): [hi | hi | lo] of scale*x
//   layout 1 (base):    [hi | lo | hi]
// so one MMA over the 3*Kp1 columns sums q_hi.b_hi + q_hi.b_lo + q_lo.b_hi
// (only q_lo.b_lo and the residuals r are left out).  Per row: lonorm = ||lo||,
// resid = ||r||; norms / flags / side block / stats as prep_rows.
int prep_rows_split(const float *x, long ld, int n, int d, float scale, int layout,
                    double *norm64, float *norm32, unsigned char *flags, float *lonorm,
                    float *resid, __nv_bfloat16 *packed, int Kp1, __nv_bfloat16 *normpart,
                    int normpart_mode, SetStats *stats, cudaStream_t st);

int stats_reset(SetStats *stats, cudaStream_t st);

}  // namespace yg
