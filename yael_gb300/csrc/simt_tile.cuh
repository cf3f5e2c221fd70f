// FP32 CUDA-core 128x128 tile main loop shared by the fused selection pass and
// the cross-distance kernel.  256 threads; thread (tx, ty) = (tid % 16,
// tid / 16) owns rows {ty*4+i, 64+ty*4+i} and columns {tx*4+j, 64+tx*4+j}.
#pragma once
#include "common.cuh"

namespace yg {
namespace simt {

constexpr int BM = 128, BN = 128, BK = 16, NT = 256, APAD = 4;
constexpr int ST_LD = BN + 1;  // staging tile row pitch (floats)
constexpr size_t kOperandFloats = 2 * BK * (BM + APAD) + 2 * BK * (BN + APAD);

__device__ __forceinline__ int row_of(int i, int ty) { return i < 4 ? ty * 4 + i : 64 + ty * 4 + (i - 4); }
__device__ __forceinline__ int col_of(int j, int tx) { return j < 4 ? tx * 4 + j : 64 + tx * 4 + (j - 4); }

// acc[i][j] = sum_k A[q0 + row_of(i)][k] * B[j0 + col_of(j)][k]; rows past na /
// nb read as zero.  smem must hold kOperandFloats floats.
__device__ __forceinline__ void tile_mainloop(const float *__restrict__ A, long lda, int na,
                                              long i0, const float *__restrict__ B, long ldb,
                                              int nb, long j0, int d, float *smem,
                                              float acc[8][8]) {
  float *As = smem;
  float *Bs = As + 2 * BK * (BM + APAD);
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  const int lr = tid >> 1, lc = (tid & 1) * 8;
  const int nk = (int)ceil_div(d, BK);
#pragma unroll
  for (int i = 0; i < 8; i++)
#pragma unroll
    for (int j = 0; j < 8; j++) acc[i][j] = 0.f;
  float ra[8], rb[8];
  auto gload = [&](int k0) {
    const long ia = i0 + lr, jb = j0 + lr;
#pragma unroll
    for (int i = 0; i < 8; i++) {
      const int k = k0 + lc + i;
      ra[i] = (ia < na && k < d) ? __ldg(A + ia * lda + k) : 0.f;
      rb[i] = (jb < nb && k < d) ? __ldg(B + jb * ldb + k) : 0.f;
    }
  };
  auto sstore = [&](int buf) {
    float *a = As + buf * BK * (BM + APAD);
    float *b = Bs + buf * BK * (BN + APAD);
#pragma unroll
    for (int i = 0; i < 8; i++) {
      a[(lc + i) * (BM + APAD) + lr] = ra[i];
      b[(lc + i) * (BN + APAD) + lr] = rb[i];
    }
  };
  gload(0);
  sstore(0);
  __syncthreads();
  for (int kb = 0; kb < nk; kb++) {
    const int buf = kb & 1;
    if (kb + 1 < nk) gload((kb + 1) * BK);
    const float *a = As + buf * BK * (BM + APAD);
    const float *b = Bs + buf * BK * (BN + APAD);
#pragma unroll
    for (int kk = 0; kk < BK; kk++) {
      const float4 a0 = *reinterpret_cast<const float4 *>(a + kk * (BM + APAD) + ty * 4);
      const float4 a1 = *reinterpret_cast<const float4 *>(a + kk * (BM + APAD) + 64 + ty * 4);
      const float4 b0 = *reinterpret_cast<const float4 *>(b + kk * (BN + APAD) + tx * 4);
      const float4 b1 = *reinterpret_cast<const float4 *>(b + kk * (BN + APAD) + 64 + tx * 4);
      const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
      const float bv[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
      for (int i = 0; i < 8; i++)
#pragma unroll
        for (int j = 0; j < 8; j++) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
    }
    if (kb + 1 < nk) sstore(buf ^ 1);
    __syncthreads();
  }
}

}  // namespace simt
}  // namespace yg
