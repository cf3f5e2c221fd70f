// Row preparation: norms, exact-class flags, bf16 packing (see prep.cuh).
#include "prep.cuh"

namespace yg {

__global__ void prep_rows_kernel(const float *__restrict__ x, long ld, int n, int d,
                                 float scale, double *norm64, float *norm32,
                                 unsigned char *flags, float *resid,
                                 __nv_bfloat16 *packed, int Kp,
                                 __nv_bfloat16 *normpart, int normpart_mode,
                                 SetStats *stats) {
  const int lane = threadIdx.x & 31;
  const long row = (long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (row >= n) return;
  const float *xr = x + row * ld;
  double s = 0, r = 0;
  int exact = 1, bad = 0;
  const int cols = packed ? (Kp > d ? Kp : d) : d;
  for (int c = lane; c < cols; c += 32) {
    float v = c < d ? __ldg(xr + c) : 0.f;
    if (c < d) {
      s += (double)v * (double)v;
      exact &= (v == rintf(v)) && (fabsf(v) <= 256.f);
      bad |= !isfinite(v);
      __nv_bfloat16 h = __float2bfloat16_rn(v);
      double dv = (double)v - (double)__bfloat162float(h);
      r += dv * dv;
    }
    if (packed && c < Kp) packed[row * Kp + c] = __float2bfloat16_rn(scale * v);
  }
  for (int o = 16; o > 0; o >>= 1) {
    s += __shfl_xor_sync(0xffffffffu, s, o);
    r += __shfl_xor_sync(0xffffffffu, r, o);
    exact &= __shfl_xor_sync(0xffffffffu, exact, o);
    bad |= __shfl_xor_sync(0xffffffffu, bad, o);
  }
  exact &= (s <= kExactNorm2Max) && !bad;
  if (normpart && lane < 16) {
    __nv_bfloat16 val = __float2bfloat16_rn(0.f);
    if (normpart_mode == 1) {
      // three bf16 parts whose exact sum is the float norm
      float n32 = (float)s;
      __nv_bfloat16 hi = __float2bfloat16_rn(n32);
      float r1 = n32 - __bfloat162float(hi);
      __nv_bfloat16 mid = __float2bfloat16_rn(r1);
      float r2 = r1 - __bfloat162float(mid);
      __nv_bfloat16 lo = __float2bfloat16_rn(r2);
      val = lane == 0 ? hi : lane == 1 ? mid : lane == 2 ? lo : val;
    } else if (normpart_mode == 2) {
      val = __float2bfloat16_rn(lane < 3 ? 1.f : 0.f);
    }
    normpart[row * 16 + lane] = val;
  }
  if (lane == 0) {
    if (norm64) norm64[row] = s;
    if (norm32) norm32[row] = (float)s;
    if (flags) flags[row] = (unsigned char)exact;
    float rr = (float)(sqrt(r) * (1.0 + 1e-6));
    if (resid) resid[row] = rr;
    if (stats) {
      float nr = (float)(sqrt(s) * (1.0 + 1e-6));
      if (!bad) {
        atomicMax(&stats->max_norm_bits, __float_as_uint(nr));
        atomicMax(&stats->max_resid_bits, __float_as_uint(rr));
      } else {
        atomicAdd(&stats->n_nan, 1);
      }
      if (!exact) atomicAnd(&stats->all_exact, 0);
    }
  }
}

int stats_reset(SetStats *stats, cudaStream_t st) {
  SetStats h{0u, 0u, 1, 0};
  YG_CUDA(cudaMemcpyAsync(stats, &h, sizeof(h), cudaMemcpyHostToDevice, st));
  return OK;
}

int prep_rows(const float *x, long ld, int n, int d, float scale, double *norm64,
              float *norm32, unsigned char *flags, float *resid,
              __nv_bfloat16 *packed, int Kp, __nv_bfloat16 *normpart,
              int normpart_mode, SetStats *stats, cudaStream_t st) {
  if (n <= 0) return OK;
  const int warps = 8;
  dim3 grid((unsigned)ceil_div(n, warps));
  prep_rows_kernel<<<grid, warps * 32, 0, st>>>(x, ld, n, d, scale, norm64, norm32,
                                                flags, resid, packed, Kp, normpart,
                                                normpart_mode, stats);
  YG_LAUNCH_CHECK();
  return OK;
}

}  // namespace yg
