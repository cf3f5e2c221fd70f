// Row preparation: norms, exact-class flags, bf16 packing (see prep.cuh).
#include "prep.cuh"

namespace yg {

namespace {
constexpr int PW = 8;  // warps per block

__global__ void __launch_bounds__(PW * 32)
    prep_rows_kernel(const float *__restrict__ x, long ld, int n, int d, float scale,
                     double *norm64, float *norm32, unsigned char *flags, float *resid,
                     __nv_bfloat16 *packed, int Kp, __nv_bfloat16 *normpart,
                     int normpart_mode, SetStats *stats) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const long nwarps = (long)gridDim.x * PW;
  // per-warp running statistics, reduced once per block at the end
  float w_maxnorm = 0.f, w_maxres = 0.f;
  int w_exact = 1, w_nan = 0;
  const int cols = packed ? (Kp > d ? Kp : d) : d;
  // vectorised path: 4 consecutive coordinates per lane (d % 4 == 0, aligned rows)
  const bool vec = (d % 4 == 0) && (ld % 4 == 0) && ((reinterpret_cast<uintptr_t>(x) & 15) == 0) &&
                   (!packed || Kp % 4 == 0);
  for (long row = (long)blockIdx.x * PW + wid; row < n; row += nwarps) {
    const float *xr = x + row * ld;
    // FP32 per element: exact for integer data (partial sums < 2^24), within
    // (d/32 + 6) ulp otherwise -- the certificate's error bound covers that
    float s = 0.f, r = 0.f;
    int exact = 1, bad = 0;
    if (vec) {
      for (int c = lane * 4; c < cols; c += 128) {
        float4 q4 = make_float4(0.f, 0.f, 0.f, 0.f);
        if (c < d) q4 = __ldg(reinterpret_cast<const float4 *>(xr + c));
        const float e[4] = {q4.x, q4.y, q4.z, q4.w};
        __nv_bfloat16 hb[4];
#pragma unroll
        for (int t = 0; t < 4; t++) {
          const float v = e[t];
          if (c + t < d) {
            s = fmaf(v, v, s);
            exact &= (v == rintf(v)) && (fabsf(v) <= 256.f);
            bad |= !isfinite(v);
            const float dv = v - __bfloat162float(__float2bfloat16_rn(v));  // exact
            r = fmaf(dv, dv, r);
          }
          hb[t] = __float2bfloat16_rn(scale * v);
        }
        if (packed && c < Kp) {
          uint2 w;
          w.x = (uint32_t)__bfloat16_as_ushort(hb[0]) | ((uint32_t)__bfloat16_as_ushort(hb[1]) << 16);
          w.y = (uint32_t)__bfloat16_as_ushort(hb[2]) | ((uint32_t)__bfloat16_as_ushort(hb[3]) << 16);
          *reinterpret_cast<uint2 *>(packed + row * Kp + c) = w;
        }
      }
    } else {
      for (int c = lane; c < cols; c += 32) {
        const float v = c < d ? __ldg(xr + c) : 0.f;
        if (c < d) {
          s = fmaf(v, v, s);
          exact &= (v == rintf(v)) && (fabsf(v) <= 256.f);
          bad |= !isfinite(v);
          const float dv = v - __bfloat162float(__float2bfloat16_rn(v));
          r = fmaf(dv, dv, r);
        }
        if (packed && c < Kp) packed[row * Kp + c] = __float2bfloat16_rn(scale * v);
      }
    }
#pragma unroll
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
        const float n32 = (float)s;
        const __nv_bfloat16 hi = __float2bfloat16_rn(n32);
        const float r1 = n32 - __bfloat162float(hi);
        const __nv_bfloat16 mid = __float2bfloat16_rn(r1);
        const float r2 = r1 - __bfloat162float(mid);
        const __nv_bfloat16 lo = __float2bfloat16_rn(r2);
        val = lane == 0 ? hi : lane == 1 ? mid : lane == 2 ? lo : val;
      } else if (normpart_mode == 2) {
        val = __float2bfloat16_rn(lane < 3 ? 1.f : 0.f);
      }
      normpart[row * 16 + lane] = val;
    }
    const float rr = sqrtf(r) * (1.f + 1e-5f);
    if (lane == 0) {
      if (norm64) norm64[row] = (double)s;
      if (norm32) norm32[row] = (float)s;
      if (flags) flags[row] = (unsigned char)exact;
      if (resid) resid[row] = rr;
    }
    if (!bad) {
      w_maxnorm = fmaxf(w_maxnorm, sqrtf(s) * (1.f + 1e-5f));
      w_maxres = fmaxf(w_maxres, rr);
    } else {
      w_nan++;
    }
    w_exact &= exact;
  }
  if (!stats) return;
  __shared__ float s_norm[PW], s_res[PW];
  __shared__ int s_exact[PW], s_nan[PW];
  if (lane == 0) {
    s_norm[wid] = w_maxnorm;
    s_res[wid] = w_maxres;
    s_exact[wid] = w_exact;
    s_nan[wid] = w_nan;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float mn = 0.f, mr = 0.f;
    int ex = 1, nn = 0;
    for (int w = 0; w < PW; w++) {
      mn = fmaxf(mn, s_norm[w]);
      mr = fmaxf(mr, s_res[w]);
      ex &= s_exact[w];
      nn += s_nan[w];
    }
    atomicMax(&stats->max_norm_bits, __float_as_uint(mn));
    atomicMax(&stats->max_resid_bits, __float_as_uint(mr));
    if (!ex) atomicAnd(&stats->all_exact, 0);
    if (nn) atomicAdd(&stats->n_nan, nn);
  }
}

// The vectorised form for d <= 32 * 4 * LPR / ... with LPR lanes per row:
// 32 / LPR rows per warp step, each lane four consecutive coordinates per
// float4 (several independent loads in flight), reductions over LPR lanes.
// Same outputs as prep_rows_kernel.
template <int LPR>
__global__ void __launch_bounds__(PW * 32)
    prep_rows_vec_kernel(const float *__restrict__ x, long ld, int n, int d, float scale,
                         double *norm64, float *norm32, unsigned char *flags, float *resid,
                         __nv_bfloat16 *packed, int Kp, __nv_bfloat16 *normpart,
                         int normpart_mode, SetStats *stats) {
  constexpr int RPW = 32 / LPR;  // rows per warp step
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int sub = lane / LPR, sl = lane % LPR;
  const int wpb = (int)(blockDim.x >> 5);  // warps per block (<= PW)
  const long nwarps = (long)gridDim.x * wpb;
  float w_maxnorm = 0.f, w_maxres = 0.f;
  int w_exact = 1, w_nan = 0;
  const int cols = packed ? (Kp > d ? Kp : d) : d;
  for (long rbase = ((long)blockIdx.x * wpb + wid) * RPW; rbase < n; rbase += nwarps * RPW) {
    const long row = rbase + sub;
    const bool rv = row < n;
    const float *xr = x + row * ld;
    float s = 0.f, r = 0.f;
    int exact = 1, bad = 0;
    // every load of the row first (cols <= 128, the launch condition), then
    // the conversions: NIT float4 loads of each lane in flight at once
    constexpr int NIT = 128 / (4 * LPR);
    float4 q4s[NIT];
#pragma unroll
    for (int it = 0; it < NIT; it++) {
      const int c = sl * 4 + it * 4 * LPR;
      q4s[it] = make_float4(0.f, 0.f, 0.f, 0.f);
      if (rv && c < d) q4s[it] = __ldg(reinterpret_cast<const float4 *>(xr + c));
    }
#pragma unroll
    for (int it = 0; it < NIT; it++) {
      const int c = sl * 4 + it * 4 * LPR;
      if (c >= cols) break;
      const float4 q4 = q4s[it];
      const float e[4] = {q4.x, q4.y, q4.z, q4.w};
      __nv_bfloat16 hb[4];
#pragma unroll
      for (int t = 0; t < 4; t++) {
        const float v = e[t];
        if (c + t < d) {
          s = fmaf(v, v, s);
          exact &= (v == rintf(v)) && (fabsf(v) <= 256.f);
          bad |= !isfinite(v);
          const float dv = v - __bfloat162float(__float2bfloat16_rn(v));  // exact
          r = fmaf(dv, dv, r);
        }
        hb[t] = __float2bfloat16_rn(scale * v);
      }
      if (rv && packed && c < Kp) {
        uint2 w;
        w.x = (uint32_t)__bfloat16_as_ushort(hb[0]) | ((uint32_t)__bfloat16_as_ushort(hb[1]) << 16);
        w.y = (uint32_t)__bfloat16_as_ushort(hb[2]) | ((uint32_t)__bfloat16_as_ushort(hb[3]) << 16);
        *reinterpret_cast<uint2 *>(packed + row * Kp + c) = w;
      }
    }
#pragma unroll
    for (int o = LPR / 2; o > 0; o >>= 1) {  // stays inside the row's LPR-lane group
      s += __shfl_xor_sync(0xffffffffu, s, o);
      r += __shfl_xor_sync(0xffffffffu, r, o);
      exact &= __shfl_xor_sync(0xffffffffu, exact, o);
      bad |= __shfl_xor_sync(0xffffffffu, bad, o);
    }
    exact &= (s <= kExactNorm2Max) && !bad;
    const float rr = sqrtf(r) * (1.f + 1e-5f);
    if (rv && sl == 0) {
      if (normpart) {
        __nv_bfloat16 part[16];
#pragma unroll
        for (int i = 0; i < 16; i++) part[i] = __float2bfloat16_rn(0.f);
        if (normpart_mode == 1) {
          // three bf16 parts whose exact sum is the float norm
          const float n32 = s;
          const __nv_bfloat16 hi = __float2bfloat16_rn(n32);
          const float r1 = n32 - __bfloat162float(hi);
          const __nv_bfloat16 mid = __float2bfloat16_rn(r1);
          const float r2 = r1 - __bfloat162float(mid);
          part[0] = hi;
          part[1] = mid;
          part[2] = __float2bfloat16_rn(r2);
        } else if (normpart_mode == 2) {
          part[0] = part[1] = part[2] = __float2bfloat16_rn(1.f);
        }
        uint4 w0, w1;
        uint32_t *u0 = reinterpret_cast<uint32_t *>(&w0), *u1 = reinterpret_cast<uint32_t *>(&w1);
#pragma unroll
        for (int i = 0; i < 4; i++) {
          u0[i] = (uint32_t)__bfloat16_as_ushort(part[2 * i]) |
                  ((uint32_t)__bfloat16_as_ushort(part[2 * i + 1]) << 16);
          u1[i] = (uint32_t)__bfloat16_as_ushort(part[8 + 2 * i]) |
                  ((uint32_t)__bfloat16_as_ushort(part[8 + 2 * i + 1]) << 16);
        }
        uint4 *dst = reinterpret_cast<uint4 *>(normpart + row * 16);
        dst[0] = w0;
        dst[1] = w1;
      }
      if (norm64) norm64[row] = (double)s;
      if (norm32) norm32[row] = s;
      if (flags) flags[row] = (unsigned char)exact;
      if (resid) resid[row] = rr;
    }
    if (rv) {
      if (!bad) {
        w_maxnorm = fmaxf(w_maxnorm, sqrtf(s) * (1.f + 1e-5f));
        w_maxres = fmaxf(w_maxres, rr);
      } else if (sl == 0) {
        w_nan++;
      }
      w_exact &= exact;
    }
  }
  if (!stats) return;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {  // the warp's rows
    w_maxnorm = fmaxf(w_maxnorm, __shfl_xor_sync(0xffffffffu, w_maxnorm, o));
    w_maxres = fmaxf(w_maxres, __shfl_xor_sync(0xffffffffu, w_maxres, o));
    w_exact &= __shfl_xor_sync(0xffffffffu, w_exact, o);
    w_nan += __shfl_xor_sync(0xffffffffu, w_nan, o);
  }
  __shared__ float s_norm[PW], s_res[PW];
  __shared__ int s_exact[PW], s_nan[PW];
  if (lane == 0) {
    s_norm[wid] = w_maxnorm;
    s_res[wid] = w_maxres;
    s_exact[wid] = w_exact;
    s_nan[wid] = w_nan;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float mn = 0.f, mr = 0.f;
    int ex = 1, nn = 0;
    for (int w = 0; w < wpb; w++) {
      mn = fmaxf(mn, s_norm[w]);
      mr = fmaxf(mr, s_res[w]);
      ex &= s_exact[w];
      nn += s_nan[w];
    }
    atomicMax(&stats->max_norm_bits, __float_as_uint(mn));
    atomicMax(&stats->max_resid_bits, __float_as_uint(mr));
    if (!ex) atomicAnd(&stats->all_exact, 0);
    if (nn) atomicAdd(&stats->n_nan, nn);
  }
}

__global__ void __launch_bounds__(PW * 32)
    prep_split_kernel(const float *__restrict__ x, long ld, int n, int d, float scale, int layout,
                      double *norm64, float *norm32, unsigned char *flags, float *lonorm,
                      float *resid, __nv_bfloat16 *packed, int Kp1, __nv_bfloat16 *normpart,
                      int normpart_mode, SetStats *stats) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const long nwarps = (long)gridDim.x * PW;
  const int Kp = 3 * Kp1;
  float w_maxnorm = 0.f, w_maxres = 0.f, w_maxlo = 0.f;
  int w_exact = 1, w_nan = 0;
  for (long row = (long)blockIdx.x * PW + wid; row < n; row += nwarps) {
    const float *xr = x + row * ld;
    float s = 0.f, r = 0.f, l = 0.f;
    int exact = 1, bad = 0;
    for (int c = lane; c < Kp1; c += 32) {
      const float v = c < d ? __ldg(xr + c) : 0.f;
      const __nv_bfloat16 hi = __float2bfloat16_rn(v);
      const float rest = v - __bfloat162float(hi);             // exact
      const __nv_bfloat16 lo = __float2bfloat16_rn(rest);
      const float r2 = rest - __bfloat162float(lo);            // exact
      if (c < d) {
        s = fmaf(v, v, s);
        exact &= (v == rintf(v)) && (fabsf(v) <= 256.f);
        bad |= !isfinite(v);
        const float lf = __bfloat162float(lo);
        l = fmaf(lf, lf, l);
        r = fmaf(r2, r2, r);
      }
      const __nv_bfloat16 shi = __float2bfloat16_rn(scale * __bfloat162float(hi));
      const __nv_bfloat16 slo = __float2bfloat16_rn(scale * __bfloat162float(lo));
      __nv_bfloat16 *pr = packed + row * Kp;
      pr[c] = shi;
      pr[Kp1 + c] = layout == 0 ? shi : slo;
      pr[2 * Kp1 + c] = layout == 0 ? slo : shi;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      s += __shfl_xor_sync(0xffffffffu, s, o);
      r += __shfl_xor_sync(0xffffffffu, r, o);
      l += __shfl_xor_sync(0xffffffffu, l, o);
      exact &= __shfl_xor_sync(0xffffffffu, exact, o);
      bad |= __shfl_xor_sync(0xffffffffu, bad, o);
    }
    exact &= (s <= kExactNorm2Max) && !bad;
    if (normpart && lane < 16) {
      __nv_bfloat16 val = __float2bfloat16_rn(0.f);
      if (normpart_mode == 1) {
        const float n32 = s;
        const __nv_bfloat16 hi = __float2bfloat16_rn(n32);
        const float r1 = n32 - __bfloat162float(hi);
        const __nv_bfloat16 mid = __float2bfloat16_rn(r1);
        const float r2 = r1 - __bfloat162float(mid);
        const __nv_bfloat16 lo = __float2bfloat16_rn(r2);
        val = lane == 0 ? hi : lane == 1 ? mid : lane == 2 ? lo : val;
      } else if (normpart_mode == 2) {
        val = __float2bfloat16_rn(lane < 3 ? 1.f : 0.f);
      }
      normpart[row * 16 + lane] = val;
    }
    const float rr = sqrtf(r) * (1.f + 1e-5f), ll = sqrtf(l) * (1.f + 1e-5f);
    if (lane == 0) {
      if (norm64) norm64[row] = (double)s;
      if (norm32) norm32[row] = s;
      if (flags) flags[row] = (unsigned char)exact;
      if (resid) resid[row] = rr;
      if (lonorm) lonorm[row] = ll;
    }
    if (!bad) {
      w_maxnorm = fmaxf(w_maxnorm, sqrtf(s) * (1.f + 1e-5f));
      w_maxres = fmaxf(w_maxres, rr);
      w_maxlo = fmaxf(w_maxlo, ll);
    } else {
      w_nan++;
    }
    w_exact &= exact;
  }
  if (!stats) return;
  __shared__ float s_norm[PW], s_res[PW], s_lo[PW];
  __shared__ int s_exact[PW], s_nan[PW];
  if (lane == 0) {
    s_norm[wid] = w_maxnorm;
    s_res[wid] = w_maxres;
    s_lo[wid] = w_maxlo;
    s_exact[wid] = w_exact;
    s_nan[wid] = w_nan;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float mn = 0.f, mr = 0.f, ml = 0.f;
    int ex = 1, nn = 0;
    for (int w = 0; w < PW; w++) {
      mn = fmaxf(mn, s_norm[w]);
      mr = fmaxf(mr, s_res[w]);
      ml = fmaxf(ml, s_lo[w]);
      ex &= s_exact[w];
      nn += s_nan[w];
    }
    atomicMax(&stats->max_norm_bits, __float_as_uint(mn));
    atomicMax(&stats->max_resid_bits, __float_as_uint(mr));
    atomicMax(&stats->max_lo_bits, __float_as_uint(ml));
    if (!ex) atomicAnd(&stats->all_exact, 0);
    if (nn) atomicAdd(&stats->n_nan, nn);
  }
}
}  // namespace

int stats_reset(SetStats *stats, cudaStream_t st) {
  SetStats h{0u, 0u, 1, 0, 0u};
  YG_CUDA(cudaMemcpyAsync(stats, &h, sizeof(h), cudaMemcpyHostToDevice, st));
  return OK;
}

int prep_rows(const float *x, long ld, int n, int d, float scale, double *norm64,
              float *norm32, unsigned char *flags, float *resid,
              __nv_bfloat16 *packed, int Kp, __nv_bfloat16 *normpart,
              int normpart_mode, SetStats *stats, cudaStream_t st, int warps) {
  if (n <= 0) return OK;
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    YG_CUDA(cudaGetDevice(&dev));
    YG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  }
  const long cap = (long)sms * 16;
  // eight lanes per row (four rows per warp step) when a row is at most 128
  // float4-aligned columns; one warp per row otherwise
  const int cols = packed ? (Kp > d ? Kp : d) : d;
  const bool vec = (d % 4 == 0) && (ld % 4 == 0) &&
                   ((reinterpret_cast<uintptr_t>(x) & 15) == 0) && (!packed || Kp % 4 == 0) &&
                   (!normpart || (reinterpret_cast<uintptr_t>(normpart) & 15) == 0);
  if (vec && cols <= 128) {
    const int wpb = warps >= 1 && warps <= PW ? warps : PW;
    long blocks = ceil_div(n, wpb * 4);
    if (blocks > cap * PW / wpb) blocks = cap * PW / wpb;
    prep_rows_vec_kernel<8><<<(unsigned)blocks, wpb * 32, 0, st>>>(
        x, ld, n, d, scale, norm64, norm32, flags, resid, packed, Kp, normpart, normpart_mode,
        stats);
  } else {
    long blocks = ceil_div(n, PW);
    if (blocks > cap) blocks = cap;
    prep_rows_kernel<<<(unsigned)blocks, PW * 32, 0, st>>>(x, ld, n, d, scale, norm64, norm32,
                                                           flags, resid, packed, Kp, normpart,
                                                           normpart_mode, stats);
  }
  YG_LAUNCH_CHECK();
  return OK;
}

int prep_rows_split(const float *x, long ld, int n, int d, float scale, int layout,
                    double *norm64, float *norm32, unsigned char *flags, float *lonorm,
                    float *resid, __nv_bfloat16 *packed, int Kp1, __nv_bfloat16 *normpart,
                    int normpart_mode, SetStats *stats, cudaStream_t st) {
  if (n <= 0) return OK;
  int dev = 0, sms = 0;
  YG_CUDA(cudaGetDevice(&dev));
  YG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  long blocks = ceil_div(n, PW);
  if (blocks > (long)sms * 16) blocks = (long)sms * 16;
  prep_split_kernel<<<(unsigned)blocks, PW * 32, 0, st>>>(x, ld, n, d, scale, layout, norm64,
                                                          norm32, flags, lonorm, resid, packed,
                                                          Kp1, normpart, normpart_mode, stats);
  YG_LAUNCH_CHECK();
  return OK;
}

}  // namespace yg
