// Row preparation: norms, exact-class flags, bf16 packing (see prep.cuh).
#include "prep.cuh"

namespace yg {

namespace {
constexpr int PW = 8;  // warps per block

// 16-bit operand encoding of the tensor-core passes: bf16 (F16 = false) or
// IEEE fp16 (F16 = true), both round to nearest even
template <bool F16>
__device__ __forceinline__ uint16_t to16(float v) {
  if (F16) return __half_as_ushort(__float2half_rn(v));
  return __bfloat16_as_ushort(__float2bfloat16_rn(v));
}
template <bool F16>
__device__ __forceinline__ float from16(uint16_t h) {
  if (F16) return __half2float(__ushort_as_half(h));
  return __bfloat162float(__ushort_as_bfloat16(h));
}

// the rounding error of the packed value of v: bf16 shares float's exponent
// range, so bf16(scale * v) = scale * bf16(v) for the power-of-two scales
// used (1, -2); fp16 does not (overflow above 65504, subnormals below 2^-14),
// so its error is taken from the packed value itself (an overflow gives an
// infinite error, which rejects the row's every result)
template <bool F16>
__device__ __forceinline__ float pack_err(float v, float scale, uint16_t packed) {
  if (F16) return v - from16<true>(packed) / scale;
  return v - __bfloat162float(__float2bfloat16_rn(v));
}

// the translation row of row r (null without one)
__device__ __forceinline__ const float *row_mu(const RowShift &sh, long r, int d) {
  if (!sh.mu) return nullptr;
  const long i = sh.row_inst ? (long)sh.row_inst[r] : r / sh.rows_per_inst;
  return sh.mu + i * d;
}

__device__ __forceinline__ float4 sub4(float4 a, float4 b) {
  return make_float4(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z),
                     __fsub_rn(a.w, b.w));
}

// the float norm as three 16-bit parts (11 + 11 + 11 or 8 + 8 + 8 significant
// bits).  bf16 parts sum to n32 exactly.  fp16 parts do when n32 >= 1/2; below
// that the last part may fall among fp16's subnormals, whose spacing is 2^-24,
// and the sum is then within 2^-25 of n32 (the distance bounds of the fp16
// passes add 2^-24 for it).  *ok = false when fp16 cannot hold the norm
// (n32 >= 2^15), *exact = false when the sum is not n32.
template <bool F16>
__device__ __forceinline__ void norm_parts(float n32, uint16_t *p, bool *ok, bool *exact) {
  p[0] = to16<F16>(n32);
  const float r1 = n32 - from16<F16>(p[0]);
  p[1] = to16<F16>(r1);
  const float r2 = r1 - from16<F16>(p[1]);
  p[2] = to16<F16>(r2);
  *ok = !F16 || n32 < 32768.f;
  *exact = !F16 || (*ok && r2 - from16<F16>(p[2]) == 0.f);
}

template <bool F16>
__global__ void __launch_bounds__(PW * 32)
    prep_rows_kernel(const float *__restrict__ x, long ld, int n, int d, float scale,
                     double *norm64, float *norm32, unsigned char *flags, float *resid,
                     uint16_t *packed, int Kp, uint16_t *normpart,
                     int normpart_mode, SetStats *stats, RowShift sh) {
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
    const float *mr = row_mu(sh, row, d);
    // FP32 per element: exact for integer data (partial sums < 2^24), within
    // (d/32 + 6) ulp otherwise -- the certificate's error bound covers that
    float s = 0.f, r = 0.f;
    int exact = 1, bad = 0;
    if (vec) {
      for (int c = lane * 4; c < cols; c += 128) {
        float4 q4 = make_float4(0.f, 0.f, 0.f, 0.f);
        if (c < d) q4 = __ldg(reinterpret_cast<const float4 *>(xr + c));
        if (mr && c < d) q4 = sub4(q4, __ldg(reinterpret_cast<const float4 *>(mr + c)));
        const float e[4] = {q4.x, q4.y, q4.z, q4.w};
        uint16_t hb[4];
#pragma unroll
        for (int t = 0; t < 4; t++) {
          const float v = e[t];
          hb[t] = to16<F16>(scale * v);
          if (c + t < d) {
            s = fmaf(v, v, s);
            exact &= (v == rintf(v)) && (fabsf(v) <= 256.f);
            bad |= !isfinite(v);
            const float dv = pack_err<F16>(v, scale, hb[t]);  // exact
            r = fmaf(dv, dv, r);
          }
        }
        if (packed && c < Kp) {
          uint2 w;
          w.x = (uint32_t)hb[0] | ((uint32_t)hb[1] << 16);
          w.y = (uint32_t)hb[2] | ((uint32_t)hb[3] << 16);
          *reinterpret_cast<uint2 *>(packed + row * Kp + c) = w;
        }
      }
    } else {
      for (int c = lane; c < cols; c += 32) {
        const float v = c < d ? (mr ? __fsub_rn(__ldg(xr + c), __ldg(mr + c)) : __ldg(xr + c))
                              : 0.f;
        const uint16_t h = to16<F16>(scale * v);
        if (c < d) {
          s = fmaf(v, v, s);
          exact &= (v == rintf(v)) && (fabsf(v) <= 256.f);
          bad |= !isfinite(v);
          const float dv = pack_err<F16>(v, scale, h);
          r = fmaf(dv, dv, r);
        }
        if (packed && c < Kp) packed[row * Kp + c] = h;
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
    bool nok = true, nexact = true;
    if (normpart && lane < 16) {
      uint16_t val = to16<F16>(0.f);
      if (normpart_mode == 1) {
        uint16_t p[3];
        norm_parts<F16>((float)s, p, &nok, &nexact);
        val = lane < 3 ? p[lane] : val;
      } else if (normpart_mode == 2) {
        val = to16<F16>(lane < 3 ? 1.f : 0.f);
      }
      normpart[row * 16 + lane] = val;
    }
    const float rr = nok ? sqrtf(r) * (1.f + 1e-5f) : INFINITY;
    // exact class also needs every packed value and norm part to be exact,
    // which fp16 cannot promise for large values and norms
    if (F16) exact &= nok && nexact && r == 0.f;
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
template <int LPR, bool F16>
__global__ void __launch_bounds__(PW * 32)
    prep_rows_vec_kernel(const float *__restrict__ x, long ld, int n, int d, float scale,
                         double *norm64, float *norm32, unsigned char *flags, float *resid,
                         uint16_t *packed, int Kp, uint16_t *normpart,
                         int normpart_mode, SetStats *stats, RowShift sh) {
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
    const float *mr = rv ? row_mu(sh, row, d) : nullptr;
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
      if (mr && c < d) q4s[it] = sub4(q4s[it], __ldg(reinterpret_cast<const float4 *>(mr + c)));
    }
#pragma unroll
    for (int it = 0; it < NIT; it++) {
      const int c = sl * 4 + it * 4 * LPR;
      if (c >= cols) break;
      const float4 q4 = q4s[it];
      const float e[4] = {q4.x, q4.y, q4.z, q4.w};
      uint16_t hb[4];
#pragma unroll
      for (int t = 0; t < 4; t++) {
        const float v = e[t];
        hb[t] = to16<F16>(scale * v);
        if (c + t < d) {
          s = fmaf(v, v, s);
          exact &= (v == rintf(v)) && (fabsf(v) <= 256.f);
          bad |= !isfinite(v);
          const float dv = pack_err<F16>(v, scale, hb[t]);  // exact
          r = fmaf(dv, dv, r);
        }
      }
      if (rv && packed && c < Kp) {
        uint2 w;
        w.x = (uint32_t)hb[0] | ((uint32_t)hb[1] << 16);
        w.y = (uint32_t)hb[2] | ((uint32_t)hb[3] << 16);
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
    bool nok = true, nexact = true;
    uint16_t part[16];
#pragma unroll
    for (int i = 0; i < 16; i++) part[i] = to16<F16>(0.f);
    if (normpart_mode == 1) {
      norm_parts<F16>(s, part, &nok, &nexact);
    } else if (normpart_mode == 2) {
      part[0] = part[1] = part[2] = to16<F16>(1.f);
    }
    const float rr = nok ? sqrtf(r) * (1.f + 1e-5f) : INFINITY;
    if (F16) exact &= nok && nexact && r == 0.f;
    if (rv && sl == 0) {
      if (normpart) {
        uint4 w0, w1;
        uint32_t *u0 = reinterpret_cast<uint32_t *>(&w0), *u1 = reinterpret_cast<uint32_t *>(&w1);
#pragma unroll
        for (int i = 0; i < 4; i++) {
          u0[i] = (uint32_t)part[2 * i] | ((uint32_t)part[2 * i + 1] << 16);
          u1[i] = (uint32_t)part[8 + 2 * i] | ((uint32_t)part[8 + 2 * i + 1] << 16);
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

__global__ void stats_reset_kernel(SetStats *stats) { *stats = SetStats{0u, 0u, 1, 0, 0u}; }

// a kernel, not a copy from a host variable: it may be captured in a CUDA graph
int stats_reset(SetStats *stats, cudaStream_t st) {
  stats_reset_kernel<<<1, 1, 0, st>>>(stats);
  YG_LAUNCH_CHECK();
  return OK;
}

int prep_rows(const float *x, long ld, int n, int d, float scale, double *norm64,
              float *norm32, unsigned char *flags, float *resid,
              __nv_bfloat16 *packed_bf, int Kp, __nv_bfloat16 *normpart_bf,
              int normpart_mode, SetStats *stats, cudaStream_t st, int warps, int f16,
              RowShift shift) {
  uint16_t *packed = reinterpret_cast<uint16_t *>(packed_bf);
  uint16_t *normpart = reinterpret_cast<uint16_t *>(normpart_bf);
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
                   (!normpart || (reinterpret_cast<uintptr_t>(normpart) & 15) == 0) &&
                   (!shift.mu || (reinterpret_cast<uintptr_t>(shift.mu) & 15) == 0);
  if (shift.mu && !shift.row_inst && shift.rows_per_inst < 1) {
    set_error(E_ARG, "prep_rows: rows_per_inst = %d", shift.rows_per_inst);
    return E_ARG;
  }
  if (vec && cols <= 128) {
    const int wpb = warps >= 1 && warps <= PW ? warps : PW;
    long blocks = ceil_div(n, wpb * 4);
    if (blocks > cap * PW / wpb) blocks = cap * PW / wpb;
    auto kern = f16 ? prep_rows_vec_kernel<8, true> : prep_rows_vec_kernel<8, false>;
    kern<<<(unsigned)blocks, wpb * 32, 0, st>>>(x, ld, n, d, scale, norm64, norm32, flags, resid,
                                              packed, Kp, normpart, normpart_mode, stats, shift);
  } else {
    long blocks = ceil_div(n, PW);
    if (blocks > cap) blocks = cap;
    auto kern = f16 ? prep_rows_kernel<true> : prep_rows_kernel<false>;
    kern<<<(unsigned)blocks, PW * 32, 0, st>>>(x, ld, n, d, scale, norm64, norm32, flags, resid,
                                               packed, Kp, normpart, normpart_mode, stats, shift);
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
