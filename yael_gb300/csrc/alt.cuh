// The per-coordinate distance types of yael (yael/nn.c:164-350), in the
// reference's arithmetic on x86: L1 (type 1) and chi2 (type 3) with
// d % 4 == 0 in four float lanes (its SSE2 form: lane l takes the coordinates
// c = l mod 4, the lanes are then added left to right); every other case a
// double sum, in coordinate order, of float terms, rounded to float.  All
// operations are round-to-nearest and unfused, so a caller that walks the
// coordinates in order reproduces the reference's value exactly.
#pragma once
#include "common.cuh"

namespace yg {

// metric codes of these types in the k-NN pipeline (beside METRIC_L2 / _DOT)
constexpr int METRIC_ALT0 = 100;  // METRIC_ALT0 + t, t in {1, 3, 4, 5, 6}

struct AltAcc {
  double sum = 0.0;
  float lane[4] = {0.f, 0.f, 0.f, 0.f};
};

template <int TYPE, bool SSE>
__device__ __forceinline__ void alt_step(AltAcc &s, float av, float bv, int c) {
  if (SSE) {
    float t;
    if (TYPE == 1) {
      t = fabsf(__fsub_rn(av, bv));
    } else {  // chi2: (a - b)^2 / (a + b) where a != b, else 0
      const float df = __fsub_rn(av, bv);
      t = av != bv ? __fdiv_rn(__fmul_rn(df, df), __fadd_rn(av, bv)) : 0.f;
    }
    s.lane[c & 3] = __fadd_rn(s.lane[c & 3], t);
  } else if (TYPE == 1) {
    s.sum = __dadd_rn(s.sum, (double)fabsf(__fsub_rn(av, bv)));
  } else if (TYPE == 2) {
    const double df = (double)__fsub_rn(av, bv);
    s.sum = __dadd_rn(s.sum, __dmul_rn(df, df));
  } else if (TYPE == 3) {
    const float sm = __fadd_rn(av, bv);
    if (sm != 0.f) {
      const double df = (double)__fsub_rn(av, bv);
      s.sum = __dadd_rn(s.sum, __ddiv_rn(__dmul_rn(df, df), (double)sm));
    }
  } else if (TYPE == 4) {
    const float den = fabsf(__fadd_rn(av, bv));
    if (den != 0.f) {
      const double df = (double)__fsub_rn(av, bv);
      s.sum = __dadd_rn(s.sum, __ddiv_rn(__dmul_rn(df, df), (double)den));
    }
  } else if (TYPE == 5) {
    s.sum = __dadd_rn(s.sum, (double)(av < bv ? av : bv));
  } else {  // 6
    s.sum = __dadd_rn(s.sum, (double)__fmul_rn(av, bv));
  }
}

template <bool SSE>
__device__ __forceinline__ float alt_finish(const AltAcc &s) {
  return SSE ? __fadd_rn(__fadd_rn(__fadd_rn(s.lane[0], s.lane[1]), s.lane[2]), s.lane[3])
             : (float)s.sum;
}

}  // namespace yg
