// The exact nearest-centroid step of k-means for k <= 256 on the tensor cores
// (yael/kmeans.c:242-244: knn_full with k = 1 against the centroids, which the
// reference runs through sgemm; its nearest-index rule is yael/nn.c:404-435),
// fused with the fixed-point centroid sums of the update (yael/kmeans.c:277-288,
// exact integer sums here) when they fit shared memory.
//
// One persistent CTA per SM walks a contiguous range of units (128-point
// tiles of one instance), so consecutive units mostly share an instance:
//   warp 0      TMA producer: a ring of S stages, each the tile's packed
//               16-bit points (Kp/64 blocks of 128 rows x 128 B, 128B swizzle),
//               their 16-column side block of ones, their per-point norm and
//               packing error (1 KB) and, when two stages fit with them, their
//               FP32 rows (one untiled bulk copy); the instance's packed
//               centroids (and their norm parts, and their FP32 rows when few)
//               in one resident slot, reloaded when the instance changes and
//               its last MMA is done.
//   warp 1      TMEM owner (two 128 x N FP32 accumulators) and MMA issuer:
//               Kp/16 tcgen05.mma 128xNx16 per tile plus one K = 16 step over
//               the side blocks, so the accumulator holds
//               v_j = ||c_j'||^2 - 2 x'.c_j' of every centroid j (x', c': the
//               rows less their instance's mean).
//   warps 2-9   epilogue.  Warps 2-5 (one TMEM lane quadrant each, a thread
//               per point) find the smallest v and mark the band of centroids
//               within 2 eps of it (eps: the rigorous error bound of the
//               16-bit products, the k-NN certificate's bound with the
//               instance's own centroid norms and errors); all eight warps
//               then take sixteen points each (two lanes per point): FP32
//               direct differences over the band, near ties settled by the
//               sign of the distance difference or FP64, and the points that
//               change centroid moved in the fixed-point sums (atomics).
// Every wait is bounded (tc_ptx.cuh); on expiry *err is set, every role leaves
// its loop, the copies and MMAs already issued are waited for, and TMEM is
// freed.
#include <cudaTypedefs.h>
#include <limits.h>
#include <math.h>

#include "kmeans.cuh"
#include "tc_kernel.cuh"

namespace yg {
namespace kmtc {
using namespace ptx;

constexpr int NT = 320;
constexpr int BW = 9;  // band mask words per point (k <= 256: 8 used; odd: no bank conflicts)
constexpr int A_BLK = 128 * 128;  // 128 rows x 64 16-bit columns
constexpr int A_SIDE = 128 * 32;  // 128 rows x 16 16-bit columns

struct Lay {
  int nkb, N, S, fuse, csm, xs;
  size_t stage_bytes, x_off, ts_off, b_off, bside_off, cf_off, band_off, lst_off, acc_off, cnt_off,
      bar_off, total;
};

// xs: every stage also holds the tile's FP32 point rows (128 x d floats)
__host__ __device__ inline Lay make_lay(int nkb, int N, int S, int fuse, int k, int d,
                                       int csm, int xs) {
  Lay L;
  L.nkb = nkb; L.N = N; L.S = S; L.fuse = fuse; L.csm = csm; L.xs = xs;
  size_t off = 0;
  L.x_off = (size_t)nkb * A_BLK + A_SIDE;
  // the tile's per-point norm and packing error (128 x float2) after its rows
  L.ts_off = L.x_off + (xs ? (((size_t)128 * d * 4 + 1023) & ~(size_t)1023) : 0);
  L.stage_bytes = L.ts_off + 1024;
  off += (size_t)S * L.stage_bytes;
  L.b_off = off;     off += (size_t)nkb * N * 128;  // N % 32 == 0: 1024-aligned blocks
  L.bside_off = off; off += (size_t)N * 32;
  L.cf_off = off;    off += csm ? (size_t)N * d * 4 : 0;  // FP32 centroid rows (d % 4 == 0)
  L.band_off = off;  off += (size_t)2 * 128 * BW * 4;
  L.lst_off = off;   off += (size_t)256 * 4;  // the tile's moves: new and old centroids
  off = (off + 15) & ~(size_t)15;
  L.acc_off = off;   off += fuse ? (size_t)k * d * 8 : 0;
  L.cnt_off = off;   off += fuse ? (size_t)k * 4 : 0;
  off = (off + 15) & ~(size_t)15;
  L.bar_off = off;   off += (size_t)(2 * S + 8) * 8 + 16;
  L.total = off + 1024;  // alignment slack of the 1024-byte aligned base
  return L;
}

struct Params {
  const KmTcUnit *units;
  int nunits;
  int d, k, N, Kp, f16;
  const float *v, *C;
  const float2 *tside;         // per unit, per point: (||x'|| rounded up, packing error)
  const float2 *ib;            // per instance: (max centroid norm, max centroid packing error)
  const SetStats *cs;
  const unsigned char *active;
  int *assign;
  float *dis;
  long long *acc;
  int *counts;
  const int *shift;
  int *err;
  int acc_global;              // sums added straight to acc / counts (k * d too large
                               // for shared memory)
  int csm;                     // the instance's FP32 centroid rows staged in shared memory
  int xs;                      // the tile's FP32 point rows staged with it
  int centered;                // the packed rows are translated by the instance's mean
  int delta;                   // the sums hold the previous assignment's: only moves are added
  unsigned long long wait_ns;  // bound of every wait (0: kWaitLimitNs)
  int withhold;                // test switch: the producer issues no load
};

__device__ __forceinline__ float warp_sum(float x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

// fixed_of without branches (the same value): integral x 2^S by a shift,
// otherwise rounded to nearest even from the 24-bit mantissa
__device__ __forceinline__ long long fixed_of_nb(float x, int S) {
  const unsigned u = __float_as_uint(x);
  const int ex = (int)((u >> 23) & 0xffu);
  const unsigned m = (u & 0x7fffffu) | (ex ? 0x800000u : 0u);
  const int sh = (ex ? ex - 150 : -149) + S;
  const int rs = max(1, min(-sh, 31));  // the rounding form's shift (unused for sh >= 0)
  const unsigned q = rs >= 25 ? 0u : m >> rs;
  const unsigned rem = rs >= 25 ? m : m & ((1u << rs) - 1u);
  const unsigned half = rs >= 25 ? 0xffffffffu : 1u << (rs - 1);
  const unsigned rq = q + ((rem > half || (rem == half && (q & 1u))) ? 1u : 0u);
  const long long r = sh >= 0 ? (long long)((unsigned long long)m << min(sh, 63)) : (long long)rq;
  return ex == 0xff ? 0 : (u >> 31) ? -r : r;
}

// fixed_of when x 2^S is an integer (exponent field ex >= 150 - S, not
// Inf/NaN): the 24-bit mantissa shifted left, with the sign
__device__ __forceinline__ long long fixed_of_shift(float x, int S) {
  const unsigned u = __float_as_uint(x);
  const int ex = (int)((u >> 23) & 0xffu);
  const unsigned m = (u & 0x7fffffu) | (ex ? 0x800000u : 0u);
  const unsigned long long r = (unsigned long long)m << (ex - 150 + S);
  const unsigned long long sg = (unsigned long long)((long long)(int)u >> 31);  // 0 or all ones
  return (long long)((r ^ sg) - sg);
}

// whether fixed_of_shift gives fixed_of(x, S): a normal x with x 2^S an
// integer, or +-0 (subnormals, Inf and NaN take fixed_of_nb)
__device__ __forceinline__ bool fixed_shift_ok(float x, int S) {
  const int ex = (int)((__float_as_uint(x) >> 23) & 0xffu);
  return (ex >= 150 - S && ex != 0xff && ex != 0) || (__float_as_uint(x) << 1) == 0u;
}

// The exact decision for the sixteen points r0 .. r0 + 15 of a warp, two
// lanes per point (lanes 2 p and 2 p + 1 for point p; h = lane & 1 takes the
// float4 columns q = 2 i + h).  The lanes of point p start at i = p and wrap
// around, so that any eight consecutive lanes (four points, both halves) read
// eight different bank groups when the rows are a multiple of 128 bytes.
// Per band member the FP32 distance sum_c (x_c - c_c)^2 is summed in that
// order (four partial sums, the two halves added last: deterministic); members come in increasing index order and
// strict '<' keeps the lower index on equal values; a near tie of the best
// two is settled by the sign of their distance difference when that clears
// its rounding bound, by FP64 otherwise (lowest index on equal values).  Writes assign / dis and, for the fused sums, the
// point's move: the centroid it joins to toj and the one it leaves to toa
// (-1 for none; with P.delta == 0 every point joins and none leaves, else
// only a point whose centroid changed moves).
// X: the tile's rows (staged, or global from the tile's first point);
// Ci: the instance's centroid rows (staged or global).
template <bool CSM>
__device__ __forceinline__ void phase_b_decide(const Params &P, const unsigned *bm, int r0,
                                               int np, long p0, const float *X, const float *Ci,
                                               int lane, int d, int k, float rho, int *toj) {
  const int r = r0 + (lane >> 1), h = lane & 1;
  const bool val = r < np;
  // the previous assignment, loaded first (its latency under the distances)
  const int oa = (P.delta && val && h == 0) ? P.assign[p0 + r] : -1;
  const int d4 = d >> 2;
  const int nh = (d4 + 1 - h) >> 1;  // this half's float4 columns
  // the band: a bit per centroid, words of 32
  const int nw = (k + 31) >> 5;
  const unsigned *bw = bm + r * BW;
  int nm = 0;
  for (int w = 0; w < nw; w++) nm += val ? __popc(bw[w]) : 0;
  unsigned mk = val ? bw[0] : 0u;
  int wi = 0;
  const int mmax = (int)__reduce_max_sync(0xffffffffu, (unsigned)nm);
  const float4 *xr = reinterpret_cast<const float4 *>(X + (long)(val ? r : 0) * d);
  const int i0 = (lane >> 1) % max(nh, 1);  // this lane's first column
  float e1 = INFINITY, e2 = INFINITY, e3 = INFINITY;
  int j1 = -1, j2 = -1;
  for (int m = 0; m < mmax; m++) {
    int j = 0;
    if (m < nm) {  // the next member (one is left)
      while (mk == 0u) mk = bw[++wi];
      j = wi * 32 + __ffs(mk) - 1;
      mk &= mk - 1;
    }
    float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
    if (m < nm) {
      const float4 *cr = reinterpret_cast<const float4 *>(Ci + (long)j * d);
#pragma unroll 4
      for (int t = 0; t < nh; t++) {
        int i = i0 + t;
        if (i >= nh) i -= nh;
        const int q = 2 * i + h;
        const float4 xv = xr[q];
        const float4 cv = CSM ? cr[q] : __ldg(cr + q);
        float u = xv.x - cv.x;
        s0 = fmaf(u, u, s0);
        u = xv.y - cv.y;
        s1 = fmaf(u, u, s1);
        u = xv.z - cv.z;
        s2 = fmaf(u, u, s2);
        u = xv.w - cv.w;
        s3 = fmaf(u, u, s3);
      }
    }
    float e = (s0 + s1) + (s2 + s3);
    e += __shfl_xor_sync(0xffffffffu, e, 1);  // the other half (same sum in both lanes)
    if (m < nm) {
      if (e < e1) {
        e3 = e2; e2 = e1; j2 = j1; e1 = e; j1 = j;
      } else if (e < e2) {
        e3 = e2; e2 = e; j2 = j;
      } else if (e < e3) {
        e3 = e;
      }
    }
  }
  int oj = -1;
  float od = 1e30f;
  if (j1 >= 0 && e1 < 1e30f) { oj = j1; od = e1; }
  const bool tie = oj >= 0 && e2 < INFINITY && e2 - e1 <= rho * (e1 + e2);
  bool need64 = tie;
  if (__any_sync(0xffffffffu, tie)) {
    // A near tie of the best two alone (a third is clearly worse than the
    // best): the sign of D_a - D_b = sum_c (a_c - b_c)(a_c + b_c - 2 x_c)
    // (a = j1, b = j2) in FP32 with its rounding bound.  When the sum clears
    // that bound plus the rounding of the two FP64 sequential sums that decide
    // a tie (each within (d + 2) 2^-53 of its value), FP64 would find the same
    // order: typically the two halves of a split centroid, 1e-7 apart.
    const bool pair = tie && !(e3 < INFINITY && e3 - e1 <= rho * (e1 + e3));
    float dl = 0.f, sa = 0.f, sb = 0.f;
    if (pair) {
      const float4 *ca = reinterpret_cast<const float4 *>(Ci + (long)j1 * d);
      const float4 *cb = reinterpret_cast<const float4 *>(Ci + (long)j2 * d);
      for (int t = 0; t < nh; t++) {
        int i = i0 + t;
        if (i >= nh) i -= nh;
        const int q = 2 * i + h;
        const float4 xv = xr[q];
        const float4 av = CSM ? ca[q] : __ldg(ca + q);
        const float4 bv = CSM ? cb[q] : __ldg(cb + q);
        const float ax[4] = {av.x, av.y, av.z, av.w}, bx[4] = {bv.x, bv.y, bv.z, bv.w};
        const float xx[4] = {xv.x, xv.y, xv.z, xv.w};
#pragma unroll
        for (int c = 0; c < 4; c++) {
          const float pp = __fsub_rn(ax[c], bx[c]), s1 = __fadd_rn(ax[c], bx[c]);
          const float tt = __fmul_rn(pp, __fsub_rn(s1, __fadd_rn(xx[c], xx[c])));
          dl = __fadd_rn(dl, tt);
          sa = __fadd_rn(sa, fabsf(tt));
          sb = __fadd_rn(sb, fabsf(pp) * fabsf(s1));
        }
      }
    }
    dl += __shfl_xor_sync(0xffffffffu, dl, 1);
    sa += __shfl_xor_sync(0xffffffffu, sa, 1);
    sb += __shfl_xor_sync(0xffffffffu, sb, 1);
    if (pair) {
      // per coordinate p = fl(a - b), s = fl(a + b), t = fl(p fl(s - 2x)):
      // |t - exact| <= u |p| (|a + b| + 3 |s - 2x|) to first order, and the
      // d / 2 + 1 additions add u per term: |dl - (D_a - D_b)| <=
      // 1.02 u (sum |p| |s| + (d + 10) sum |t|); then the FP64 sums' error
      const float bound = 1.02f * 5.9604645e-08f * (sb + (float)(d + 10) * sa) +
                          (float)(d + 4) * 1.12e-16f * (e1 + e2) * 1.1f;
      if (fabsf(dl) > bound) {
        need64 = false;
        if (dl > 0.f) { oj = j2; od = e2; }
      }
    }
  }
  if (__any_sync(0xffffffffu, need64)) {
    // near tie: FP64 over the members, sequential over coordinates, the two
    // lanes of the point taking alternate members
    double best = INFINITY;
    int bj = INT_MAX;
    if (need64) {
      const float *xs = X + (long)r * d;
      unsigned tk = bw[0];
      int tw = 0;
      for (int m = 0; m < nm; m++) {
        while (tk == 0u) tk = bw[++tw];
        const int j = tw * 32 + __ffs(tk) - 1;
        tk &= tk - 1;
        if ((m & 1) != h) continue;
        const float *cr = Ci + (long)j * d;
        double sd = 0;
        for (int c = 0; c < d; c++) {
          const double t = (double)xs[c] - (double)cr[c];
          sd = add_sq64(sd, t);
        }
        if (sd < best || (sd == best && j < bj)) { best = sd; bj = j; }
      }
    }
    const double ob = __shfl_xor_sync(0xffffffffu, best, 1);
    const int oj2 = __shfl_xor_sync(0xffffffffu, bj, 1);
    if (ob < best || (ob == best && oj2 < bj)) { best = ob; bj = oj2; }
    if (need64) {
      if (bj != INT_MAX && best < 1e30) { oj = bj; od = (float)best; }
      else { oj = -1; od = 1e30f; }
    }
  }
  if (val && h == 0) {
    P.assign[p0 + r] = oj;
    P.dis[p0 + r] = od;
    if (toj) {
      toj[r] = oj != oa ? oj : -1;
      toj[128 + r] = oj != oa ? oa : -1;
    }
  } else if (toj && h == 0) {
    toj[r] = -1;
    toj[128 + r] = -1;
  }
}

// The fused sums of the warp's sixteen points (r0 .. r0 + 15): their moves
// (joins toj[r], leaves toj[128 + r], written by the warp's own decision),
// one after another, lanes over coordinates (lane + 32 i), as 64-bit integer
// atomics into the sums (rows: k x d, in shared memory for an instance whose
// sums fit there, else the instance's global ones) and counts.  Integer sums,
// whose result does not depend on the order; the warps need not wait for one
// another.  X: the tile's rows.
template <int N32>
__device__ __forceinline__ void phase_b_sums(unsigned long long *rows, int *cnts, const int *toj,
                                             int r0, int np, const float *X, int lane, int d,
                                             int sh) {
  // lanes 0-15 hold the sixteen points' (join, leave); a moving point's row
  // is read and converted once for both
  const int r = r0 + (lane & 15);
  const bool pv = lane < 16 && r < np;
  const int oj = pv ? toj[r] : -1, oa = pv ? toj[128 + r] : -1;
  unsigned m = __ballot_sync(0xffffffffu, oj >= 0 || oa >= 0);
  while (m) {
    const int b = __ffs(m) - 1;
    m &= m - 1;
    const int jn = __shfl_sync(0xffffffffu, oj, b), jo = __shfl_sync(0xffffffffu, oa, b);
    const float *xr = X + (long)(r0 + b) * d;
    float xv[N32];
    bool fast = true;
#pragma unroll
    for (int i = 0; i < N32; i++) {
      const int col = lane + 32 * i;
      xv[i] = col < d ? xr[col] : 0.f;
      fast = fast && fixed_shift_ok(xv[i], sh);
    }
    fast = __all_sync(0xffffffffu, fast);  // almost always: no tiny coordinate
#pragma unroll
    for (int i = 0; i < N32; i++) {
      const int col = lane + 32 * i;
      if (col < d) {
        const long long f = fast ? fixed_of_shift(xv[i], sh) : fixed_of_nb(xv[i], sh);
        if (jn >= 0) atomicAdd(rows + (long)jn * d + col, (unsigned long long)f);
        if (jo >= 0) atomicAdd(rows + (long)jo * d + col, (unsigned long long)(-f));
      }
    }
    if (lane == 0) {
      if (jn >= 0) atomicAdd(cnts + jn, 1);
      if (jo >= 0) atomicAdd(cnts + jo, -1);
    }
  }
}

template <int ND>
__global__ void __launch_bounds__(NT, 1)
    km_tc_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapAs,
                 const __grid_constant__ CUtensorMap mapB, const __grid_constant__ CUtensorMap mapBs,
                 const __grid_constant__ CUtensorMap mapC, int S, Params P) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  // aligned by pointer arithmetic on smem_raw (not through an integer), so
  // that the compiler keeps these pointers in the shared address space
  uint8_t *base = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
  const int nkb = P.Kp / 64, N = P.N, k = P.k, d = P.d;
  const bool fuse = P.acc != nullptr;
  const bool sfuse = fuse && !P.acc_global;  // shared-memory sums
  const Lay lay = make_lay(nkb, N, S, sfuse ? 1 : 0, k, d, P.csm, P.xs);
  uint8_t *Stg = base;
  uint8_t *Bs = base + lay.b_off;
  uint8_t *Bside = base + lay.bside_off;
  float *Cf = reinterpret_cast<float *>(base + lay.cf_off);
  unsigned *band = reinterpret_cast<unsigned *>(base + lay.band_off);  // [2][128][BW]
  int *toj = reinterpret_cast<int *>(base + lay.lst_off);    // the tile's chosen centroids
  unsigned long long *sacc = reinterpret_cast<unsigned long long *>(base + lay.acc_off);
  int *scnt = reinterpret_cast<int *>(base + lay.cnt_off);
  uint64_t *bars = reinterpret_cast<uint64_t *>(base + lay.bar_off);
  uint64_t *full = bars, *empty = bars + S, *tfull = bars + 2 * S, *tempty = bars + 2 * S + 2;
  uint64_t *bfull = bars + 2 * S + 4, *bempty = bars + 2 * S + 5, *mdone = bars + 2 * S + 6;
  uint64_t *cempty = bars + 2 * S + 7;  // the staged FP32 centroids read by the epilogue
  uint32_t *tmem_holder = reinterpret_cast<uint32_t *>(bars + 2 * S + 8);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_holder + 1);
  const uint64_t wl = P.wait_ns ? (uint64_t)P.wait_ns : kWaitLimitNs;
  const uint32_t tcols = N * 2 <= 32 ? 32u : N * 2 <= 64 ? 64u : N * 2 <= 128 ? 128u
                         : N * 2 <= 256 ? 256u : 512u;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // this CTA's contiguous range of units
  const int w0 = (int)((long)blockIdx.x * P.nunits / gridDim.x);
  const int w1 = (int)((long)(blockIdx.x + 1) * P.nunits / gridDim.x);

  if (threadIdx.x == 0) {
    for (int s = 0; s < S; s++) {
      mbar_init(&full[s], 1);
      // the MMAs' commit and the eight epilogue warps (the stage's side data,
      // and its FP32 rows when staged)
      mbar_init(&empty[s], 9);
    }
    for (int a = 0; a < 2; a++) {
      mbar_init(&tfull[a], 1);
      mbar_init(&tempty[a], 4);  // the four lane-quadrant warps of the epilogue
    }
    mbar_init(bfull, 1);
    mbar_init(bempty, 1);
    mbar_init(mdone, 1);
    mbar_init(cempty, 8);  // the eight epilogue warps
    *abort_flag = 0;
    fence_mbar_init();
  }
  if (warp == 1) {
    tmem_alloc(tmem_holder, tcols);
    tmem_relinquish();
  }
  if (sfuse && warp >= 2) {
    for (int i = threadIdx.x - 64; i < k * d; i += 256) sacc[i] = 0ull;
    for (int i = threadIdx.x - 64; i < k; i += 256) scnt[i] = 0;
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_holder;

  if (warp == 0) {
    // ---------------- TMA producer
    if (lane == 0 && !P.withhold) {
      int sn = 0;
      uint32_t phn = 0;
      uint32_t issued = 0, last_par = 0;  // per stage: issued at least once, parity of the last
      int cur = -1, nbl = 0;
      bool ok = true;
      const uint32_t abytes0 = (uint32_t)(nkb * A_BLK + A_SIDE);
      const uint32_t bbytes = (uint32_t)(nkb * N * 128 + N * 32 + (P.csm ? N * d * 4 : 0));
      for (int w = w0; w < w1 && ok; w++) {
        const KmTcUnit u = P.units[w];
        if (!P.active[u.inst]) continue;
        if (u.inst != cur) {
          // the previous instance's centroids are free once its MMAs are done
          if (nbl > 0 && !mbar_wait(bempty, (uint32_t)((nbl - 1) & 1), abort_flag, wl)) {
            ok = false;
            break;
          }
          // and the staged FP32 rows once the epilogue is done with them
          if (nbl > 0 && P.csm && !mbar_wait(cempty, (uint32_t)((nbl - 1) & 1), abort_flag, wl)) {
            ok = false;
            break;
          }
          mbar_arrive_expect_tx(bfull, bbytes);
          for (int kb = 0; kb < nkb; kb++)
            tma_load_2d(&mapB, bfull, Bs + (size_t)kb * N * 128, kb * 64, u.inst * k);
          tma_load_2d(&mapBs, bfull, Bside, 0, u.inst * k);
          if (P.csm) tma_load_2d(&mapC, bfull, Cf, 0, u.inst * k);
          nbl++;
          cur = u.inst;
        }
        const int s = sn;
        const uint32_t ph = phn;
        if (++sn == S) { sn = 0; phn ^= 1; }
        if (!mbar_wait(&empty[s], ph ^ 1, abort_flag, wl)) { ok = false; break; }
        uint8_t *sp = Stg + (size_t)s * lay.stage_bytes;
        const uint32_t xbytes = P.xs ? (uint32_t)u.np * d * 4 : 0u;
        mbar_arrive_expect_tx(&full[s], abytes0 + xbytes + 1024u);
        if (P.xs) bulk_load(sp + lay.x_off, P.v + u.p0 * d, xbytes, &full[s]);
        bulk_load(sp + lay.ts_off, P.tside + (long)w * 128, 1024u, &full[s]);
        for (int kb = 0; kb < nkb; kb++)
          tma_load_2d(&mapA, &full[s], sp + (size_t)kb * A_BLK, kb * 64, (int)u.p0);
        tma_load_2d(&mapAs, &full[s], sp + (size_t)nkb * A_BLK, 0, (int)u.p0);
        issued |= 1u << s;
        last_par = (last_par & ~(1u << s)) | (ph << s);
      }
      // every copy issued has landed before the CTA's shared memory is released
      for (int s = 0; s < S; s++)
        if (issued >> s & 1) mbar_wait_drain(&full[s], last_par >> s & 1);
      if (nbl > 0) mbar_wait_drain(bfull, (uint32_t)((nbl - 1) & 1));
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer
    if (lane == 0) {
      const uint32_t idesc = idesc_16_f32(128, N, P.f16 != 0);
      int sn = 0;
      uint32_t phn = 0;
      int it = 0, cur = -1, nbl = 0;
      bool ok = true, any = false;
      for (int w = w0; w < w1 && ok; w++) {
        const KmTcUnit u = P.units[w];
        if (!P.active[u.inst]) continue;
        if (u.inst != cur) {
          if (nbl > 0) umma_commit(bempty);  // the previous centroids' last reads done
          if (!mbar_wait(bfull, (uint32_t)(nbl & 1), abort_flag, wl)) { ok = false; break; }
          nbl++;
          cur = u.inst;
        }
        const int a = it & 1;
        const uint32_t uu = (uint32_t)(it >> 1);
        if (!mbar_wait(&tempty[a], (uu & 1) ^ 1, abort_flag, wl)) { ok = false; break; }
        const int s = sn;
        const uint32_t ph = phn;
        if (++sn == S) { sn = 0; phn ^= 1; }
        if (!mbar_wait(&full[s], ph, abort_flag, wl)) { ok = false; break; }
        tc_fence_after();
        const uint32_t dt = tmem + (uint32_t)(a * N);
        const uint32_t sa = smem_u32(Stg + (size_t)s * lay.stage_bytes);
        const uint32_t sb = smem_u32(Bs);
        for (int kb = 0; kb < nkb; kb++) {
          const uint64_t da = desc_k_sw128(sa + (uint32_t)(kb * A_BLK));
          const uint64_t db = desc_k_sw128(sb + (uint32_t)(kb * N * 128));
#pragma unroll
          for (int kk = 0; kk < 4; kk++)
            umma_bf16(dt, da + (uint64_t)(kk * 2), db + (uint64_t)(kk * 2), idesc,
                      (kb > 0 || kk > 0) ? 1u : 0u);
        }
        umma_bf16(dt, desc_k_sw32(sa + (uint32_t)(nkb * A_BLK)), desc_k_sw32(smem_u32(Bside)),
                  idesc, 1u);
        any = true;
        umma_commit(&empty[s]);
        umma_commit(&tfull[a]);
        it++;
      }
      // every MMA issued has finished with TMEM and shared memory
      if (any) {
        umma_commit(mdone);
        mbar_wait_drain(mdone, 0);
      }
    }
  } else {
    // ---------------- epilogue
    const int ew = warp - 2;       // 0..7
    const int grp = warp & 3;      // TMEM lane quadrant (warps 2-5 read TMEM)
    const int row = grp * 32 + lane;
    const uint32_t lane_base = (uint32_t)(grp * 32) << 16;
    const float u24 = 5.9604645e-08f;
    const float rho = (float)(d + 4) * u24;
    const float Kt = (float)(P.Kp + 16);
    const float un = (float)((d + 31) / 32 + 6) * u24;
    int it = 0, cur = -1;
    bool ok = true;
    auto flush = [&](int inst) {
      asm volatile("bar.sync 1, 256;" ::: "memory");
      const long g0 = (long)inst * k;
      for (int i = threadIdx.x - 64; i < k * d; i += 256) {
        const unsigned long long x = sacc[i];
        if (x) atomicAdd((unsigned long long *)(P.acc + g0 * d + i), x);
        sacc[i] = 0ull;
      }
      for (int i = threadIdx.x - 64; i < k; i += 256) {
        if (scnt[i]) atomicAdd(P.counts + g0 + i, scnt[i]);
        scnt[i] = 0;
      }
      asm volatile("bar.sync 1, 256;" ::: "memory");
    };
    int nbl = 0;  // centroid tiles seen (the staged FP32 rows' bfull phases)
    int esn = 0;  // the ring's stage and phase, followed as the producer does
    uint32_t ephn = 0;
    for (int w = w0; w < w1 && ok; w++) {
      const KmTcUnit u = P.units[w];
      if (!P.active[u.inst]) continue;
      if (u.inst != cur) {
        if (sfuse && cur >= 0) flush(cur);
        // the previous instance's staged rows are no longer read by this warp
        if (P.csm && cur >= 0 && lane == 0) mbar_arrive(cempty);
        if (P.csm) {
          // the new instance's rows have landed (the MMA warp waits on the same
          // phase of bfull before its first MMA of the instance)
          ok = mbar_wait(bfull, (uint32_t)(nbl & 1), abort_flag, wl);
          __syncwarp();
          ok = __all_sync(0xffffffffu, ok);
        }
        nbl++;
        cur = u.inst;
      }
      const int a = it & 1;
      unsigned *bl = band + a * 128 * BW;
      const int xs_s = esn;  // the stage this tile came in
      const uint32_t xs_ph = ephn;
      if (++esn == S) { esn = 0; ephn ^= 1; }
      // the tile's copies have landed (the MMAs waited for them too: this
      // wait only makes them visible here)
      ok = ok && mbar_wait(&full[xs_s], xs_ph, abort_flag, wl);
      __syncwarp();
      ok = __all_sync(0xffffffffu, ok);
      const float2 *ts = reinterpret_cast<const float2 *>(Stg + (size_t)xs_s * lay.stage_bytes +
                                                          lay.ts_off);
      if (ew < 4) {
        const uint32_t uu = (uint32_t)(it >> 1);
        const bool rv = row < u.np;
        ok = ok && mbar_wait(&tfull[a], uu & 1, abort_flag, wl);
        __syncwarp();
        ok = __all_sync(0xffffffffu, ok);
        if (ok) {
          tc_fence_after();
          float eps = 0.f;
          if (rv) {
            const float2 nd = ts[row];
            const float qn = nd.x, dq = nd.y;
            const float2 bd = P.ib[u.inst];  // the instance's centroids
            const float B = bd.x, dB = bd.y;
            const float dot = dq * (B + dB) + qn * dB;
            const float accb = Kt * 2.f * u24 * (2.f * (qn + dq) * (B + dB) + 1.001f * B * B);
            // the translation: x' = fl(x - mu), c' = fl(c - mu) are off by
            // at most u ||x'||, u ||c'||, which moves ||x - c||^2 - ||x'||^2
            // away from ||x' - c'||^2 - ||x'||^2 by at most 2 u (qn + B)^2 (1 + tiny)
            const float tr = P.centered ? 2.01f * u24 * (qn + B) * (qn + B) : 0.f;
            // (fp16 norm parts: their sum is within 2^-25 of ||c'||^2)
            eps = (2.f * dot + u24 * B * B + accb + un * (qn * qn + B * B) + tr +
                   (P.f16 ? u24 : 0.f)) * 1.1f + 1e-30f;
            // an infinite residual (a row fp16 cannot hold) times a zero one
            // is NaN: such a point re-checks every centroid
            if (!(eps <= 3.0e38f)) eps = INFINITY;
          }
          const uint32_t tc = tmem + lane_base + (uint32_t)(a * N);
          uint32_t r[32];
          float vmin = INFINITY;
          for (int c0 = 0; c0 < N; c0 += 32) {
            tmem_ld32(tc + (uint32_t)c0, r);
            tmem_ld_wait(r);
            // a tree of minima (fminf: any order gives the same minimum)
            float m16[16];
#pragma unroll
            for (int i = 0; i < 16; i++)
              m16[i] = fminf(c0 + i < k ? __uint_as_float(r[i]) : INFINITY,
                             c0 + i + 16 < k ? __uint_as_float(r[i + 16]) : INFINITY);
#pragma unroll
            for (int w = 8; w > 0; w >>= 1)
#pragma unroll
              for (int i = 0; i < w; i++) m16[i] = fminf(m16[i], m16[i + w]);
            vmin = fminf(vmin, m16[0]);
          }
          const float lim = vmin + 2.f * eps;
          // the members: a bit per centroid within 2 eps of the smallest; all
          // of them without a usable bound, none for no point (or no finite
          // distance)
          const bool all = rv && eps == INFINITY, none = !rv || (!all && !(vmin < INFINITY));
          for (int c0 = 0; c0 < N; c0 += 32) {
            if (N > 32) {  // with one chunk r still holds it
              tmem_ld32(tc + (uint32_t)c0, r);
              tmem_ld_wait(r);
            }
            unsigned mk = 0u;
#pragma unroll
            for (int i = 0; i < 32; i++)
              mk |= (c0 + i < k && (all || __uint_as_float(r[i]) <= lim)) ? 1u << i : 0u;
            bl[row * BW + (c0 >> 5)] = none ? 0u : mk;
          }
          tc_fence_before();
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&tempty[a]);
      }
      // the band lists of this tile are written (and the other buffer's were
      // read by every warp before it): one barrier per tile, all warps agree
      ok = bar_red_and_256(ok);
      if (!ok) break;
      // phase B: the exact decision, sixteen points per warp, then the sums
      const int sh = fuse ? P.shift[u.inst] : 0;
      const float *Ci = P.csm ? Cf : P.C + (long)u.inst * k * d;
      const float *Xs = reinterpret_cast<const float *>(Stg + (size_t)xs_s * lay.stage_bytes +
                                                        lay.x_off);
      const float *X = P.xs ? Xs : P.v + u.p0 * d;
      if (P.csm)
        phase_b_decide<true>(P, bl, ew * 16, u.np, u.p0, X, Ci, lane, d, k, rho,
                             fuse ? toj : nullptr);
      else
        phase_b_decide<false>(P, bl, ew * 16, u.np, u.p0, X, Ci, lane, d, k, rho,
                              fuse ? toj : nullptr);
      if (fuse) {
        __syncwarp();  // the warp's own moves are in toj
        if (sfuse)
          phase_b_sums<ND>(sacc, scnt, toj, ew * 16, u.np, X, lane, d, sh);
        else
          phase_b_sums<ND>(reinterpret_cast<unsigned long long *>(P.acc) + (long)u.inst * k * d,
                           P.counts + (long)u.inst * k, toj, ew * 16, u.np, X, lane, d, sh);
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[xs_s]);  // this warp is done with the tile's stage
      it++;
    }
    if (sfuse && ok && cur >= 0) flush(cur);
  }

  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 1) {
    __syncwarp();
    tmem_dealloc(tmem, tcols);
  }
  if (threadIdx.x == 0 && *abort_flag && P.err) atomicExch(P.err, 1);
}

}  // namespace kmtc

namespace {
// a tensor map over FP32 rows, no swizzle (box: cols x rows)
int make_map_f32(CUtensorMap *m, const void *ptr, uint64_t cols, uint64_t rows, uint32_t box_cols,
                 uint32_t box_rows) {
  YG_CHECK(tck::get_encode());
  if (!ptr || (reinterpret_cast<uintptr_t>(ptr) & 15) || ((cols * 4) & 15) || rows == 0) {
    set_error(E_ARG, "tensor map (f32): null / misaligned operand");
    return E_ARG;
  }
  cuuint64_t dims[2] = {cols, rows};
  cuuint64_t strides[1] = {cols * 4};
  cuuint32_t box[2] = {box_cols, box_rows};
  cuuint32_t es[2] = {1, 1};
  CUresult r = tck::g_encode(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void *>(ptr), dims,
                             strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                             CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error(E_CUDA, "cuTensorMapEncodeTiled (f32) failed (%d)", (int)r);
    return E_CUDA;
  }
  return OK;
}
}  // namespace

namespace {
__global__ void tile_side_kernel(const KmTcUnit *units, const double *xn64, const float *xres,
                                 float2 *tside) {
  const KmTcUnit u = units[blockIdx.x];
  const int r = threadIdx.x;
  float2 o = make_float2(0.f, 0.f);
  if (r < u.np) {
    const long p = u.p0 + r;
    o.x = sqrtf(fmaxf((float)xn64[p], 0.f)) * (1.f + 1e-5f);
    o.y = xres[p];
  }
  tside[(long)blockIdx.x * 128 + r] = o;
}
}  // namespace

int km_tc_tile_side(const KmTcUnit *units, int nunits, const double *xn64, const float *xres,
                    float2 *tside, cudaStream_t st) {
  if (nunits <= 0) return OK;
  tile_side_kernel<<<nunits, 128, 0, st>>>(units, xn64, xres, tside);
  YG_LAUNCH_CHECK();
  return OK;
}

namespace {
// per instance, over its k centroid rows: (max ||c'|| as the packing's
// statistics round it, max packing error).  fmaxf passes over NaN (a row with
// a NaN value is never chosen: its distances are NaN) and keeps +inf (an
// overflowing norm or a row fp16 cannot hold: no usable bound)
__global__ void inst_bound_kernel(const float *cnorm, const float *cres, int k, float2 *ib) {
  const long r0 = (long)blockIdx.x * k;
  float b = 0.f, e = 0.f;
  for (int j = threadIdx.x; j < k; j += 32) {
    b = fmaxf(b, sqrtf(cnorm[r0 + j]) * (1.f + 1e-5f));
    e = fmaxf(e, cres[r0 + j]);
  }
  for (int o = 16; o > 0; o >>= 1) {
    b = fmaxf(b, __shfl_xor_sync(0xffffffffu, b, o));
    e = fmaxf(e, __shfl_xor_sync(0xffffffffu, e, o));
  }
  if (threadIdx.x == 0) ib[blockIdx.x] = make_float2(b, e);
}
}  // namespace

bool km_tc_supported(int d, int k, const float *v, const float *C) {
  if (!(d >= 4 && d % 4 == 0 && d <= 256 && k >= 1 && k <= kTcMaxK &&
        (reinterpret_cast<uintptr_t>(v) & 15) == 0 && (reinterpret_cast<uintptr_t>(C) & 15) == 0))
    return false;
  // a ring of two stages beside the centroid tile, without staging or
  // shared-memory sums, must fit (not so for d > 128 with k > 224)
  const int Kp = ((d + 63) / 64) * 64, N = ((k + 31) / 32) * 32;
  return kmtc::make_lay(Kp / 64, N, 2, 0, k, d, 0, 0).total <= 227 * 1024;
}

bool km_tc_fuses(int d, int k) { return (size_t)k * d * 8 <= 48 * 1024; }

int km_tc_assign(const KmTcUnit *units, int nunits, const KmTcPoints &P, const float *v, int d,
                 const float *C, int ninst, int k, void *cpk, void *cside, float *cscratch,
                 float2 *ibound, SetStats *cstats, const unsigned char *active, int *assign,
                 float *dis, long long *acc, int *counts, const int *shift, int delta, int *err,
                 cudaStream_t st) {
  using namespace kmtc;
  if (nunits <= 0) return OK;
  if (!km_tc_supported(d, k, v, C) || P.Kp != ((d + 63) / 64) * 64) {
    set_error(E_UNSUPPORTED, "km_tc_assign: d=%d k=%d Kp=%d", d, k, P.Kp);
    return E_UNSUPPORTED;
  }
  const int N = ((k + 31) / 32) * 32, nkb = P.Kp / 64;
  const long ncl = (long)ninst * k;
  // the centroids, packed as the points are (same 16-bit format)
  YG_CHECK(stats_reset(cstats, st));
  RowShift rs;
  rs.mu = P.mu;
  rs.rows_per_inst = k;
  float *cnorm = cscratch, *cres = cscratch + ncl;
  YG_CHECK(prep_rows(C, d, (int)ncl, d, 1.f, nullptr, cnorm, nullptr, cres,
                     (__nv_bfloat16 *)cpk, P.Kp, (__nv_bfloat16 *)cside, 1, cstats, st, 8, P.f16,
                     rs));
  // each instance's own largest centroid norm and packing error: a point is
  // compared with its instance's centroids only, so these bound its errors
  inst_bound_kernel<<<(unsigned)ninst, 32, 0, st>>>(cnorm, cres, k, ibound);
  YG_LAUNCH_CHECK();
  // the sums go through shared memory when an instance's k x d fit, else
  // straight to the global accumulators; the instance's FP32 centroid rows
  // are staged when they are few.  Both give way, staging first, when a ring
  // of two stages would not fit beside them.
  int acc_global = acc != nullptr && !km_tc_fuses(d, k);
  int fuse = acc != nullptr && !acc_global;
  int csm = (size_t)N * d * 4 <= 32 * 1024;
  int xs = 1;
  auto fits = [&](int S_) {
    return make_lay(nkb, N, S_, fuse, k, d, csm, xs).total <= 227 * 1024;
  };
  // the tile's FP32 rows are staged when two stages still fit with them
  if (!fits(2)) xs = 0;
  if (!fits(2)) csm = 0;
  if (!fits(2) && fuse) {
    fuse = 0;
    acc_global = 1;
  }
  int S = 6;
  while (S > 2 && !fits(S)) S--;
  const Lay lay = make_lay(nkb, N, S, fuse, k, d, csm, xs);
  if (lay.total > 227 * 1024) {
    set_error(E_UNSUPPORTED, "km_tc_assign: shared memory %zu too large (d=%d k=%d)", lay.total,
              d, k);
    return E_UNSUPPORTED;
  }
  const int d4 = d / 4;
  auto kern = d4 <= 16 ? km_tc_kernel<2> : d4 <= 24 ? km_tc_kernel<3> : d4 <= 32 ? km_tc_kernel<4>
              : d4 <= 48 ? km_tc_kernel<6> : km_tc_kernel<8>;
  YG_CHECK(ensure_smem((const void *)kern, lay.total));
  CUtensorMap mA, mAs, mB, mBs, mC;
  YG_CHECK(tck::make_map(&mA, P.pk, P.Kp, P.n, (uint64_t)P.Kp * 2, 64, 128,
                         CU_TENSOR_MAP_SWIZZLE_128B));
  YG_CHECK(tck::make_map(&mAs, P.side, 16, P.n, 32, 16, 128, CU_TENSOR_MAP_SWIZZLE_32B));
  YG_CHECK(tck::make_map(&mB, cpk, P.Kp, ncl, (uint64_t)P.Kp * 2, 64, (uint32_t)N,
                         CU_TENSOR_MAP_SWIZZLE_128B));
  YG_CHECK(tck::make_map(&mBs, cside, 16, ncl, 32, 16, (uint32_t)N, CU_TENSOR_MAP_SWIZZLE_32B));
  if (csm) YG_CHECK(make_map_f32(&mC, C, d, ncl, (uint32_t)d, (uint32_t)N));
  else mC = mBs;
  int dev = 0, nsm = 0;
  YG_CUDA(cudaGetDevice(&dev));
  YG_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  Params p;
  p.units = units; p.nunits = nunits; p.d = d; p.k = k; p.N = N; p.Kp = P.Kp; p.f16 = P.f16;
  p.v = v; p.C = C; p.tside = P.tside; p.ib = ibound; p.cs = cstats; p.active = active;
  p.assign = assign; p.dis = dis; p.acc = acc; p.counts = counts; p.shift = shift; p.err = err;
  p.acc_global = acc_global;
  p.csm = csm;
  p.xs = xs;
  p.centered = P.mu != nullptr;
  p.delta = acc != nullptr && delta ? 1 : 0;
  p.wait_ns = wait_limit_ns();
  p.withhold = test_withhold_loads() ? 1 : 0;
  const unsigned g = (unsigned)(nunits < nsm ? nunits : nsm);
  kern<<<g, NT, lay.total, st>>>(mA, mAs, mB, mBs, mC, S, p);
  YG_LAUNCH_CHECK();
  return OK;
}

}  // namespace yg
