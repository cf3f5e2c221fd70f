// Candidate re-ranking with the exactness certificate, THRESH thresholds,
// per-query error bounds, and the exhaustive FP64 fallback (see select.cuh).
#include <float.h>
#include <math.h>

#include "alt.cuh"
#include "select.cuh"

namespace yg {

namespace {

constexpr int RT = 256;  // threads per re-rank block
constexpr int kMaxRegions = 2048;  // candidate regions per query (chunks x halves)
constexpr float kU = 5.9604645e-08f;  // 2^-24

__device__ __forceinline__ bool lex_less(unsigned long long ka, int ia,
                                         unsigned long long kb, int ib) {
  return ka < kb || (ka == kb && (unsigned)ia < (unsigned)ib);
}

// ascending bitonic sort of n (power of two) (key, id) pairs in shared memory
// Ascending bitonic sort of n (a power of two) keys with ids, by the whole
// block.  In a stage of stride s <= 32, thread i handles pairs inside elements
// [64 (i/32 + r blockDim/32), +64) (r = 0, 1, ...): the same 64-element
// segments for its warp in every such stage.  So a stage of stride <= 16 (its
// predecessor has stride <= 32, hence was warp-local too) needs only a warp
// barrier; stages of stride >= 32 follow a stage that may have crossed
// segments and take a block barrier.
__device__ void bitonic_sort(unsigned long long *K, int *I, int n) {
  for (int size = 2; size <= n; size <<= 1) {
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      if (stride >= 32) __syncthreads();
      for (int i = threadIdx.x; i < (n >> 1); i += blockDim.x) {
        const int lo = 2 * i - (i & (stride - 1));
        const int hi = lo + stride;
        const bool up = (lo & size) == 0;
        const unsigned long long klo = K[lo], khi = K[hi];
        const int ilo = I[lo], ihi = I[hi];
        const bool gt = lex_less(khi, ihi, klo, ilo);
        if (gt == up) {
          K[lo] = khi; K[hi] = klo;
          I[lo] = ihi; I[hi] = ilo;
        }
      }
      __syncwarp();
    }
  }
  __syncthreads();
}

__device__ __forceinline__ int next_pow2(int x) {
  int p = 1;
  while (p < x) p <<= 1;
  return p;
}

// distance of query row qv (in shared memory) to base row j, FP32, by one warp
__device__ __forceinline__ float warp_dist32(const float *qv, const float *brow, int d,
                                             int metric) {
  const int lane = threadIdx.x & 31;
  float acc = 0.f;
  for (int c = lane; c < d; c += 32) {
    const float bv = __ldg(brow + c);
    if (metric == METRIC_L2) {
      const float t = qv[c] - bv;
      acc = fmaf(t, t, acc);
    } else {
      acc = fmaf(qv[c], bv, acc);
    }
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  return acc;
}

// FP64 distance, sequential over coordinates (the oracle's summation order)
__device__ __forceinline__ double dist64_seq(const float *qv, const float *brow, int d,
                                             int metric) {
  double s = 0;
  for (int c = 0; c < d; c++) {
    if (metric == METRIC_L2) {
      const double t = (double)qv[c] - (double)__ldg(brow + c);
      s = add_sq64(s, t);
    } else {
      s = add_mul64(s, (double)qv[c], (double)__ldg(brow + c));
    }
  }
  return s;
}

__global__ void __launch_bounds__(RT) rerank_kernel(RerankArgs a, int Mp_alloc) {
  extern __shared__ __align__(16) unsigned char sm_raw[];
  unsigned long long *K = reinterpret_cast<unsigned long long *>(sm_raw);
  int *I = reinterpret_cast<int *>(K + Mp_alloc);
  float *E = reinterpret_cast<float *>(I + Mp_alloc);
  float *qv = E + Mp_alloc;  // the query row, d floats
  __shared__ int sM, sfail, snband, sneed64;
  __shared__ unsigned long long sT;  // TOPC boundary key (lexicographic (v, id))

  const int q = blockIdx.x;
  const int tid = threadIdx.x;
  const int k = a.k, d = a.d;
  const bool L2 = a.metric == METRIC_L2;
  const double qn = L2 ? a.qn64[q] : 0.0;
  const float eps = a.eps ? a.eps[q] : 0.f;
  const bool ex = a.qexact ? a.qexact[q] != 0 : false;
  // a grouped row reads its pair's candidate regions, base, statistics and
  // outputs; otherwise the pass-wide ones
  const GroupPair *gp = a.qpair ? &a.gpairs[a.qpair[q]] : nullptr;
  const long qloc = gp ? (long)(q - gp->qoff) : (long)q;
  const long nqv = gp ? (long)gp->nq : (long)a.nq;
  const long cnt_base = gp ? gp->cnt_off : 0, cand_base = gp ? gp->cand_off : 0;
  const int cap = gp ? gp->cap : a.sel.cap;
  const float *B = gp ? gp->b : a.b;
  const long ldb = gp ? (long)d : a.ldb;
  int *oidx = gp ? gp->out_idx : a.out_idx;
  float *odis = gp ? gp->out_dis : a.out_dis;
  const SetStats *bst = gp ? gp->bs : a.bstats;

  if (tid == 0) {
    sM = 0; sfail = 0; sneed64 = 0;
    sT = ~0ull;
  }
  const float *qrow = gp ? gp->q + qloc * d : a.q + (long)q * a.ldq;
  for (int c = tid; c < d; c += RT) qv[c] = qrow[c];
  __syncthreads();

  // ---- 1. gather candidates as (approx dist, id)
  const ScanSel &s = a.sel;
  if (s.mode == SCAN_TOPC) {
    const int total = s.nchunk * s.C;
    for (int idx = tid; idx < total; idx += RT) {
      const int ch = idx / s.C, sl = idx - ch * s.C;
      const long o = ((long)ch * a.nq + q) * s.C + sl;
      const int id = s.topi[o];
      if (id < 0) continue;
      const float v = s.topv[o];
      const float av = L2 ? (float)((double)v + qn) : v;
      const int pos = atomicAdd(&sM, 1);
      K[pos] = f2ord(av);
      I[pos] = id;
      if (sl == s.C - 1) {  // full chunk: its last entry bounds everything it dropped
        const unsigned long long key = ((unsigned long long)f2ord(av) << 32) | (unsigned)id;
        atomicMin(&sT, key);
      }
    }
  } else {
    // regions (chunk, half) of this query; any overflowing region fails the
    // query.  Offsets first (one thread), then one sweep over all regions.
    const int nreg = gp ? gp->nreg : s.nregion();
    __shared__ int s_off[kMaxRegions + 1];
    __shared__ int s_wsum[RT / 32];
    if (nreg > kMaxRegions) {
      if (tid == 0) sfail = 1;
    } else {
      // exclusive scan of the region counts, RT regions per round
      int run = 0;
      for (int r0 = 0; r0 < nreg; r0 += RT) {
        const int r = r0 + tid;
        int cnt = r < nreg ? s.cnt[cnt_base + (long)r * nqv + qloc] : 0;
        if (cnt > cap) sfail = 1;
        int x = cnt;  // inclusive scan within the warp
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int y = __shfl_up_sync(0xffffffffu, x, o);
          if ((tid & 31) >= o) x += y;
        }
        if ((tid & 31) == 31) s_wsum[tid >> 5] = x;
        __syncthreads();
        int wpre = 0;
        for (int w = 0; w < (tid >> 5); w++) wpre += s_wsum[w];
        int tot = 0;
        for (int w = 0; w < RT / 32; w++) tot += s_wsum[w];
        if (r < nreg) s_off[r] = run + wpre + x - cnt;
        run += tot;
        __syncthreads();
      }
      if (tid == 0) {
        s_off[nreg] = run;
        sM = run;
      }
    }
    __syncthreads();
    if (!sfail && sM <= Mp_alloc) {
      // every slot at once: slot e belongs to the last region r with s_off[r] <= e
      const int M0 = sM;
      for (int e = tid; e < M0; e += RT) {
        int lo = 0, hi = nreg - 1;
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (s_off[mid] <= e) lo = mid; else hi = mid - 1;
        }
        const long o = cand_base + ((long)lo * nqv + qloc) * cap + (e - s_off[lo]);
        const float v = s.candv[o];
        const float av = L2 ? (float)((double)v + qn) : v;
        K[e] = f2ord(av);
        I[e] = s.candi[o];
      }
    }
  }
  __syncthreads();
  const int M = sM;
  float kth_hi = INFINITY;  // upper bound of the k-th exact distance, when found
  if (sfail || M < k || M > Mp_alloc) goto failed;
  {
    const int Mp = next_pow2(M);
    for (int i = M + tid; i < Mp; i += RT) { K[i] = ~0ull; I[i] = 0x7fffffff; }
    __syncthreads();
    bitonic_sort(K, I, Mp);
    if (a.n_cand && tid == 0) atomicAdd(a.n_cand, (unsigned long long)M);

    // boundary of the non-candidates, dist space
    double bound;        // every non-candidate has approx >= bound (TOPC) / > bound (THRESH)
    bool bound_strict;   // true: non-candidates are strictly above bound
    if (s.mode == SCAN_TOPC) {
      bound = (sT == ~0ull) ? INFINITY : (double)ord2f((unsigned)(sT >> 32));
      bound_strict = false;
    } else {
      const float t = s.thr[q];
      bound = L2 ? (double)t + qn : (double)t;
      bound_strict = true;
    }

    if (ex) {
      // approx values are exact: the sorted prefix is the answer.  TOPC:
      // certified when (a_k, id_k) <= the lexicographic boundary.
      if (s.mode == SCAN_TOPC && sT != ~0ull) {
        const unsigned long long kk = K[k - 1];
        const unsigned long long tk = sT >> 32;
        const int tidb = (int)(sT & 0xffffffffu);
        if (!(kk < tk || (kk == tk && (unsigned)I[k - 1] <= (unsigned)tidb))) {
          kth_hi = ord2f((unsigned)kk);  // exact values
          goto failed;
        }
      }
      for (int r = tid; r < k; r += RT) {
        oidx[qloc * k + r] = I[r];
        odis[qloc * k + r] = ord2f((unsigned)K[r]);
      }
      return;
    }

    // ---- 2. band of candidates that can still be in the top k
    const float ak = ord2f((unsigned)K[k - 1]);
    const double slack = 4e-7 * fabs((double)ak) + 1e-30;
    const double lim = (double)ak + 2.0 * (double)eps + slack;
    if (tid == 0) snband = 0;
    __syncthreads();
    {
      int local = 0;
      for (int i = tid; i < M; i += RT)
        if ((double)ord2f((unsigned)K[i]) <= lim) local++;
      atomicAdd(&snband, local);
    }
    __syncthreads();
    const int nband = snband;  // >= k: the sorted prefix up to a_k is inside

    // ---- 3. FP32 re-rank of the band
    const int warp = tid >> 5, nw = RT / 32;
    for (int i = warp; i < nband; i += nw) {
      const float e = warp_dist32(qv, B + (long)I[i] * ldb, d, a.metric);
      if ((tid & 31) == 0) E[i] = e;
    }
    __syncthreads();
    const int nbp = next_pow2(nband);
    for (int i = tid; i < nbp; i += RT) {
      if (i < nband) K[i] = f2ord(E[i]);
      else { K[i] = ~0ull; I[i] = 0x7fffffff; }
    }
    __syncthreads();
    bitonic_sort(K, I, nbp);

    // error model of the FP32 re-rank
    const float rho = (float)(d + 4) * kU;
    float eta = 0.f;
    if (!L2) {
      const float B = __uint_as_float(bst->max_norm_bits);
      eta = (float)(d + 4) * kU * (float)sqrt(fmax(a.qn64 ? a.qn64[q] : 0.0, 0.0)) * B;
    }
    // near ties anywhere up to position k -> FP64 for the whole band
    const int lastpair = imin(k, nband - 1);
    for (int i = tid; i < lastpair; i += RT) {
      const float e0 = ord2f((unsigned)K[i]), e1 = ord2f((unsigned)K[i + 1]);
      const float tol = rho * (fabsf(e0) + fabsf(e1)) + 2.f * eta;
      if (e1 - e0 <= tol) sneed64 = 1;
    }
    __syncthreads();
    double ek_hi;
    if (sneed64) {
      // one thread per candidate, sequential FP64 sum
      for (int i = tid; i < nband; i += RT) {
        const double e = dist64_seq(qv, B + (long)I[i] * ldb, d, a.metric);
        K[i] = d2ord(e);
      }
      __syncthreads();
      bitonic_sort(K, I, nbp);
      const unsigned long long kk = K[k - 1];
      const unsigned long long u = (kk & 0x8000000000000000ull) ? (kk & 0x7fffffffffffffffull) : ~kk;
      const double ek = __longlong_as_double((long long)u);
      ek_hi = ek + 1e-12 * fabs(ek);
      for (int r = tid; r < k; r += RT) {
        const unsigned long long kr = K[r];
        const unsigned long long ur = (kr & 0x8000000000000000ull) ? (kr & 0x7fffffffffffffffull) : ~kr;
        oidx[qloc * k + r] = I[r];
        odis[qloc * k + r] = (float)__longlong_as_double((long long)ur);
      }
    } else {
      const float ek = ord2f((unsigned)K[k - 1]);
      ek_hi = (double)ek + (double)rho * fabs((double)ek) + (double)eta;
      for (int r = tid; r < k; r += RT) {
        oidx[qloc * k + r] = I[r];
        odis[qloc * k + r] = ord2f((unsigned)K[r]);
      }
    }
    // ---- 4. certificate: every non-candidate is provably worse than the k-th
    const double bslack = 4e-7 * fabs(bound);
    const double lowest_outside = bound - (double)eps - bslack;
    const bool ok = bound_strict ? (ek_hi <= lowest_outside) : (ek_hi < lowest_outside);
    if (ok) return;
    // widened so that it also bounds a later FP32 re-rank of the same k-th value
    kth_hi = __double2float_ru(ek_hi + 2.0 * (double)rho * fabs(ek_hi) + 2.0 * (double)eta);
    __syncthreads();
  }
failed:
  if (tid == 0) {
    const int pos = atomicAdd(a.fail_cnt, 1);
    a.fail_list[pos] = q;
    if (a.kth_out) a.kth_out[q] = kth_hi;
  }
}

// ---- group-per-query variant for short TOPC lists (nchunk * C <= 32) ------
// G lanes (8, 16 or 32) hold one query's candidates, one per lane.

template <int G>
__device__ __forceinline__ void group_sort(unsigned long long &key, int &id, unsigned gm) {
  const int gl = threadIdx.x & (G - 1);
#pragma unroll
  for (int size = 2; size <= G; size <<= 1) {
#pragma unroll
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      const unsigned long long pk = __shfl_xor_sync(gm, key, stride);
      const int pi = __shfl_xor_sync(gm, id, stride);
      const bool up = (gl & size) == 0 || size == G;
      const bool lower = (gl & stride) == 0;
      const bool pless = lex_less(pk, pi, key, id);
      const bool take = (lower == up) ? pless : (!pless && (pk != key || pi != id));
      if (take) { key = pk; id = pi; }
    }
  }
}

// FP32 distance of one base row, the group's lanes over strided coordinates
template <int G>
__device__ __forceinline__ float group_dist32(const float *qv, const float *brow, int d,
                                              int metric, unsigned gm) {
  const int gl = threadIdx.x & (G - 1);
  float acc = 0.f;
  for (int c = gl; c < d; c += G) {
    const float bv = __ldg(brow + c);
    if (metric == METRIC_L2) {
      const float t = qv[c] - bv;
      acc = fmaf(t, t, acc);
    } else {
      acc = fmaf(qv[c], bv, acc);
    }
  }
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(gm, acc, o);
  return acc;
}

// Two base rows at once (their loads overlap): each value is the one
// group_dist32 gives, the same per-lane order and the same butterfly.
template <int G>
__device__ __forceinline__ void group_dist32x2(const float *qv, const float *ra, const float *rb,
                                               int d, int metric, unsigned gm, float &ea,
                                               float &eb) {
  const int gl = threadIdx.x & (G - 1);
  float aa = 0.f, ab = 0.f;
  for (int c = gl; c < d; c += G) {
    const float va = __ldg(ra + c), vb = __ldg(rb + c), x = qv[c];
    if (metric == METRIC_L2) {
      const float ta = x - va, tb = x - vb;
      aa = fmaf(ta, ta, aa);
      ab = fmaf(tb, tb, ab);
    } else {
      aa = fmaf(x, va, aa);
      ab = fmaf(x, vb, ab);
    }
  }
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) {
    aa += __shfl_xor_sync(gm, aa, o);
    ab += __shfl_xor_sync(gm, ab, o);
  }
  ea = aa;
  eb = ab;
}

// D_a - D_b = sum_c (a_c - b_c)(a_c + b_c - 2 x_c) for base rows a, b, in
// FP32 without contraction, the group's lanes over strided coordinates then a
// butterfly (every term goes through at most d / G + log2 G <= d + 7
// additions), with the two sums its rounding bound needs: sum |t| and
// sum |a - b| |a + b| (t the rounded terms).
template <int G>
__device__ __forceinline__ void group_pair_diff(const float *qv, const float *ra, const float *rb,
                                                int d, unsigned gm, float &dl, float &st,
                                                float &sps) {
  const int gl = threadIdx.x & (G - 1);
  float t0 = 0.f, t1 = 0.f, t2 = 0.f;
  for (int c = gl; c < d; c += G) {
    const float av = __ldg(ra + c), bv = __ldg(rb + c), x = qv[c];
    const float pp = __fsub_rn(av, bv), s1 = __fadd_rn(av, bv);
    const float tt = __fmul_rn(pp, __fsub_rn(s1, __fadd_rn(x, x)));
    t0 = __fadd_rn(t0, tt);
    t1 = __fadd_rn(t1, fabsf(tt));
    t2 = __fadd_rn(t2, __fmul_rn(fabsf(pp), fabsf(s1)));
  }
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) {
    t0 = __fadd_rn(t0, __shfl_xor_sync(gm, t0, o));
    t1 = __fadd_rn(t1, __shfl_xor_sync(gm, t1, o));
    t2 = __fadd_rn(t2, __shfl_xor_sync(gm, t2, o));
  }
  dl = t0;
  st = t1;
  sps = t2;
}

__device__ __forceinline__ double ord2d(unsigned long long k) {
  const unsigned long long u = (k & 0x8000000000000000ull) ? (k & 0x7fffffffffffffffull) : ~k;
  return __longlong_as_double((long long)u);
}

// One query q by its group of G lanes; returns the number of candidates the
// re-rank looked at (in the group's first lane, 0 elsewhere).
template <int G>
__device__ __forceinline__ unsigned rerank_small_query(const RerankArgs &a, int q) {
  const int gl = threadIdx.x & (G - 1);
  const int gbase = (threadIdx.x & 31) & ~(G - 1);  // first lane of the group in its warp
  const unsigned gm = G == 32 ? 0xffffffffu : (((1u << G) - 1u) << gbase);
  unsigned ncand = 0;
  auto gballot = [&](bool p) -> unsigned {
    const unsigned b = __ballot_sync(gm, p);
    return G == 32 ? b : (b >> gbase) & ((1u << G) - 1u);
  };
  const ScanSel &s = a.sel;
  const bool thresh = s.mode == SCAN_THRESH;
  const int k = a.k, d = a.d;
  const bool L2 = a.metric == METRIC_L2;
  const double qn = L2 ? a.qn64[q] : 0.0;
  const float eps = a.eps ? a.eps[q] : 0.f;
  const bool ex = a.qexact ? a.qexact[q] != 0 : false;
  const float *qv = a.q + (long)q * a.ldq;

  unsigned long long key = ~0ull, tkey = ~0ull;
  int id = 0x7fffffff;
  bool overflow = false;
  if (thresh) {
    // THRESH regions of cap slots (regions * cap <= G): every row with
    // approx <= thr[q]; a region that had more hits than slots fails the query
    if (gl < s.nregion() * s.cap) {
      const int r = gl / s.cap, sl = gl - r * s.cap;
      const int cnt = s.cnt[(long)r * a.nq + q];
      overflow = cnt > s.cap;
      if (sl < cnt && sl < s.cap) {
        const long o = ((long)r * a.nq + q) * s.cap + sl;
        const float v = s.candv[o];
        key = f2ord(L2 ? (float)((double)v + qn) : v);
        id = s.candi[o];
      }
    }
  } else {
    const int M = s.nchunk * s.C;
    if (gl < M) {
      const int ch = gl / s.C, sl = gl - ch * s.C;
      const long o = ((long)ch * a.nq + q) * s.C + sl;
      const int j = s.topi[o];
      if (j >= 0) {
        const float v = s.topv[o];
        const float av = L2 ? (float)((double)v + qn) : v;
        key = f2ord(av);
        id = j;
        if (sl == s.C - 1) tkey = ((unsigned long long)f2ord(av) << 32) | (unsigned)j;
      }
    }
    // boundary: smallest (value, id) that closes a full chunk list
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) {
      const unsigned long long t = __shfl_xor_sync(gm, tkey, o);
      tkey = t < tkey ? t : tkey;
    }
  }
  const int nvalid = __popc(gballot(id != 0x7fffffff));
  bool ok = nvalid >= k && gballot(overflow) == 0u;
  float kth_hi = INFINITY;  // upper bound of the k-th exact distance, when found
  if (ok) {
    if (gl == 0) ncand = (unsigned)nvalid;
    group_sort<G>(key, id, gm);
    if (ex) {
      // THRESH: non-candidates are above thr, so the sorted prefix is the answer
      if (!thresh && tkey != ~0ull) {
        const unsigned long long kk = __shfl_sync(gm, key, k - 1, G);
        const int ik = __shfl_sync(gm, id, k - 1, G);
        const unsigned long long tk = tkey >> 32;
        const unsigned tid_b = (unsigned)(tkey & 0xffffffffu);
        ok = kk < tk || (kk == tk && (unsigned)ik <= tid_b);
        kth_hi = ord2f((unsigned)kk);  // exact values
      }
      if (ok && gl < k) {
        a.out_idx[(long)q * k + gl] = id;
        a.out_dis[(long)q * k + gl] = ord2f((unsigned)key);
      }
    } else {
      const float ak = ord2f((unsigned)__shfl_sync(gm, key, k - 1, G));
      const double lim = (double)ak + 2.0 * (double)eps + 4e-7 * fabs((double)ak) + 1e-30;
      const bool inband = id != 0x7fffffff && (double)ord2f((unsigned)key) <= lim;
      const int nband = __popc(gballot(inband));
      // FP32 re-rank of the band, two candidates at a time across the group
      float e = INFINITY;
      for (int c = 0; c < nband; c += 2) {
        const int ca = __shfl_sync(gm, id, c, G);
        const int cb = __shfl_sync(gm, id, imin(c + 1, nband - 1), G);
        float ea, eb;
        group_dist32x2<G>(qv, a.b + (long)ca * a.ldb, a.b + (long)cb * a.ldb, d, a.metric, gm,
                          ea, eb);
        if (gl == c) e = ea;
        if (gl == c + 1) e = eb;
      }
      key = gl < nband ? (unsigned long long)f2ord(e) : ~0ull;
      if (gl >= nband) id = 0x7fffffff;
      group_sort<G>(key, id, gm);
      const float rho = (float)(d + 4) * kU;
      float eta = 0.f;
      if (!L2) eta = (float)(d + 4) * kU * (float)sqrt(fmax(a.qn64[q], 0.0)) *
                     __uint_as_float(a.bstats->max_norm_bits);
      const float e0 = ord2f((unsigned)key);
      const float e1 = ord2f((unsigned)__shfl_down_sync(gm, key, 1, G));
      const bool tie = gl < imin(k, nband - 1) && (e1 - e0 <= rho * (fabsf(e0) + fabsf(e1)) + 2.f * eta);
      bool need64 = __any_sync(gm, tie);
      if (need64 && k == 1 && L2) {
        // A near tie of the best two alone (the third, if any, clearly worse
        // than the best): the sign of D_a - D_b = sum_c (a_c - b_c)(a_c +
        // b_c - 2 x_c) in FP32 with its rounding bound.  Per coordinate
        // p = fl(a - b), s = fl(a + b), t = fl(p fl(s - 2x)) is within
        // u (|p| |s| + 3 |t|) of its exact term to first order, and the sum
        // adds at most (d + 7) u |t| per term, so |dl - (D_a - D_b)| <=
        // 1.02 u (sum |p| |s| + (d + 10) sum |t|); past that and the rounding
        // of the two FP64 sequential sums that decide a tie (each within
        // (d + 2) 2^-53 of its value), FP64 finds the same order.  Typically
        // the two halves of a split centroid, ~1e-7 of their norm apart.
        const float ea = ord2f((unsigned)__shfl_sync(gm, key, 0, G));
        const float eb = ord2f((unsigned)__shfl_sync(gm, key, 1, G));
        const float ec = nband > 2 ? ord2f((unsigned)__shfl_sync(gm, key, 2, G)) : INFINITY;
        if (!(ec < INFINITY && ec - ea <= rho * (ea + ec))) {
          const int ja = __shfl_sync(gm, id, 0, G), jb = __shfl_sync(gm, id, 1, G);
          float dl, st, sps;
          group_pair_diff<G>(qv, a.b + (long)ja * a.ldb, a.b + (long)jb * a.ldb, d, gm, dl, st,
                             sps);
          const float bound = 1.02f * kU * (sps + (float)(d + 10) * st) +
                              (float)(d + 4) * 1.12e-16f * (ea + eb) * 1.1f;
          if (fabsf(dl) > bound) {
            need64 = false;
            if (dl > 0.f) {  // b is nearer: it takes the first place
              const unsigned long long ko = __shfl_xor_sync(gm, key, 1);
              const int io = __shfl_xor_sync(gm, id, 1);
              if (gl < 2) { key = ko; id = io; }
            }
          }
        }
      }
      double ek_hi;
      if (need64) {
        // FP64, sequential over coordinates, for the whole band
        unsigned long long k64 = ~0ull;
        if (gl < nband) k64 = d2ord(dist64_seq(qv, a.b + (long)id * a.ldb, d, a.metric));
        key = k64;
        group_sort<G>(key, id, gm);
        const double ek = ord2d(__shfl_sync(gm, key, k - 1, G));
        ek_hi = ek + 1e-12 * fabs(ek);
        if (gl < k) {
          a.out_idx[(long)q * k + gl] = id;
          a.out_dis[(long)q * k + gl] = (float)ord2d(key);
        }
      } else {
        const float ek = ord2f((unsigned)__shfl_sync(gm, key, k - 1, G));
        ek_hi = (double)ek + (double)rho * fabs((double)ek) + (double)eta;
        if (gl < k) {
          a.out_idx[(long)q * k + gl] = id;
          a.out_dis[(long)q * k + gl] = ord2f((unsigned)key);
        }
      }
      if (thresh) {
        // every non-candidate has approx > thr, so exact > thr + ||q||^2 - eps
        const float t = s.thr[q];
        const double bound = L2 ? (double)t + qn : (double)t;
        ok = ek_hi <= bound - (double)eps - 4e-7 * fabs(bound);
      } else {
        const double bound = tkey == ~0ull ? INFINITY : (double)ord2f((unsigned)(tkey >> 32));
        ok = ek_hi < bound - (double)eps - 4e-7 * fabs(bound);
      }
      kth_hi = __double2float_ru(ek_hi + 2.0 * (double)rho * fabs(ek_hi) + 2.0 * (double)eta);
    }
  }
  if (!ok && thresh && nvalid >= k && kth_hi == INFINITY && a.kth_out) {
    // a region overflowed: the candidates it did keep are rows of the base,
    // so the k-th smallest of their exact distances bounds the query's k-th
    // from above; the band pass that settles the query starts from it instead
    // of the looser threshold this pass was given
    group_sort<G>(key, id, gm);  // the valid ones first
    float e = INFINITY;
    for (int c = 0; c < nvalid; c++) {
      const int cid = __shfl_sync(gm, id, c, G);
      const float ec = group_dist32<G>(qv, a.b + (long)cid * a.ldb, d, a.metric, gm);
      if (gl == c) e = ec;
    }
    unsigned long long ekey = gl < nvalid ? (unsigned long long)f2ord(e) : ~0ull;
    int eid = id;
    group_sort<G>(ekey, eid, gm);
    const float ek = ord2f((unsigned)__shfl_sync(gm, ekey, k - 1, G));
    const float rho = (float)(d + 4) * kU;
    float eta = 0.f;
    if (!L2) eta = (float)(d + 4) * kU * (float)sqrt(fmax(a.qn64[q], 0.0)) *
                   __uint_as_float(a.bstats->max_norm_bits);
    const double hi = (double)ek + (double)rho * fabs((double)ek) + (double)eta;
    kth_hi = __double2float_ru(hi + 2.0 * (double)rho * fabs(hi) + 2.0 * (double)eta);
  }
  if (!ok && gl == 0) {
    const int pos = atomicAdd(a.fail_cnt, 1);
    a.fail_list[pos] = q;
    if (a.kth_out) a.kth_out[q] = kth_hi;
  }
  return ncand;
}

// The lexicographic minimum of (key, id) over the group's lanes (ids as
// unsigned), by two reductions: the least key, then the least id holding it.
template <int G>
__device__ __forceinline__ void group_argmin(unsigned key, int id, unsigned gm, unsigned &mk,
                                             int &mi) {
  mk = __reduce_min_sync(gm, key);
  mi = (int)__reduce_min_sync(gm, key == mk ? (unsigned)id : 0xffffffffu);
}

// rerank_small_query for k = 1 (the k-means assignment): the same candidates,
// band, distances, tie rules, certificate and outputs, with the orderings
// the general form takes from two sorts of the group's lanes read off by
// reductions instead (the least, second and third (value, id) of the band).
template <int G>
__device__ __forceinline__ unsigned rerank_small_k1(const RerankArgs &a, int q) {
  const int gl = threadIdx.x & (G - 1);
  const int gbase = (threadIdx.x & 31) & ~(G - 1);  // first lane of the group in its warp
  const unsigned gm = G == 32 ? 0xffffffffu : (((1u << G) - 1u) << gbase);
  unsigned ncand = 0;
  auto gballot = [&](bool p) -> unsigned {
    const unsigned b = __ballot_sync(gm, p);
    return G == 32 ? b : (b >> gbase) & ((1u << G) - 1u);
  };
  const ScanSel &s = a.sel;
  const bool thresh = s.mode == SCAN_THRESH;
  const int d = a.d;
  const bool L2 = a.metric == METRIC_L2;
  const double qn = L2 ? a.qn64[q] : 0.0;
  const float eps = a.eps ? a.eps[q] : 0.f;
  const bool ex = a.qexact ? a.qexact[q] != 0 : false;
  const float *qv = a.q + (long)q * a.ldq;

  unsigned key = 0xffffffffu;  // f2ord of the approximate value
  int id = 0x7fffffff;         // 0x7fffffff: no candidate in this lane
  unsigned long long tkey = ~0ull;
  bool overflow = false;
  if (thresh) {
    if (gl < s.nregion() * s.cap) {
      const int r = gl / s.cap, sl = gl - r * s.cap;
      const int cnt = s.cnt[(long)r * a.nq + q];
      overflow = cnt > s.cap;
      if (sl < cnt && sl < s.cap) {
        const long o = ((long)r * a.nq + q) * s.cap + sl;
        const float v = s.candv[o];
        key = f2ord(L2 ? (float)((double)v + qn) : v);
        id = s.candi[o];
      }
    }
  } else {
    const int M = s.nchunk * s.C;
    unsigned tk = 0xffffffffu, ti = 0xffffffffu;
    if (gl < M) {
      const int ch = gl / s.C, sl = gl - ch * s.C;
      const long o = ((long)ch * a.nq + q) * s.C + sl;
      const int j = s.topi[o];
      if (j >= 0) {
        const float v = s.topv[o];
        const float av = L2 ? (float)((double)v + qn) : v;
        key = f2ord(av);
        id = j;
        if (sl == s.C - 1) { tk = key; ti = (unsigned)j; }
      }
    }
    // boundary: smallest (value, id) that closes a full chunk list
    const unsigned mtk = __reduce_min_sync(gm, tk);
    const unsigned mti = __reduce_min_sync(gm, tk == mtk ? ti : 0xffffffffu);
    tkey = ((unsigned long long)mtk << 32) | mti;
  }
  const bool valid = id != 0x7fffffff;
  const int nvalid = __popc(gballot(valid));
  bool ok = nvalid >= 1 && gballot(overflow) == 0u;
  float kth_hi = INFINITY;  // upper bound of the exact nearest distance, when found
  if (ok) {
    if (gl == 0) ncand = (unsigned)nvalid;
    unsigned k0;
    int i0;
    group_argmin<G>(key, id, gm, k0, i0);
    if (ex) {
      // THRESH: non-candidates are above thr, so the least is the answer
      if (!thresh && tkey != ~0ull) {
        const unsigned tk = (unsigned)(tkey >> 32);
        const unsigned tid_b = (unsigned)(tkey & 0xffffffffu);
        ok = k0 < tk || (k0 == tk && (unsigned)i0 <= tid_b);
        kth_hi = ord2f(k0);  // exact values
      }
      if (ok && gl == 0) {
        a.out_idx[q] = i0;
        a.out_dis[q] = ord2f(k0);
      }
    } else {
      const float ak = ord2f(k0);
      // The band's limit ak + 2 eps + 4e-7 |ak| + 1e-30 in FP32, rounded up,
      // with larger constants and a relative margin: at least its FP64 value,
      // so the band holds every row whose exact distance can be the least.
      // (This part's FP64 pipe runs at 1/64 of the FP32 rate: FP64 is kept
      // for the keys and the THRESH bound.)
      float limf = __fadd_ru(__fadd_ru(ak, __fmul_ru(2.f, eps)),
                             __fadd_ru(__fmul_ru(4.01e-7f, fabsf(ak)), 1.01e-30f));
      limf = __fadd_ru(limf, __fmul_ru(fabsf(limf), 1.2e-7f));
      const bool inband = valid && ord2f(key) <= limf;
      const unsigned bmask = gballot(inband);
      const int nband = __popc(bmask);
      // FP32 distances of the band's members, two at a time across the group
      float e = INFINITY;
      for (unsigned m = bmask; m;) {
        const int la = __ffs(m) - 1;
        m &= m - 1;
        const int lb = m ? __ffs(m) - 1 : la;
        if (m) m &= m - 1;
        const int ca = __shfl_sync(gm, id, la, G);
        const int cb = __shfl_sync(gm, id, lb, G);
        float ea, eb;
        group_dist32x2<G>(qv, a.b + (long)ca * a.ldb, a.b + (long)cb * a.ldb, d, a.metric, gm,
                          ea, eb);
        if (gl == la) e = ea;
        if (gl == lb) e = eb;
      }
      const unsigned ek32 = inband ? f2ord(e) : 0xffffffffu;
      const int eid = inband ? id : 0x7fffffff;
      unsigned e0k, e1k = 0xffffffffu, e2k = 0xffffffffu;
      int j0, j1 = 0x7fffffff;
      group_argmin<G>(ek32, eid, gm, e0k, j0);
      if (nband > 1) {
        const bool r1 = eid != j0;
        group_argmin<G>(r1 ? ek32 : 0xffffffffu, r1 ? eid : 0x7fffffff, gm, e1k, j1);
      }
      const float rho = (float)(d + 4) * kU;
      float eta = 0.f;
      if (!L2) eta = (float)(d + 4) * kU * (float)sqrt(fmax(a.qn64[q], 0.0)) *
                     __uint_as_float(a.bstats->max_norm_bits);
      const float e0 = ord2f(e0k), e1 = ord2f(e1k);
      bool need64 = nband > 1 && (e1 - e0 <= rho * (fabsf(e0) + fabsf(e1)) + 2.f * eta);
      unsigned wk = e0k;
      int wj = j0;
      if (need64 && L2) {
        // the near tie of the best two alone, settled by the sign of their
        // distance difference (rerank_small_query gives the bound)
        if (nband > 2) {
          const bool r2 = eid != j0 && eid != j1;
          e2k = __reduce_min_sync(gm, r2 ? ek32 : 0xffffffffu);
        }
        const float ec = nband > 2 ? ord2f(e2k) : INFINITY;
        if (!(ec < INFINITY && ec - e0 <= rho * (e0 + ec))) {
          float dl, st, sps;
          group_pair_diff<G>(qv, a.b + (long)j0 * a.ldb, a.b + (long)j1 * a.ldb, d, gm, dl, st,
                             sps);
          const float bound = 1.02f * kU * (sps + (float)(d + 10) * st) +
                              (float)(d + 4) * 1.12e-16f * (e0 + e1) * 1.1f;
          if (fabsf(dl) > bound) {
            need64 = false;
            if (dl > 0.f) { wk = e1k; wj = j1; }
          }
        }
      }
      // ekh: an upper bound of the exact nearest distance, rounded up to FP32
      float ekh, ekf = 0.f;
      double ek_hi64 = 0.0;
      if (need64) {
        // FP64, sequential over coordinates, for the whole band
        unsigned long long k64 = ~0ull;
        int i64 = 0x7fffffff;
        if (inband) {
          k64 = d2ord(dist64_seq(qv, a.b + (long)id * a.ldb, d, a.metric));
          i64 = id;
        }
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) {
          const unsigned long long pk = __shfl_xor_sync(gm, k64, o);
          const int pi = __shfl_xor_sync(gm, i64, o);
          if (lex_less(pk, pi, k64, i64)) { k64 = pk; i64 = pi; }
        }
        const double ek = ord2d(k64);
        ek_hi64 = ek + 1e-12 * fabs(ek);
        ekh = __double2float_ru(ek_hi64);
        if (gl == 0) {
          a.out_idx[q] = i64;
          a.out_dis[q] = (float)ek;
        }
      } else {
        ekf = ord2f(wk);
        ekh = __fadd_ru(__fadd_ru(ekf, __fmul_ru(rho, fabsf(ekf))), eta);
        if (gl == 0) {
          a.out_idx[q] = wj;
          a.out_dis[q] = ekf;
        }
      }
      // The certificate ek_hi <= bound - eps - 4e-7 |bound| in FP32 with
      // outward rounding (and 4.01e-7 for the FP64 roundings of the bound): it
      // holds only where the FP64 form holds, so every query it accepts is
      // settled; the few it may reject at the edge go to the band pass.
      if (thresh) {
        // every non-candidate has approx > thr, so exact > thr + ||q||^2 - eps
        const float t = s.thr[q];
        float blo = t, babs = fabsf(t);
        if (L2) {
          const double bd = (double)t + qn;
          blo = __double2float_rd(bd);
          babs = fmaxf(fabsf(blo), fabsf(__double2float_ru(bd)));
        }
        ok = ekh <= __fsub_rd(__fsub_rd(blo, eps), __fmul_ru(4.01e-7f, babs));
      } else {
        const float b = tkey == ~0ull ? INFINITY : ord2f((unsigned)(tkey >> 32));
        ok = ekh < __fsub_rd(__fsub_rd(b, eps), __fmul_ru(4.01e-7f, fabsf(b)));
      }
      if (!ok) {
        // the bound the band pass starts from (as the general form gives it)
        const double ek_hi =
            need64 ? ek_hi64 : (double)ekf + (double)rho * fabs((double)ekf) + (double)eta;
        kth_hi = __double2float_ru(ek_hi + 2.0 * (double)rho * fabs(ek_hi) + 2.0 * (double)eta);
      }
    }
  }
  if (!ok && thresh && nvalid >= 1 && kth_hi == INFINITY && a.kth_out) {
    // a region overflowed: the candidates it did keep are rows of the base,
    // so the least of their exact distances bounds the query's nearest from
    // above; the band pass that settles the query starts from it
    const unsigned vmask = gballot(valid);
    float e = INFINITY;
    for (unsigned m = vmask; m;) {
      const int la = __ffs(m) - 1;
      m &= m - 1;
      const int lb = m ? __ffs(m) - 1 : la;
      if (m) m &= m - 1;
      const int ca = __shfl_sync(gm, id, la, G);
      const int cb = __shfl_sync(gm, id, lb, G);
      float ea, eb;
      group_dist32x2<G>(qv, a.b + (long)ca * a.ldb, a.b + (long)cb * a.ldb, d, a.metric, gm, ea,
                        eb);
      if (gl == la) e = ea;
      if (gl == lb) e = eb;
    }
    const float ek = ord2f(__reduce_min_sync(gm, valid ? f2ord(e) : 0xffffffffu));
    const float rho = (float)(d + 4) * kU;
    float eta = 0.f;
    if (!L2) eta = (float)(d + 4) * kU * (float)sqrt(fmax(a.qn64[q], 0.0)) *
                   __uint_as_float(a.bstats->max_norm_bits);
    const double hi = (double)ek + (double)rho * fabs((double)ek) + (double)eta;
    kth_hi = __double2float_ru(hi + 2.0 * (double)rho * fabs(hi) + 2.0 * (double)eta);
  }
  if (!ok && gl == 0) {
    const int pos = atomicAdd(a.fail_cnt, 1);
    a.fail_list[pos] = q;
    if (a.kth_out) a.kth_out[q] = kth_hi;
  }
  return ncand;
}

// A group of G lanes per query (K1: the k = 1 form); the candidate count goes
// to a.n_cand once per block, from the block's last warp to finish (no
// barrier at the end: a warp whose queries are done leaves at once, however
// long the others take).
template <int G, bool K1>
__global__ void __launch_bounds__(256) rerank_small_kernel(RerankArgs a) {
  constexpr int QPB = 256 / G;  // queries per block
  __shared__ unsigned long long s_cand;
  __shared__ unsigned s_done;
  if (threadIdx.x == 0) {
    s_cand = 0;
    s_done = 0;
  }
  __syncthreads();
  const int q = blockIdx.x * QPB + (int)(threadIdx.x / G);
  unsigned nc = 0;
  if (q < a.nq)  // uniform per group
    nc = K1 ? rerank_small_k1<G>(a, q) : rerank_small_query<G>(a, q);
  if (a.n_cand) {
    const unsigned w = __reduce_add_sync(0xffffffffu, nc);
    if ((threadIdx.x & 31) == 0) {
      if (w) atomicAdd(&s_cand, (unsigned long long)w);
      __threadfence_block();
      if (atomicAdd(&s_done, 1u) == blockDim.x / 32 - 1) {
        __threadfence_block();
        const unsigned long long t = atomicAdd(&s_cand, 0ull);  // every warp's count is in
        if (t) atomicAdd(a.n_cand, t);
      }
    }
  }
}

__global__ void eps_kernel(int nq, int d, int prec, int metric, const double *qn64,
                           const float *qres, const unsigned char *qflag,
                           const SetStats *bs, float *eps, unsigned char *qexact,
                           const int *qpair, const GroupPair *gpairs) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq) return;
  if (qpair) bs = gpairs[qpair[q]].bs;  // grouped: the query's own pair
  const bool ex = qflag[q] && bs->all_exact;
  qexact[q] = ex;
  if (ex) { eps[q] = 0.f; return; }
  const double u = 5.9604644775390625e-08;  // 2^-24
  // norms are FP32 sums: relative error <= (d/32 + 6) u, on both sides
  const double un = ((d + 31) / 32 + 6) * u;
  const double qn = sqrt(fmax(qn64[q], 0.0)) * (1 + 1e-5);
  const double B = (double)__uint_as_float(bs->max_norm_bits);
  double e;
  if (prec == PREC_FP32) {
    const double g = (d + 2) * u * 1.01;
    e = metric == METRIC_L2 ? 2 * g * qn * B + u * (B * B + 2 * qn * B) + u * B * B
                            : g * qn * B;
  } else {
    const double dq = qres ? (double)qres[q] : 0.0;
    const double dB = (double)__uint_as_float(bs->max_resid_bits);
    const double dot = dq * (B + dB) + qn * dB;
    const double Kt = (double)(((d + 63) / 64) * 64 + 16);
    const double acc = Kt * 2 * u * ((metric == METRIC_L2 ? 2 : 1) * (qn + dq) * (B + dB) +
                                     (metric == METRIC_L2 ? 1.001 * B * B : 0.0));
    e = metric == METRIC_L2 ? 2 * dot + u * B * B + acc : dot + acc;
  }
  // ||q||^2 (added in the re-rank) and ||b||^2 (inside v) each off by un relative
  e += un * (qn * qn + B * B);
  // fp16 norm parts: their sum is within 2^-25 of ||b||^2
  if (prec == PREC_FP16) e += u;
  e = e * 1.1 + 1e-30;
  eps[q] = isfinite(e) ? (float)e : INFINITY;
}

__global__ void eps_split_kernel(int nq, int d, int metric, const double *qn64, const float *qlo,
                                 const float *qres2, const unsigned char *qflag,
                                 const SetStats *bs, float *eps, unsigned char *qexact) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq) return;
  const bool ex = qflag[q] && bs->all_exact;
  qexact[q] = ex;
  if (ex) { eps[q] = 0.f; return; }
  const double u = 5.9604644775390625e-08;  // 2^-24
  const double un = ((d + 31) / 32 + 6) * u;
  const double qn = sqrt(fmax(qn64[q], 0.0)) * (1 + 1e-5);
  const double B = (double)__uint_as_float(bs->max_norm_bits);
  const double LB = (double)__uint_as_float(bs->max_lo_bits);
  const double RB = (double)__uint_as_float(bs->max_resid_bits);
  const double lq = (double)qlo[q], rq = (double)qres2[q];
  // q.b - (qh.bh + qh.bl + ql.bh) = ql.bl + rq.b + (q - rq).rb
  const double dot = lq * LB + rq * B + qn * RB;
  const double Kt = (double)(3 * ((d + 63) / 64) * 64 + 16);
  const double L2 = metric == METRIC_L2;
  const double acc = Kt * 2 * u * ((L2 ? 2 : 1) * qn * B * 1.02 + (L2 ? 1.001 * B * B : 0.0));
  double e = (L2 ? 2 * dot + u * B * B : dot) + acc + un * (qn * qn + B * B);
  e = e * 1.1 + 1e-30;
  eps[q] = isfinite(e) ? (float)e : INFINITY;
}

__global__ void thresh_kernel(int nq, int nchunk, int C, int c, const float *topv,
                              const float *eps, float *thr) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq) return;
  // c-th smallest across the sorted per-chunk lists (small: linear merge)
  int heads[64];
  const int nc = nchunk < 64 ? nchunk : 64;
  for (int i = 0; i < nc; i++) heads[i] = 0;
  float v = INFINITY;
  for (int r = 0; r < c; r++) {
    int best = -1;
    float bv = INFINITY;
    for (int i = 0; i < nc; i++) {
      if (heads[i] >= C) continue;
      const float x = topv[((long)i * nq + q) * C + heads[i]];
      if (x < bv) { bv = x; best = i; }
    }
    if (best < 0) { v = INFINITY; break; }
    heads[best]++;
    v = bv;
  }
  const double t = (double)v + 2.0 * (double)eps[q];
  thr[q] = isfinite(t) ? __double2float_ru(t * (1 + 1e-7) + (t < 0 ? -t * 2e-7 : 0.0))
                       : INFINITY;
}

__global__ void band_thr_kernel(int nq, int metric, const float *kth, const double *qn64,
                                const float *eps, float *thr) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq) return;
  const double kk = (double)kth[q], e = (double)eps[q];
  if (!isfinite(kk) || !isfinite(e)) {
    thr[q] = INFINITY;
    return;
  }
  // a row with exact distance x <= kk has approx <= x + e; its v value is
  // approx - ||q||^2 (L2).  The 1e-6 relative margin exceeds the re-rank's
  // 4e-7 boundary slack, so the certificate passes whenever the band held
  // every candidate.
  const double hi = kk + e + 1e-6 * (fabs(kk) + e);
  const double t = metric == METRIC_L2 ? hi - qn64[q] : hi;
  thr[q] = __double2float_ru(t);
}

// ---- exhaustive FP64 path ------------------------------------------------

__global__ void fb_rows_kernel(const int *qlist, int q0, int nb, int d, int metric,
                               const float *__restrict__ Q, long ldq,
                               const float *__restrict__ B, long ldb,
                               const float *__restrict__ w,
                               unsigned long long *rows) {
  extern __shared__ float qs[];
  const int r = blockIdx.y;
  const int qi = qlist ? qlist[q0 + r] : q0 + r;
  for (int c = threadIdx.x; c < d; c += blockDim.x) qs[c] = Q[(long)qi * ldq + c];
  __syncthreads();
  const long j = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nb) return;
  double e = dist64_seq(qs, B + j * ldb, d, metric);
  if (w) e *= (double)w[j];
  // NaN (whatever its sign bit) gets the largest key and is never selected
  rows[(long)r * nb + j] = isnan(e) ? ~0ull : d2ord(e);
}

// the per-coordinate distance types (alt.cuh) of one query against every base
// row: the reference's float value (base row as the first operand, as its
// knn_full passes it), times the weight in float; NaN is never selected, and
// for k = 1 neither is a value >= 1e30 (the reference's argmin starts there,
// yael/nn.c:404-435)
template <int TYPE, bool SSE>
__global__ void fb_rows_alt_kernel(const int *qlist, int q0, int nb, int d,
                                   const float *__restrict__ Q, long ldq,
                                   const float *__restrict__ B, long ldb,
                                   const float *__restrict__ w, int k1,
                                   unsigned long long *rows) {
  extern __shared__ float qs[];
  const int r = blockIdx.y;
  const int qi = qlist ? qlist[q0 + r] : q0 + r;
  for (int c = threadIdx.x; c < d; c += blockDim.x) qs[c] = Q[(long)qi * ldq + c];
  __syncthreads();
  const long j = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nb) return;
  const float *br = B + j * ldb;
  AltAcc acc;
  for (int c = 0; c < d; c++) alt_step<TYPE, SSE>(acc, __ldg(br + c), qs[c], c);
  float e = alt_finish<SSE>(acc);
  if (w) e = __fmul_rn(e, w[j]);
  rows[(long)r * nb + j] = (isnan(e) || (k1 && !(e < 1e30f))) ? ~0ull : d2ord((double)e);
}

template <int TYPE, bool SSE>
void fb_rows_alt(dim3 g, cudaStream_t st, const int *qlist, int q0, int nb, int d, const float *q,
                 long ldq, const float *b, long ldb, const float *w, int k1,
                 unsigned long long *rows) {
  fb_rows_alt_kernel<TYPE, SSE><<<g, 256, (size_t)d * 4, st>>>(qlist, q0, nb, d, q, ldq, b, ldb,
                                                                 w, k1, rows);
}

__global__ void __launch_bounds__(RT) fb_select_kernel(const int *qlist, int q0, int nb, int k,
                                                       const unsigned long long *rows,
                                                       int *out_idx, float *out_dis) {
  extern __shared__ __align__(16) unsigned char sm_raw[];
  const int kp = next_pow2(k);
  unsigned long long *K = reinterpret_cast<unsigned long long *>(sm_raw);
  int *I = reinterpret_cast<int *>(K + kp);
  __shared__ unsigned int hist[256];
  __shared__ unsigned long long sprefix, smask;
  __shared__ int srank, snless, sneq_taken, svalid;
  const int r = blockIdx.x;
  const int qi = qlist ? qlist[q0 + r] : q0 + r;
  const unsigned long long *row = rows + (long)r * nb;
  const int tid = threadIdx.x;

  // number of non-NaN entries
  if (tid == 0) svalid = 0;
  __syncthreads();
  {
    int c = 0;
    for (int j = tid; j < nb; j += RT) c += row[j] != ~0ull;
    atomicAdd(&svalid, c);
  }
  __syncthreads();
  const int keff = imin(k, svalid);
  if (keff > 0) {
    if (tid == 0) { sprefix = 0; smask = 0; srank = keff - 1; }
    __syncthreads();
    for (int pass = 0; pass < 8; pass++) {
      const int shift = 56 - 8 * pass;
      for (int i = tid; i < 256; i += RT) hist[i] = 0;
      __syncthreads();
      const unsigned long long pre = sprefix, msk = smask;
      for (int j = tid; j < nb; j += RT) {
        const unsigned long long key = row[j];
        if ((key & msk) == pre) atomicAdd(&hist[(key >> shift) & 255], 1u);
      }
      __syncthreads();
      if (tid == 0) {
        int rank = srank;
        unsigned int cum = 0;
        int dg = 0;
        for (; dg < 256; dg++) {
          if ((int)(cum + hist[dg]) > rank) break;
          cum += hist[dg];
        }
        srank = rank - (int)cum;
        sprefix = pre | ((unsigned long long)dg << shift);
        smask = msk | (255ull << shift);
      }
      __syncthreads();
    }
    // sprefix = k-th key; take all smaller keys and the first srank+1 equal keys in index order
    const unsigned long long kth = sprefix;
    const int need_eq = srank + 1;
    if (tid == 0) { snless = 0; sneq_taken = 0; }
    __syncthreads();
    for (int j0 = 0; j0 < nb; j0 += RT) {
      const int j = j0 + tid;
      const unsigned long long key = j < nb ? row[j] : ~0ull;
      if (key < kth) {
        const int pos = atomicAdd(&snless, 1);
        K[pos] = key; I[pos] = j;
      }
      // ordered selection of equal keys
      const bool eq = key == kth;
      const unsigned ball = __ballot_sync(0xffffffffu, eq);
      __shared__ int wsum[RT / 32];
      const int lane = tid & 31, wid = tid >> 5;
      if (lane == 0) wsum[wid] = __popc(ball);
      __syncthreads();
      int before = 0;
      for (int w2 = 0; w2 < wid; w2++) before += wsum[w2];
      const int rank_in = before + __popc(ball & ((1u << lane) - 1));
      const int base = sneq_taken;
      if (eq && base + rank_in < need_eq) {
        const int pos = (keff - need_eq) + base + rank_in;
        K[pos] = key; I[pos] = j;
      }
      __syncthreads();
      if (tid == 0) {
        int tot = 0;
        for (int w2 = 0; w2 < RT / 32; w2++) tot += wsum[w2];
        sneq_taken = base + tot;
      }
      __syncthreads();
    }
    for (int i = keff + tid; i < kp; i += RT) { K[i] = ~0ull; I[i] = 0x7fffffff; }
    __syncthreads();
    bitonic_sort(K, I, kp);
  }
  for (int i = tid; i < k; i += RT) {
    if (i < keff) {
      const unsigned long long kr = K[i];
      const unsigned long long ur = (kr & 0x8000000000000000ull) ? (kr & 0x7fffffffffffffffull) : ~kr;
      const float dv = (float)__longlong_as_double((long long)ur);
      if (k == 1 && !(dv < 1e30f)) {
        out_idx[(long)qi * k] = -1;
        out_dis[(long)qi * k] = 1e30f;
      } else {
        out_idx[(long)qi * k + i] = I[i];
        out_dis[(long)qi * k + i] = dv;
      }
    } else if (k == 1) {
      out_idx[(long)qi * k] = -1;
      out_dis[(long)qi * k] = 1e30f;
    } else {
      out_idx[(long)qi * k + i] = -1;
      out_dis[(long)qi * k + i] = __uint_as_float(0xffffffffu);
    }
  }
}

}  // namespace

int rerank(const RerankArgs &a, cudaStream_t st) {
  if (a.nq <= 0) return OK;
  // short candidate sets: a group of 8 to 32 lanes per query
  const bool small_topc = a.sel.mode == SCAN_TOPC && a.sel.nchunk * a.sel.C <= 32;
  const bool small_thresh = a.sel.mode == SCAN_THRESH && !a.gpairs && a.sel.cap > 0 &&
                            a.sel.nregion() * a.sel.cap <= 32;
  if (small_topc || small_thresh) {
    const int M = small_topc ? a.sel.nchunk * a.sel.C : a.sel.nregion() * a.sel.cap;
    const bool k1 = a.k == 1;
    if (M <= 8) {
      if (k1) rerank_small_kernel<8, true><<<(unsigned)ceil_div(a.nq, 32), 256, 0, st>>>(a);
      else rerank_small_kernel<8, false><<<(unsigned)ceil_div(a.nq, 32), 256, 0, st>>>(a);
    } else if (M <= 16) {
      if (k1) rerank_small_kernel<16, true><<<(unsigned)ceil_div(a.nq, 16), 256, 0, st>>>(a);
      else rerank_small_kernel<16, false><<<(unsigned)ceil_div(a.nq, 16), 256, 0, st>>>(a);
    } else {
      if (k1) rerank_small_kernel<32, true><<<(unsigned)ceil_div(a.nq, 8), 256, 0, st>>>(a);
      else rerank_small_kernel<32, false><<<(unsigned)ceil_div(a.nq, 8), 256, 0, st>>>(a);
    }
    YG_LAUNCH_CHECK();
    return OK;
  }
  int Mmax = a.sel.mode == SCAN_TOPC ? a.sel.nchunk * a.sel.C : a.sel.nregion() * a.sel.cap;
  if (a.sel.mode == SCAN_THRESH && a.m_expect > 0 && Mmax > 4 * a.m_expect + 64)
    Mmax = 4 * a.m_expect + 64;
  if (a.gpairs) Mmax = a.max_candidates;  // grouped: sized by the caller over all pairs
  if (Mmax < a.k) Mmax = a.k;
  if (Mmax > kMaxCandidates) Mmax = kMaxCandidates;  // more candidates than this fail the query
  int Mp = 1;
  while (Mp < Mmax) Mp <<= 1;
  // K (8 B) + I (4 B) + E (4 B) per slot, then the query row
  const size_t smem = (size_t)Mp * 16 + (size_t)a.d * 4 + 16;
  YG_CHECK(ensure_smem((const void *)rerank_kernel, smem));
  rerank_kernel<<<a.nq, RT, smem, st>>>(a, Mp);
  YG_LAUNCH_CHECK();
  return OK;
}

int compute_eps(int nq, int d, int prec, int metric, const double *qn64,
                const float *qres, const unsigned char *qflag, const SetStats *bstats,
                float *eps, unsigned char *qexact, cudaStream_t st, const int *qpair,
                const GroupPair *gpairs) {
  if (nq <= 0) return OK;
  eps_kernel<<<(unsigned)ceil_div(nq, 256), 256, 0, st>>>(nq, d, prec, metric, qn64, qres,
                                                          qflag, bstats, eps, qexact, qpair,
                                                          gpairs);
  YG_LAUNCH_CHECK();
  return OK;
}

int compute_eps_split(int nq, int d, int metric, const double *qn64, const float *qlo,
                      const float *qres2, const unsigned char *qflag, const SetStats *bstats,
                      float *eps, unsigned char *qexact, cudaStream_t st) {
  if (nq <= 0) return OK;
  eps_split_kernel<<<(unsigned)ceil_div(nq, 256), 256, 0, st>>>(nq, d, metric, qn64, qlo, qres2,
                                                                qflag, bstats, eps, qexact);
  YG_LAUNCH_CHECK();
  return OK;
}

int thresh_from_sample(int nq, int nchunk, int C, int c, const float *topv,
                       const float *eps, float *thr, cudaStream_t st) {
  if (nq <= 0) return OK;
  if (nchunk > 64) {
    set_error(E_ARG, "thresh_from_sample: %d chunks > 64", nchunk);
    return E_ARG;
  }
  thresh_kernel<<<(unsigned)ceil_div(nq, 128), 128, 0, st>>>(nq, nchunk, C, c, topv, eps, thr);
  YG_LAUNCH_CHECK();
  return OK;
}

int band_thresholds(int nq, int metric, const float *kth, const double *qn64, const float *eps,
                    float *thr, cudaStream_t st) {
  if (nq <= 0) return OK;
  band_thr_kernel<<<(unsigned)ceil_div(nq, 128), 128, 0, st>>>(nq, metric, kth, qn64, eps, thr);
  YG_LAUNCH_CHECK();
  return OK;
}

int exhaustive(int nlist, const int *qlist_dev, int nb, int d, int k, int metric,
               const float *q, long ldq, const float *b, long ldb, const float *w,
               int *out_idx, float *out_dis, void *scratch, size_t scratch_bytes,
               cudaStream_t st) {
  if (nlist <= 0) return OK;
  if (k > kMaxK) {
    set_error(E_UNSUPPORTED, "k=%d above the supported maximum %d", k, kMaxK);
    return E_UNSUPPORTED;
  }
  const size_t per = (size_t)nb * 8;
  int batch = (int)(scratch_bytes / per);
  if (batch < 1) {
    set_error(E_NOMEM, "exhaustive: scratch of %zu bytes below one row of %zu", scratch_bytes, per);
    return E_NOMEM;
  }
  if (batch > 65535) batch = 65535;
  int kp = 1;
  while (kp < k) kp <<= 1;
  const size_t smem_sel = (size_t)kp * 12 + 16;
  YG_CHECK(ensure_smem((const void *)fb_select_kernel, smem_sel));
  unsigned long long *rows = reinterpret_cast<unsigned long long *>(scratch);
  for (int q0 = 0; q0 < nlist; q0 += batch) {
    const int nbt = imin(batch, nlist - q0);
    dim3 g1((unsigned)ceil_div(nb, 256), (unsigned)nbt);
    if (metric >= METRIC_ALT0) {
      const int t = metric - METRIC_ALT0, k1 = k == 1;
      const bool sse = (t == 1 || t == 3) && d % 4 == 0;
      switch (t * 2 + (sse ? 1 : 0)) {
        case 2: fb_rows_alt<1, false>(g1, st, qlist_dev, q0, nb, d, q, ldq, b, ldb, w, k1, rows); break;
        case 3: fb_rows_alt<1, true>(g1, st, qlist_dev, q0, nb, d, q, ldq, b, ldb, w, k1, rows); break;
        case 6: fb_rows_alt<3, false>(g1, st, qlist_dev, q0, nb, d, q, ldq, b, ldb, w, k1, rows); break;
        case 7: fb_rows_alt<3, true>(g1, st, qlist_dev, q0, nb, d, q, ldq, b, ldb, w, k1, rows); break;
        case 8: fb_rows_alt<4, false>(g1, st, qlist_dev, q0, nb, d, q, ldq, b, ldb, w, k1, rows); break;
        case 10: fb_rows_alt<5, false>(g1, st, qlist_dev, q0, nb, d, q, ldq, b, ldb, w, k1, rows); break;
        case 12: fb_rows_alt<6, false>(g1, st, qlist_dev, q0, nb, d, q, ldq, b, ldb, w, k1, rows); break;
        default:
          set_error(E_UNSUPPORTED, "exhaustive: distance type %d", t);
          return E_UNSUPPORTED;
      }
    } else {
      fb_rows_kernel<<<g1, 256, (size_t)d * 4, st>>>(qlist_dev, q0, nb, d, metric, q, ldq, b,
                                                      ldb, w, rows);
    }
    YG_LAUNCH_CHECK();
    fb_select_kernel<<<nbt, RT, smem_sel, st>>>(qlist_dev, q0, nb, k, rows, out_idx, out_dis);
    YG_LAUNCH_CHECK();
  }
  return OK;
}

}  // namespace yg
