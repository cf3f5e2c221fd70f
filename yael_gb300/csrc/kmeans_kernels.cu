// Device kernels of the k-means Lloyd step (see kmeans.cuh).
#include <limits.h>
#include <math.h>

#include <cub/device/device_radix_sort.cuh>

#include "autotune.cuh"
#include "kmeans.cuh"

namespace yg {

namespace {

constexpr float kU = 5.9604645e-08f;  // 2^-24

// Grouped exact nearest centroid for k <= 64: one block = a run of points of
// one instance, its k x d centroids (and their norms) in shared memory.  The
// scan uses the expanded form (||x||^2 + ||c||^2 - 2 x.c, one FMA per
// coordinate and centroid, float4 loads).  Each value is within
// eps = 2 (d + 8) u (||x||^2 + max ||c||^2) of the exact distance, so only the
// centroids within 2 eps of the best (the band, usually one or two) can be the
// nearest.  The band is re-evaluated by direct differences (relative error
// (d + 4) u); when its best two are closer than that they are decided in FP64,
// sequential over coordinates, lowest index on equality (yael/nn.c:404-435
// semantics).  The reported distance is the direct-difference value.
template <int K, bool VEC>
__global__ void __launch_bounds__(256)
    assign_small_kernel(const KmWork *__restrict__ work, const float *__restrict__ v, int d,
                        const float *__restrict__ C, int k, const unsigned char *active,
                        int *assign, float *dis) {
  extern __shared__ __align__(16) float cs[];  // k x d centroids, then k norms
  float *cn = cs + (((long)k * d + 3) & ~3L);
  __shared__ float s_cmax;
  const KmWork w = work[blockIdx.x];
  if (!active[w.inst]) return;
  const float *Ci = C + (long)w.inst * k * d;
  for (int i = threadIdx.x; i < k * d; i += blockDim.x) cs[i] = Ci[i];
  __syncthreads();
  for (int j = threadIdx.x; j < k; j += blockDim.x) {
    float sn = 0.f;
    for (int c = 0; c < d; c++) sn = fmaf(cs[j * d + c], cs[j * d + c], sn);
    cn[j] = sn;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float m = 0.f;
    for (int j = 0; j < k; j++) m = fmaxf(m, cn[j]);
    s_cmax = m;
  }
  __syncthreads();
  const float cmax = s_cmax;
  for (int pi = threadIdx.x; pi < w.n; pi += blockDim.x) {
    const long p = w.p0 + pi;
    const float *x = v + p * d;
    float acc[K];
#pragma unroll
    for (int j = 0; j < K; j++) acc[j] = 0.f;
    float xn = 0.f;
    if (VEC) {
      const float4 *x4 = reinterpret_cast<const float4 *>(x);
      for (int c4 = 0; c4 < (d >> 2); c4++) {
        const float4 xv = __ldg(x4 + c4);
        xn = fmaf(xv.x, xv.x, xn);
        xn = fmaf(xv.y, xv.y, xn);
        xn = fmaf(xv.z, xv.z, xn);
        xn = fmaf(xv.w, xv.w, xn);
#pragma unroll
        for (int j = 0; j < K; j++) {
          if (j < k) {
            const float4 cv = *reinterpret_cast<const float4 *>(cs + j * d + 4 * c4);
            acc[j] = fmaf(xv.x, cv.x, acc[j]);
            acc[j] = fmaf(xv.y, cv.y, acc[j]);
            acc[j] = fmaf(xv.z, cv.z, acc[j]);
            acc[j] = fmaf(xv.w, cv.w, acc[j]);
          }
        }
      }
    } else {
      for (int c = 0; c < d; c++) {
        const float xv = __ldg(x + c);
        xn = fmaf(xv, xv, xn);
#pragma unroll
        for (int j = 0; j < K; j++)
          if (j < k) acc[j] = fmaf(xv, cs[j * d + c], acc[j]);
      }
    }
    // strict '<' from 1e30 over increasing j (yael/nn.c:404-435)
    float b1 = 1e30f, b2 = 1e30f;
    int i1 = -1;
#pragma unroll
    for (int j = 0; j < K; j++) {
      if (j < k) {
        const float a = (xn + cn[j]) - 2.f * acc[j];
        if (a < b1) {
          b2 = b1;
          b1 = a;
          i1 = j;
        } else if (a < b2) {
          b2 = a;
        }
      }
    }
    // band: every centroid that can still be the nearest (its expanded value is
    // within 2 eps of the best); non-band centroids are certified farther
    const float tol = 4.f * (float)(d + 8) * kU * (xn + cmax);
    unsigned long long band = 0;
#pragma unroll
    for (int j = 0; j < K; j++) {
      if (j < k) {
        const float a = (xn + cn[j]) - 2.f * acc[j];
        if (!(a > b1 + tol)) band |= 1ull << j;
      }
    }
    float out = 1e30f;
    if (i1 >= 0) {
      // direct differences for the band, sequential over coordinates; strict
      // '<' over increasing j
      const float rho = (float)(d + 4) * kU;
      float e1 = INFINITY, e2 = INFINITY;
      int j1 = -1;
      for (unsigned long long bm = band; bm; bm &= bm - 1) {
        const int j = __ffsll((long long)bm) - 1;
        float sd = 0.f;
        for (int c = 0; c < d; c++) {
          const float t = x[c] - cs[j * d + c];
          sd = fmaf(t, t, sd);
        }
        if (sd < e1) {
          e2 = e1;
          e1 = sd;
          j1 = j;
        } else if (sd < e2) {
          e2 = sd;
        }
      }
      if (e2 < INFINITY && e2 - e1 <= rho * (e1 + e2)) {
        // near tie: FP64, sequential over coordinates, lowest index on equality
        double best = INFINITY;
        int bi = -1;
        for (unsigned long long bm = band; bm; bm &= bm - 1) {
          const int j = __ffsll((long long)bm) - 1;
          double sd = 0;
          for (int c = 0; c < d; c++) {
            const double t = (double)x[c] - (double)cs[j * d + c];
            sd = add_sq64(sd, t);
          }
          if (sd < best) {
            best = sd;
            bi = j;
          }
        }
        i1 = bi;
        out = bi >= 0 ? (float)best : 1e30f;
      } else {
        i1 = j1;
        out = j1 >= 0 ? e1 : 1e30f;
      }
    }
    assign[p] = i1;
    dis[p] = out;
  }
}

// The grouped assignment as a register-blocked GEMM (d % 4 == 0, aligned
// rows): a block takes 128 points of one instance at a time; thread (pg, cg)
// accumulates x.c for points 4 pg .. 4 pg + 3 and centroids cg TN .. cg TN +
// TN - 1 (TN = K / 8) from 32-coordinate slices of the points staged
// transposed in shared memory and the transposed centroids, i.e. 4 TN FMAs per
// 1 + TN / 4 shared loads.  Each point's K values live in its 8 consecutive
// lanes, which reduce the best value, the certified band (values within
// 2 eps of the best, eps as assign_small_kernel), its direct-difference
// re-check (sequential over coordinates, the same order as there, so the same
// reported distance) and the FP64 decision of near ties, lowest index first.
// FULL: whole rows are staged (d <= kFullD), so the band re-check reads shared
// memory; else 32-coordinate slices and the re-check reads the rows again.
constexpr int kFullD = 136;
template <int K, bool FULL>
__global__ void __launch_bounds__(256)
    assign_gemm_kernel(const KmWork *__restrict__ work, const float *__restrict__ v, int d,
                       const float *__restrict__ C, int k, const unsigned char *active,
                       int *assign, float *dis) {
  constexpr int TP = 128, TM = 4, TN = K / 8, XS = TP + 4;
  const int DC = FULL ? d : 32;
  extern __shared__ __align__(16) float sm[];
  float *cst = sm;            // [d][K] transposed centroids (zero past k)
  float *cn = cst + d * K;    // [K] norms
  float *xs = cn + K;         // [DC][XS] transposed points (all of d when FULL)
  __shared__ float s_cmax;
  const KmWork w = work[blockIdx.x];
  if (!active[w.inst]) return;
  const int tid = threadIdx.x, pg = tid >> 3, cg = tid & 7;
  const float *Ci = C + (long)w.inst * k * d;
  for (int i = tid; i < d * K; i += blockDim.x) {
    const int c = i / K, j = i - c * K;
    cst[i] = j < k ? Ci[(long)j * d + c] : 0.f;
  }
  __syncthreads();
  for (int j = tid; j < K; j += blockDim.x) {
    float sn = 0.f;
    for (int c = 0; c < d; c++) sn = fmaf(cst[c * K + j], cst[c * K + j], sn);
    cn[j] = sn;
  }
  __syncthreads();
  if (tid == 0) {
    float m = 0.f;
    for (int j = 0; j < k; j++) m = fmaxf(m, cn[j]);
    s_cmax = m;
  }
  __syncthreads();
  const float cmax = s_cmax;
  const float rho = (float)(d + 4) * kU;
  for (int t0 = 0; t0 < w.n; t0 += TP) {
    const int np = min(TP, w.n - t0);
    const float *vt = v + (w.p0 + t0) * (long)d;
    float acc[TM][TN], xn[TM];
#pragma unroll
    for (int i = 0; i < TM; i++) {
      xn[i] = 0.f;
#pragma unroll
      for (int t = 0; t < TN; t++) acc[i][t] = 0.f;
    }
    for (int c0 = 0; c0 < d; c0 += DC) {
      const int n4 = min(DC, d - c0) >> 2, n4p = (n4 + 1) >> 1;
      __syncthreads();  // the previous slice has been read
      // a warp covers 16 consecutive points x one pair of float4 columns: each
      // pair of lanes reads one 32-byte sector and the transposed stores of a
      // warp hit 32 distinct banks (row pitch XS = 4 mod 32)
      for (int idx = tid; idx < TP * 2 * n4p; idx += blockDim.x) {
        const int ln = idx & 31, grp = idx >> 5;
        const int p = (grp % (TP / 16)) * 16 + (ln >> 1);
        const int c4 = 2 * (grp / (TP / 16)) + (ln & 1);
        if (c4 >= n4) continue;
        float4 val = make_float4(0.f, 0.f, 0.f, 0.f);
        if (p < np) val = __ldg(reinterpret_cast<const float4 *>(vt + (long)p * d + c0) + c4);
        xs[(4 * c4 + 0) * XS + p] = val.x;
        xs[(4 * c4 + 1) * XS + p] = val.y;
        xs[(4 * c4 + 2) * XS + p] = val.z;
        xs[(4 * c4 + 3) * XS + p] = val.w;
      }
      __syncthreads();
      for (int c = 0; c < 4 * n4; c++) {
        const float4 xv = *reinterpret_cast<const float4 *>(xs + c * XS + pg * TM);
        const float xa[TM] = {xv.x, xv.y, xv.z, xv.w};
        float cv[TN];
        const float *cr = cst + (c0 + c) * K + cg * TN;
#pragma unroll
        for (int t = 0; t < TN; t += 2) {
          const float2 c2 = *reinterpret_cast<const float2 *>(cr + t);
          cv[t] = c2.x;
          cv[t + 1] = c2.y;
        }
#pragma unroll
        for (int i = 0; i < TM; i++) {
          xn[i] = fmaf(xa[i], xa[i], xn[i]);
#pragma unroll
          for (int t = 0; t < TN; t++) acc[i][t] = fmaf(xa[i], cv[t], acc[i][t]);
        }
      }
    }
#pragma unroll
    for (int i = 0; i < TM; i++) {
      const int p = pg * TM + i;
      // best approximate value, lowest index on equal values, over the 8 lanes
      float a[TN];
      float bv = 1e30f;
      int bj = 0x7fffffff;
#pragma unroll
      for (int t = 0; t < TN; t++) {
        const int j = cg * TN + t;
        a[t] = (xn[i] + cn[j]) - 2.f * acc[i][t];
        if (j < k && a[t] < bv) { bv = a[t]; bj = j; }
      }
#pragma unroll
      for (int o = 1; o < 8; o <<= 1) {
        const float ov = __shfl_xor_sync(0xffffffffu, bv, o);
        const int oj = __shfl_xor_sync(0xffffffffu, bj, o);
        if (ov < bv || (ov == bv && oj < bj)) { bv = ov; bj = oj; }
      }
      const float b1 = bv;
      const float *x = vt + (long)p * d;
      const bool pv = p < np;
      // band members of this lane: direct differences, strict '<' over j
      const float tol = 4.f * (float)(d + 8) * kU * (xn[i] + cmax);
      unsigned band = 0;
      float e1 = INFINITY, e2 = INFINITY;
      int j1 = 0x7fffffff;
      if (pv && b1 < 1e30f) {
#pragma unroll
        for (int t = 0; t < TN; t++) {
          const int j = cg * TN + t;
          if (j < k && !(a[t] > b1 + tol)) band |= 1u << t;
        }
        for (unsigned bm = band; bm; bm &= bm - 1) {
          const int j = cg * TN + __ffs(bm) - 1;
          float sd = 0.f;
          for (int c = 0; c < d; c++) {
            const float tt = (FULL ? xs[c * XS + p] : __ldg(x + c)) - cst[c * K + j];
            sd = fmaf(tt, tt, sd);
          }
          if (sd < e1) { e2 = e1; e1 = sd; j1 = j; } else if (sd < e2) { e2 = sd; }
        }
      }
#pragma unroll
      for (int o = 1; o < 8; o <<= 1) {
        const float oe1 = __shfl_xor_sync(0xffffffffu, e1, o);
        const float oe2 = __shfl_xor_sync(0xffffffffu, e2, o);
        const int oj1 = __shfl_xor_sync(0xffffffffu, j1, o);
        if (oe1 < e1 || (oe1 == e1 && oj1 < j1)) {
          e2 = fminf(oe2, e1);
          e1 = oe1;
          j1 = oj1;
        } else {
          e2 = fminf(e2, oe1);
        }
      }
      int out_j = -1;
      float out_d = 1e30f;
      if (pv && b1 < 1e30f) {
        if (e2 < INFINITY && e2 - e1 <= rho * (e1 + e2)) {
          // near tie: FP64 over the band, sequential over coordinates
          double best = INFINITY;
          int bi = 0x7fffffff;
          for (unsigned bm = band; bm; bm &= bm - 1) {
            const int j = cg * TN + __ffs(bm) - 1;
            double sd = 0;
            for (int c = 0; c < d; c++) {
              const double tt = (double)(FULL ? xs[c * XS + p] : x[c]) - (double)cst[c * K + j];
              sd = add_sq64(sd, tt);
            }
            if (sd < best) { best = sd; bi = j; }
          }
          // only this point's 8 lanes take this branch (together: their
          // conditions come from values they reduced jointly)
          const unsigned gmask = 0xffu << ((threadIdx.x & 31) & ~7);
#pragma unroll
          for (int o = 1; o < 8; o <<= 1) {
            const double ob = __shfl_xor_sync(gmask, best, o);
            const int oi = __shfl_xor_sync(gmask, bi, o);
            if (ob < best || (ob == best && oi < bi)) { best = ob; bi = oi; }
          }
          if (bi != 0x7fffffff) { out_j = bi; out_d = (float)best; }
        } else if (j1 != 0x7fffffff) {
          out_j = j1;
          out_d = e1;
        }
      }
      if (pv && cg == 0) {
        assign[w.p0 + t0 + p] = out_j;
        dis[w.p0 + t0 + p] = out_d;
      }
    }
  }
}

__global__ void hist_kernel(const int *assign, const int *pinst, long n, int k,
                            const unsigned char *active, int *counts) {
  const long p = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const int inst = pinst ? pinst[p] : 0;
  const int a = assign[p];
  if (a < 0 || !active[inst]) return;
  const long g = (long)inst * k + a;
  const unsigned peers = __match_any_sync(__activemask(), g);
  const int leader = __ffs(peers) - 1;
  if ((threadIdx.x & 31) == leader) atomicAdd(counts + g, __popc(peers));
}

__global__ void scan_kernel(const int *counts, long ncl, long *offs, long *cursor) {
  // offs has ncl + 1 entries: offs[ncl] = total
  // one block of 1024: contiguous chunks per thread, then a shuffle scan of
  // the chunk sums (within warps, then over the 32 warp totals)
  __shared__ long wsum[32];
  const int t = threadIdx.x, nt = blockDim.x, lane = t & 31, w = t >> 5;
  const long per = (ncl + nt - 1) / nt;
  const long a = (long)t * per, b = a + per < ncl ? a + per : ncl;
  long s = 0;
  for (long i = a; i < b; i++) s += counts[i];
  long x = s;  // inclusive scan within the warp
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const long y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) wsum[w] = x;
  __syncthreads();
  if (w == 0) {
    long z = lane < (nt >> 5) ? wsum[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const long y = __shfl_up_sync(0xffffffffu, z, o);
      if (lane >= o) z += y;
    }
    wsum[lane] = z;  // inclusive over warps
  }
  __syncthreads();
  long run = x - s + (w > 0 ? wsum[w - 1] : 0);
  for (long i = a; i < b; i++) {
    offs[i] = run;
    cursor[i] = run;
    run += counts[i];
  }
  if (t == nt - 1) offs[ncl] = run;
}

__global__ void scatter_kernel(const int *assign, const int *pinst, long n, int k,
                               const unsigned char *active, long *cursor, long *perm) {
  const long p = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const int inst = pinst ? pinst[p] : 0;
  const int a = assign[p];
  if (a < 0 || !active[inst]) return;
  const long g = (long)inst * k + a;
  const unsigned peers = __match_any_sync(__activemask(), g);
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(peers) - 1;
  long base = 0;
  if (lane == leader) base = atomicAdd((unsigned long long *)(cursor + g),
                                       (unsigned long long)__popc(peers));
  base = __shfl_sync(peers, base, leader);
  perm[base + __popc(peers & ((1u << lane) - 1))] = p;
}

// warps walk contiguous runs of the cluster-sorted point list, accumulating
// exact integer sums in registers and flushing at cluster boundaries
template <int NDR>
__global__ void __launch_bounds__(256)
    segsum_kernel(const long *perm, const long *total, const int *assign, const int *pinst,
                  const float *__restrict__ v, int d, int k, const int *shift,
                  long long *acc) {
  constexpr int RUN = 32, PF = 4;  // points per warp; rows in flight
  const int lane = threadIdx.x & 31;
  const long wglob = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long nsorted = *total;
  const long s0 = wglob * RUN;
  if (s0 >= nsorted) return;
  const int n = (int)(nsorted - s0 < RUN ? nsorted - s0 : RUN);
  const int dbase = blockIdx.y * NDR * 32;
  // lane i holds the row, cluster and shift of the run's i-th point
  long p_l = 0, g_l = -1;
  int sh_l = 0;
  if (lane < n) {
    p_l = perm[s0 + lane];
    const int inst = pinst ? pinst[p_l] : 0;
    g_l = (long)inst * k + assign[p_l];
    sh_l = shift[inst];
  }
  long long part[NDR];
#pragma unroll
  for (int r = 0; r < NDR; r++) part[r] = 0;
  long gcur = -1;
  for (int i0 = 0; i0 < n; i0 += PF) {
    float xv[PF][NDR];
#pragma unroll
    for (int u = 0; u < PF; u++) {
      const int i = i0 + u;  // < RUN + PF: the shuffle index wraps, the value is unused
      const long p = __shfl_sync(0xffffffffu, p_l, i & 31);
#pragma unroll
      for (int r = 0; r < NDR; r++) {
        const int c = dbase + r * 32 + lane;
        xv[u][r] = (i < n && c < d) ? __ldg(v + p * d + c) : 0.f;
      }
    }
#pragma unroll
    for (int u = 0; u < PF; u++) {
      const int i = i0 + u;
      if (i >= n) break;  // uniform over the warp
      const long g = __shfl_sync(0xffffffffu, g_l, i);
      const int sh = __shfl_sync(0xffffffffu, sh_l, i);
      if (g != gcur) {
        if (gcur >= 0) {
#pragma unroll
          for (int r = 0; r < NDR; r++) {
            const int c = dbase + r * 32 + lane;
            if (c < d && part[r])
              atomicAdd((unsigned long long *)(acc + gcur * d + c), (unsigned long long)part[r]);
            part[r] = 0;
          }
        }
        gcur = g;
      }
#pragma unroll
      for (int r = 0; r < NDR; r++) {
        const int c = dbase + r * 32 + lane;
        if (c < d) part[r] += fixed_of(xv[u][r], sh);
      }
    }
  }
  if (gcur >= 0) {
#pragma unroll
    for (int r = 0; r < NDR; r++) {
      const int c = dbase + r * 32 + lane;
      if (c < d && part[r])
        atomicAdd((unsigned long long *)(acc + gcur * d + c), (unsigned long long)part[r]);
    }
  }
}

__global__ void finalize_kernel(const long long *acc, const int *counts, long ncl, int d,
                                int k, const int *shift, const unsigned char *active,
                                float *C, int *counts_out, const int *err, int *err_out) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0 && err_out) *err_out = *err;
  if (i >= ncl * d) return;
  const long g = i / d;
  if (counts_out && i == g * d) counts_out[g] = counts[g];
  const int inst = (int)(g / k);
  if (!active[inst]) return;
  const double inv = ldexp(1.0, -shift[inst]);
  const double r = 1.0 / (double)counts[g];
  C[i] = __double2float_rn(__ll2double_rn(acc[i]) * inv * r);
}

__global__ void normalize_kernel(float *C, long ncl, int d, int k, const unsigned char *active) {
  const long g = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= ncl || !active[g / k]) return;
  float *row = C + g * d;
  double s = 0;
  for (int c = 0; c < d; c++) s += (double)(row[c] * row[c]);
  const double inv = 1. / sqrt(s);
  for (int c = 0; c < d; c++) row[c] = (float)((double)row[c] * inv);
}

// L1 normalisation of the centroids (yael/vector.c:2016-2026, 2180-2191)
__global__ void normalize_l1_kernel(float *C, long ncl, int d) {
  const long g = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= ncl) return;
  float *row = C + g * d;
  double s = 0;
  for (int c = 0; c < d; c++) s += (double)fabsf(row[c]);
  const double inv = 1. / s;
  for (int c = 0; c < d; c++) row[c] = (float)((double)row[c] * inv);
}

// ---- L1 / chi2 centroids (yael/kmeans.c:253-275) ------------------------
// perm: point indices sorted by cluster, increasing within a cluster; offs:
// the cluster segments; tmp: n x d scratch, the values of one coordinate
// contiguous (the reference's tmp_v layout).

// in place: a[kth] becomes the kth smallest (0-based), a[0..kth) <= a[kth] <=
// a[kth+1..n) (Hoare partitions around a middle pivot; each round shrinks the
// range, so it ends)
__device__ void select_kth(float *a, int n, int kth) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const float p = a[(lo + hi) >> 1];
    int i = lo, j = hi;
    while (i <= j) {
      while (a[i] < p) i++;
      while (a[j] > p) j--;
      if (i <= j) {
        const float t = a[i];
        a[i] = a[j];
        a[j] = t;
        i++;
        j--;
      }
    }
    if (kth <= j) hi = j;
    else if (kth >= i) lo = i;
    else break;
  }
}

// the median of each cluster's values per coordinate (yael/sorting.c:676-703):
// the (m/2)-th smallest for odd m, half the float sum of the two middle values
// for even m; NaN for an empty cluster
__global__ void median_kernel(const int *perm, const int *offs, const float *v, int d, int k,
                              long n, float *tmp, float *C) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)k * d) return;
  const int c = (int)(t / d), j = (int)(t - (long)c * d);
  const int o0 = offs[c], m = offs[c + 1] - o0;
  float out;
  if (m == 0) {
    out = __int_as_float(0x7fc00000);
  } else if (m == 1) {
    out = v[(long)perm[o0] * d + j];
  } else {
    float *seg = tmp + (long)j * n + o0;
    for (int e = 0; e < m; e++) seg[e] = v[(long)perm[o0 + e] * d + j];
    const int half = m / 2;
    select_kth(seg, m, half);
    const float upper = seg[half];
    if (m & 1) {
      out = upper;
    } else {
      float lower = seg[0];
      for (int e = 1; e < half; e++) lower = seg[e] > lower ? seg[e] : lower;
      out = (float)(0.5 * (double)__fadd_rn(upper, lower));
    }
  }
  C[t] = out;
}

// the minimiser of sum_i (x - a_i)^2 / (x + a_i) over x >= 0 (Newton steps,
// yael/kmeans.c:95-158), the cluster's values taken in decreasing point order
// as the reference's scratch holds them; float arithmetic, unfused
__global__ void chi2_kernel(const int *perm, const int *offs, const float *v, int d, int k, long n,
                            float *tmp, float *C) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)k * d) return;
  const int c = (int)(t / d), j = (int)(t - (long)c * d);
  const int o0 = offs[c], m = offs[c + 1] - o0;
  float x;
  if (m == 0) {
    x = __int_as_float(0x7fc00000);
  } else if (m == 1) {
    x = v[(long)perm[o0] * d + j];
  } else {
    float *a = tmp + (long)j * n + o0;
    for (int e = 0; e < m; e++) a[e] = v[(long)perm[o0 + m - 1 - e] * d + j];
    float mag = 0.f;
    for (int e = 0; e < m; e++) mag = __fadd_rn(mag, a[e]);
    mag = __fdiv_rn(mag, (float)m);
    x = 0.f;
    float prev = 0.f;
    int niter = 0;
    for (;;) {
      float dv = 0.f, ddv = 0.f;
      for (int e = 0; e < m; e++) {
        const float s1 = __fadd_rn(x, a[e]);
        const float s2 = __fmul_rn(s1, s1);
        const float s3 = __fmul_rn(s1, s2);
        if (s2 == 0.f) continue;
        dv = __fadd_rn(dv, __fdiv_rn(__fmul_rn(__fsub_rn(x, a[e]), __fadd_rn(x, __fmul_rn(3.f, a[e]))),
                                     s2));
        ddv = __fadd_rn(ddv, __fdiv_rn(__fmul_rn(__fmul_rn(8.f, a[e]), a[e]), s3));
      }
      if (dv == 0.f) break;
      prev = x;
      x = __fsub_rn(x, __fdiv_rn(dv, ddv));
      if (x < 0.f) x = (float)((double)prev / 2.0);
      if (++niter == 1000) break;
      if (!(fabs((double)__fsub_rn(x, prev)) > 1e-4 * (double)mag)) break;
    }
  }
  C[t] = x;
}

__global__ void cluster_keys_kernel(const int *assign, long n, int *keys, int *vals) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  keys[i] = assign[i] < 0 ? INT_MAX : assign[i];
  vals[i] = (int)i;
}

__global__ void cluster_offsets_kernel(const int *sorted, long n, int k, int *offs) {
  const long g = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g > k) return;
  long lo = 0, hi = n;
  while (lo < hi) {
    const long mid = (lo + hi) / 2;
    if (sorted[mid] < g) lo = mid + 1; else hi = mid;
  }
  offs[g] = (int)lo;
}

// Per (slice, group of 32 columns): the column sums in FP32 (rows taken in
// a fixed order: deterministic), minima and maxima.  Block (32, 8).
__global__ void slice_stats_kernel(const KmSlice *sl, const float *v, int d, float *psum,
                                   float *pmin, float *pmax) {
  const KmSlice s = sl[blockIdx.x];
  const int c = blockIdx.y * 32 + threadIdx.x;
  float a = 0.f, lo = INFINITY, hi = -INFINITY;
  if (c < d)
    for (int i = threadIdx.y; i < s.n; i += 8) {
      const float x = v[(s.p0 + i) * d + c];
      a += x;
      lo = fminf(lo, x);
      hi = fmaxf(hi, x);
    }
  __shared__ float sa[8][32], sl_[8][32], sh[8][32];
  sa[threadIdx.y][threadIdx.x] = a;
  sl_[threadIdx.y][threadIdx.x] = lo;
  sh[threadIdx.y][threadIdx.x] = hi;
  __syncthreads();
  if (threadIdx.y == 0 && c < d) {
    for (int y = 1; y < 8; y++) {
      a += sa[y][threadIdx.x];
      lo = fminf(lo, sl_[y][threadIdx.x]);
      hi = fmaxf(hi, sh[y][threadIdx.x]);
    }
    const long o = (long)blockIdx.x * d + c;
    psum[o] = a;
    pmin[o] = lo;
    pmax[o] = hi;
  }
}

// Per instance (its slices first[i] .. + count[i] - 1, npts[i] points): the
// mean mu (FP32 sums in slice order), amax = max |v| and cmax >= max |fl(v -
// mu)| (the column extremes' distances to mu, rounded up).
__global__ void inst_stats_kernel(const int *first, const int *count, const long *npts,
                                  const float *psum, const float *pmin, const float *pmax,
                                  int d, float *mu, float *amax, float *cmax) {
  const int i = blockIdx.x;
  float am = 0.f, cm = 0.f;
  for (int c = threadIdx.x; c < d; c += blockDim.x) {
    float a = 0.f, lo = INFINITY, hi = -INFINITY;
    for (int s = 0; s < count[i]; s++) {
      const long o = (long)(first[i] + s) * d + c;
      a += psum[o];
      lo = fminf(lo, pmin[o]);
      hi = fmaxf(hi, pmax[o]);
    }
    const float m = npts[i] > 0 ? a / (float)npts[i] : 0.f;
    mu[(long)i * d + c] = m;
    if (lo <= hi) {  // a column of NaNs alone leaves both as they are
      am = fmaxf(am, fmaxf(fabsf(lo), fabsf(hi)));
      cm = fmaxf(cm, fmaxf(__fsub_ru(hi, m), __fsub_ru(m, lo)));
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    am = fmaxf(am, __shfl_xor_sync(0xffffffffu, am, o));
    cm = fmaxf(cm, __shfl_xor_sync(0xffffffffu, cm, o));
  }
  __shared__ float wa[8], wc[8];
  if ((threadIdx.x & 31) == 0) {
    wa[threadIdx.x >> 5] = am;
    wc[threadIdx.x >> 5] = cm;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); w++) {
      am = fmaxf(am, wa[w]);
      cm = fmaxf(cm, wc[w]);
    }
    amax[i] = am;
    cmax[i] = cm;
  }
}

__global__ void slice_sum_kernel(const KmSlice *sl, const float *dis, double *out) {
  const KmSlice s = sl[blockIdx.x];
  __shared__ double red[256];
  double acc = 0;
  for (int i = threadIdx.x; i < s.n; i += blockDim.x) acc += (double)dis[s.p0 + i];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = red[0];
}

__global__ void gather_kernel(const float *v, int d, const long *rows, long nrows, float *C) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nrows * d) return;
  const long r = i / d;
  C[i] = v[rows[r] * d + (i - r * d)];
}

// the same for rows of d4 float4 (16-byte aligned rows): a warp per row
// step, lanes over the row's float4
__global__ void gather4_kernel(const float4 *v, int d4, const long *rows, long nrows, float4 *C) {
  const long w = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const long nw = ((long)gridDim.x * blockDim.x) >> 5;
  for (long r = w; r < nrows; r += nw) {
    const float4 *src = v + rows[r] * d4;
    float4 *dst = C + r * d4;
    for (int c = lane; c < d4; c += 32) dst[c] = __ldg(src + c);
  }
}

template <int K, bool VEC>
int launch_assign(const KmWork *work, int nwork, const float *v, int d, const float *C, int k,
                  const unsigned char *active, int *assign, float *dis, cudaStream_t st) {
  const size_t smem = (size_t)((((long)k * d + 3) & ~3L) + k) * sizeof(float);
  YG_CHECK(ensure_smem((const void *)assign_small_kernel<K, VEC>, smem));
  assign_small_kernel<K, VEC><<<nwork, 256, smem, st>>>(work, v, d, C, k, active, assign, dis);
  YG_LAUNCH_CHECK();
  return OK;
}

// The variant of the grouped assignment is tuned per shape (autotune.cuh):
// 0 the GEMM form with whole rows staged (d <= kFullD), 1 the GEMM form over
// 32-coordinate slices, 2 one point per thread.  A trial is timed with events
// around its launch and reported after the caller's next synchronisation.
thread_local int t_trial = -1;
thread_local cudaEvent_t t_trial_ev[2] = {nullptr, nullptr};
thread_local bool t_settled = true;

template <int K>
int launch_assign_any(const KmWork *work, int nwork, const float *v, int d, const float *C,
                      int k, const unsigned char *active, int *assign, float *dis,
                      cudaStream_t st) {
  // float4 rows need d % 4 == 0 and 16-byte aligned points and centroids
  const bool vec = (d % 4 == 0) && ((reinterpret_cast<uintptr_t>(v) & 15) == 0) &&
                   ((reinterpret_cast<uintptr_t>(C) & 15) == 0);
  const bool gemm = vec && (size_t)d * K * 4 <= 120 * 1024;
  int var[3], nv = 0;
  if (gemm && d <= kFullD) var[nv++] = 0;
  if (gemm) var[nv++] = 1;
  var[nv++] = 2;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  YG_CUDA(cudaStreamIsCapturing(st, &cs));
  int ticket = -1;
  const int pick = tune_variant(TuneKey{3, 0, d, K, vec ? 1 : 0}, nv,
                                cs == cudaStreamCaptureStatusNone && t_trial < 0, &ticket,
                                &t_settled);
  if (ticket >= 0) {
    for (auto &e : t_trial_ev)
      if (!e) YG_CUDA(cudaEventCreate(&e));
    YG_CUDA(cudaEventRecord(t_trial_ev[0], st));
  }
  switch (var[pick < nv ? pick : 0]) {
    case 0: {
      const size_t smem = ((size_t)d * K + K + (size_t)d * 132) * sizeof(float);
      YG_CHECK(ensure_smem((const void *)assign_gemm_kernel<K, true>, smem));
      assign_gemm_kernel<K, true><<<nwork, 256, smem, st>>>(work, v, d, C, k, active, assign,
                                                            dis);
      YG_LAUNCH_CHECK();
      break;
    }
    case 1: {
      const size_t smem = ((size_t)d * K + K + 32 * 132) * sizeof(float);
      YG_CHECK(ensure_smem((const void *)assign_gemm_kernel<K, false>, smem));
      assign_gemm_kernel<K, false><<<nwork, 256, smem, st>>>(work, v, d, C, k, active, assign,
                                                             dis);
      YG_LAUNCH_CHECK();
      break;
    }
    default:
      if (vec) YG_CHECK((launch_assign<K, true>(work, nwork, v, d, C, k, active, assign, dis, st)));
      else YG_CHECK((launch_assign<K, false>(work, nwork, v, d, C, k, active, assign, dis, st)));
  }
  if (ticket >= 0) {
    YG_CUDA(cudaEventRecord(t_trial_ev[1], st));
    t_trial = ticket;
  }
  return OK;
}

}  // namespace

int km_assign_small(const KmWork *work, int nwork, const float *v, int d, const float *C,
                    int k, const unsigned char *active, int *assign, float *dis,
                    cudaStream_t st) {
  if (nwork <= 0) return OK;
  if ((size_t)k * d * 4 + (size_t)k * 4 + 16 > 200 * 1024) {
    set_error(E_UNSUPPORTED, "grouped assignment: k*d=%ld too large for shared memory",
              (long)k * d);
    return E_UNSUPPORTED;
  }
  if (k <= 16) return launch_assign_any<16>(work, nwork, v, d, C, k, active, assign, dis, st);
  if (k <= 32) return launch_assign_any<32>(work, nwork, v, d, C, k, active, assign, dis, st);
  if (k <= 64) return launch_assign_any<64>(work, nwork, v, d, C, k, active, assign, dis, st);
  set_error(E_ARG, "grouped assignment: k=%d > %d", k, kSmallK);
  return E_ARG;
}

size_t km_alt_sort_bytes(long n) {
  size_t tb = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, tb, (const int *)nullptr, (int *)nullptr,
                                  (const int *)nullptr, (int *)nullptr, (int)n, 0, 32);
  return tb;
}

int km_alt_update(const int *assign, long n, const float *v, int d, int k, bool l1, int *keys,
                  int *keys2, int *vals, int *vals2, int *offs, float *tmp, void *sort_tmp,
                  size_t sort_bytes, float *C, cudaStream_t st) {
  if (n > INT_MAX) {
    set_error(E_UNSUPPORTED, "L1 / chi2 k-means: %ld points", n);
    return E_UNSUPPORTED;
  }
  cluster_keys_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, st>>>(assign, n, keys, vals);
  YG_LAUNCH_CHECK();
  size_t tb = sort_bytes;
  YG_CUDA(cub::DeviceRadixSort::SortPairs(sort_tmp, tb, keys, keys2, vals, vals2, (int)n, 0, 32,
                                          st));
  cluster_offsets_kernel<<<(unsigned)ceil_div((long)k + 1, 256), 256, 0, st>>>(keys2, n, k, offs);
  YG_LAUNCH_CHECK();
  const unsigned g = (unsigned)ceil_div((long)k * d, 128);
  if (l1) median_kernel<<<g, 128, 0, st>>>(vals2, offs, v, d, k, n, tmp, C);
  else chi2_kernel<<<g, 128, 0, st>>>(vals2, offs, v, d, k, n, tmp, C);
  YG_LAUNCH_CHECK();
  return OK;
}

int km_normalize_l1(float *C, long ncl, int d, cudaStream_t st) {
  normalize_l1_kernel<<<(unsigned)ceil_div(ncl, 128), 128, 0, st>>>(C, ncl, d);
  YG_LAUNCH_CHECK();
  return OK;
}

bool km_assign_tune_collect() {
  if (t_trial < 0) return t_settled;
  float ms = 0.f;
  if (cudaEventElapsedTime(&ms, t_trial_ev[0], t_trial_ev[1]) != cudaSuccess) {
    (void)cudaGetLastError();
    ms = 0.f;
  }
  tune_report(t_trial, ms);
  t_trial = -1;
  return false;  // the next call may still be a trial
}

int km_histogram(const int *assign, const int *pinst, long n, int k,
                 const unsigned char *active, int *counts, cudaStream_t st) {
  if (n <= 0) return OK;
  hist_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, st>>>(assign, pinst, n, k, active, counts);
  YG_LAUNCH_CHECK();
  return OK;
}

int km_scan(const int *counts, long ncl, long *offs, long *cursor, cudaStream_t st) {
  scan_kernel<<<1, 1024, 0, st>>>(counts, ncl, offs, cursor);
  YG_LAUNCH_CHECK();
  return OK;
}

int km_scatter(const int *assign, const int *pinst, long n, int k,
               const unsigned char *active, long *cursor, long *perm, cudaStream_t st) {
  if (n <= 0) return OK;
  scatter_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, st>>>(assign, pinst, n, k, active,
                                                             cursor, perm);
  YG_LAUNCH_CHECK();
  return OK;
}

int km_update(const long *perm, const long *total, long nmax, const int *assign,
              const int *pinst, const int *counts, const float *v, int d, long ncl, int k,
              const int *shift, const unsigned char *active, long long *acc, float *C,
              cudaStream_t st) {
  YG_CUDA(cudaMemsetAsync(acc, 0, sizeof(long long) * ncl * d, st));
  if (nmax > 0) {
    const long warps = ceil_div(nmax, 32);
    const int nd = d <= 32 ? 1 : d <= 64 ? 2 : d <= 128 ? 4 : 8;
    dim3 grid((unsigned)ceil_div(warps * 32, 256), (unsigned)ceil_div(d, nd * 32));
    switch (nd) {
      case 1: segsum_kernel<1><<<grid, 256, 0, st>>>(perm, total, assign, pinst, v, d, k, shift, acc); break;
      case 2: segsum_kernel<2><<<grid, 256, 0, st>>>(perm, total, assign, pinst, v, d, k, shift, acc); break;
      case 4: segsum_kernel<4><<<grid, 256, 0, st>>>(perm, total, assign, pinst, v, d, k, shift, acc); break;
      default: segsum_kernel<8><<<grid, 256, 0, st>>>(perm, total, assign, pinst, v, d, k, shift, acc); break;
    }
    YG_LAUNCH_CHECK();
  }
  finalize_kernel<<<(unsigned)ceil_div(ncl * d, 256), 256, 0, st>>>(
      acc, counts, ncl, d, k, shift, active, C, nullptr, nullptr, nullptr);
  YG_LAUNCH_CHECK();
  return OK;
}

// a warp per point: FP32 direct differences to centroid assign[p] (any
// summation order), widened by their rounding bound (d + 4) 2^-24 relative,
// so that the result is >= the exact distance; +inf without a centroid
__global__ void prior_bound_kernel(const float *__restrict__ v, int d, long n,
                                   const int *__restrict__ assign, const float *__restrict__ C,
                                   float *kth) {
  const long p = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (p >= n) return;
  const int j = assign[p];
  if (j < 0) {
    if (lane == 0) kth[p] = INFINITY;
    return;
  }
  const float *x = v + p * d, *c = C + (long)j * d;
  float s = 0.f;
  for (int i = lane; i < d; i += 32) {
    const float t = __ldg(x + i) - __ldg(c + i);
    s = fmaf(t, t, s);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) {
    const float w = (float)(d + 4) * 5.9604645e-08f * 1.01f;
    kth[p] = isfinite(s) ? __fmul_ru(s, 1.f + w) + 1e-30f : INFINITY;
  }
}

int km_prior_bound(const float *v, int d, long n, const int *assign, const float *C, float *kth,
                   cudaStream_t st) {
  if (n <= 0) return OK;
  prior_bound_kernel<<<(unsigned)ceil_div(n * 32, 256), 256, 0, st>>>(v, d, n, assign, C, kth);
  YG_LAUNCH_CHECK();
  return OK;
}

int km_finalize(const long long *acc, const int *counts, long ncl, int d, int k,
                const int *shift, const unsigned char *active, float *C, cudaStream_t st,
                int *counts_out, const int *err, int *err_out) {
  finalize_kernel<<<(unsigned)ceil_div(ncl * d, 256), 256, 0, st>>>(
      acc, counts, ncl, d, k, shift, active, C, counts_out, err, err_out);
  YG_LAUNCH_CHECK();
  return OK;
}

int km_normalize(float *C, long ncl, int d, int k, const unsigned char *active,
                 cudaStream_t st) {
  normalize_kernel<<<(unsigned)ceil_div(ncl, 128), 128, 0, st>>>(C, ncl, d, k, active);
  YG_LAUNCH_CHECK();
  return OK;
}

// ---- stable grouping of points by a small key (hkm: by node) ----------------

// cnt[c * k + b] = points of chunk c with key b
__global__ void group_count_kernel(const int *key, long n, int k, long chunk, int *cnt) {
  const long c = blockIdx.x;
  const long i0 = c * chunk, i1 = min(n, i0 + chunk);
  int *row = cnt + c * (long)k;
  for (long i = i0 + threadIdx.x; i < i1; i += blockDim.x) atomicAdd(row + key[i], 1);
}

// per key b (a warp each, 32 chunks per step): cnt[c * k + b] := the points
// of chunks before c with key b; tot[b] = all of them
__global__ void group_prefix_kernel(int *cnt, long nchunk, int k, long *tot) {
  const long b = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (b >= k) return;
  long base = 0;
  for (long c0 = 0; c0 < nchunk; c0 += 32) {
    const long c = c0 + lane;
    const int x = c < nchunk ? cnt[c * k + b] : 0;
    int incl = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    if (c < nchunk) cnt[c * k + b] = (int)(base + incl - x);
    base += __shfl_sync(0xffffffffu, incl, 31);
  }
  if (lane == 0) tot[b] = base;
}

// start[b] = sum of tot[b'] for b' < b (start[k] = n), one thread
__global__ void group_start_kernel(const long *tot, int k, long *start) {
  long a = 0;
  for (int b = 0; b < k; b++) {
    start[b] = a;
    a += tot[b];
  }
  start[k] = a;
}

// one warp per chunk, 32 points at a time in index order: a point's place is
// its key's start, the points of that key in earlier chunks, those already
// placed from this chunk and those of earlier lanes (stable)
__global__ void group_scatter_kernel(const int *key, long n, int k, long chunk, int *cnt,
                                     const long *start, long *perm) {
  const long c = blockIdx.x;
  const int lane = threadIdx.x;
  const long i0 = c * chunk, i1 = min(n, i0 + chunk);
  int *row = cnt + c * (long)k;
  for (long g = i0; g < i1; g += 32) {
    const long i = g + lane;
    const bool v = i < i1;
    const int b = v ? key[i] : -1 - lane;  // distinct dummies for the lanes past the end
    const unsigned same = __match_any_sync(0xffffffffu, b);
    const int rank = __popc(same & ((1u << lane) - 1u));
    if (v) perm[start[b] + row[b] + rank] = i;
    __syncwarp();
    if (v && rank == 0) row[b] += __popc(same);
    __syncwarp();
  }
}

// pinst[j] = key[perm[j]]
__global__ void group_key_of_kernel(const int *key, const long *perm, long n, int *out) {
  const long j = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (j < n) out[j] = key[perm[j]];
}

int km_group_by_key(const int *key, long n, int k, long *perm, long *start, int *key_of,
                    Workspace &ws, int slot_cnt, int slot_tot, cudaStream_t st) {
  if (n <= 0) return OK;
  long chunk = 2048;
  while ((double)ceil_div(n, chunk) * k > 16e6) chunk *= 2;
  const long nchunk = ceil_div(n, chunk);
  int *cnt;
  long *tot;
  YG_CHECK(ws.get(slot_cnt, sizeof(int) * (size_t)nchunk * k, reinterpret_cast<void **>(&cnt)));
  YG_CHECK(ws.get(slot_tot, sizeof(long) * (size_t)k, reinterpret_cast<void **>(&tot)));
  YG_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int) * (size_t)nchunk * k, st));
  group_count_kernel<<<(unsigned)nchunk, 256, 0, st>>>(key, n, k, chunk, cnt);
  YG_LAUNCH_CHECK();
  group_prefix_kernel<<<(unsigned)ceil_div((long)k * 32, 256), 256, 0, st>>>(cnt, nchunk, k, tot);
  YG_LAUNCH_CHECK();
  group_start_kernel<<<1, 1, 0, st>>>(tot, k, start);
  YG_LAUNCH_CHECK();
  group_scatter_kernel<<<(unsigned)nchunk, 32, 0, st>>>(key, n, k, chunk, cnt, start, perm);
  YG_LAUNCH_CHECK();
  if (key_of) {
    group_key_of_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, st>>>(key, perm, n, key_of);
    YG_LAUNCH_CHECK();
  }
  return OK;
}

int km_inst_stats(const KmSlice *sl, int nsl, const float *v, int d, int ninst,
                  const int *first, const int *count, const long *npts, float *part, float *mu,
                  float *amax, float *cmax, cudaStream_t st) {
  if (nsl <= 0 || ninst <= 0) return OK;
  float *psum = part, *pmin = part + (size_t)nsl * d, *pmax = part + 2 * (size_t)nsl * d;
  slice_stats_kernel<<<dim3((unsigned)nsl, (unsigned)ceil_div(d, 32)), dim3(32, 8), 0, st>>>(
      sl, v, d, psum, pmin, pmax);
  YG_LAUNCH_CHECK();
  inst_stats_kernel<<<ninst, 128, 0, st>>>(first, count, npts, psum, pmin, pmax, d, mu, amax,
                                           cmax);
  YG_LAUNCH_CHECK();
  return OK;
}

int km_slice_sums(const KmSlice *sl, int nsl, const float *dis, double *out, cudaStream_t st) {
  if (nsl <= 0) return OK;
  slice_sum_kernel<<<nsl, 256, 0, st>>>(sl, dis, out);
  YG_LAUNCH_CHECK();
  return OK;
}

int km_gather(const float *v, int d, const long *rows, long nrows, float *C, cudaStream_t st) {
  if (nrows <= 0) return OK;
  if (d % 4 == 0 && (reinterpret_cast<uintptr_t>(v) & 15) == 0 &&
      (reinterpret_cast<uintptr_t>(C) & 15) == 0) {
    int dev = 0, sms = 0;
    YG_CUDA(cudaGetDevice(&dev));
    YG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const long blocks = std::min<long>(ceil_div(nrows, 8), (long)sms * 16);
    gather4_kernel<<<(unsigned)blocks, 256, 0, st>>>(reinterpret_cast<const float4 *>(v), d / 4,
                                                    rows, nrows, reinterpret_cast<float4 *>(C));
  } else {
    gather_kernel<<<(unsigned)ceil_div(nrows * d, 256), 256, 0, st>>>(v, d, rows, nrows, C);
  }
  YG_LAUNCH_CHECK();
  return OK;
}

}  // namespace yg
