// Full cross-distance matrices (yael/nn.c:92-162, 266-356, 777-860) and the
// short-list re-ranking entry points (yael/nn.c:528-600).
#include <math.h>
#include <string.h>

#include <algorithm>

#include "alt.cuh"
#include "knn.cuh"
#include "simt_tile.cuh"
#include "../../include/yael_gpu.h"

namespace yg {

namespace {
using namespace simt;

// dist2[i + ldd*j] for a 128 (a rows) x 128 (b rows) tile; the tile is staged in
// shared memory and written with consecutive threads on consecutive i.
__global__ void __launch_bounds__(NT, 1)
    cross_kernel(const float *__restrict__ A, long lda, int na, const float *__restrict__ B,
                 long ldb, int nb, int d, const float *__restrict__ an,
                 const double *__restrict__ bn, int metric, float *out, long ldd, int jt0) {
  extern __shared__ __align__(16) float smem[];
  float *St = smem + kOperandFloats;
  const long i0 = (long)blockIdx.x * BM;
  const long j0 = (long)(blockIdx.y + jt0) * BN;
  float acc[8][8];
  tile_mainloop(A, lda, na, i0, B, ldb, nb, j0, d, smem, acc);
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
#pragma unroll
  for (int j = 0; j < 8; j++) {
    const int col = col_of(j, tx);
    const long jg = j0 + col;
    const double bj = (metric == METRIC_L2 && jg < nb) ? bn[jg] : 0.0;
#pragma unroll
    for (int i = 0; i < 8; i++) {
      const int row = row_of(i, ty);
      const long ig = i0 + row;
      float v = acc[i][j];
      if (metric == METRIC_L2) {
        // norms summed in double and rounded, then the -2 a.b term (nn.c:116-126)
        const float base = (ig < na && jg < nb) ? (float)(bj + (double)an[ig]) : 0.f;
        v = fmaf(-2.f, v, base);
      }
      St[row * ST_LD + col] = v;
    }
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < BM * BN; idx += NT) {
    const int col = idx >> 7, row = idx & (BM - 1);
    const long ig = i0 + row, jg = j0 + col;
    if (ig < na && jg < nb) out[jg * ldd + ig] = St[row * ST_LD + col];
  }
}

__global__ void norms_kernel(const float *x, long ld, int n, int d, float *n32, double *n64) {
  const int lane = threadIdx.x & 31;
  const long r = (long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (r >= n) return;
  double s = 0;
  for (int c = lane; c < d; c += 32) {
    const float v = x[r * ld + c];
    s += (double)(v * v);
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) {
    if (n32) n32[r] = (float)s;
    if (n64) n64[r] = s;
  }
}

template <typename T>
int ws_get(Workspace &ws, int slot, size_t count, T **p) {
  void *v = nullptr;
  YG_CHECK(ws.get(slot, count * sizeof(T), &v));
  *p = reinterpret_cast<T *>(v);
  return OK;
}

// host arrays in, host matrix out (pitch ldd), chunked over b so the device
// output stays below 1 GiB
int cross_host(int metric, int d, int na, int nb, const float *a, int lda, const float *b,
               int ldb, float *dist2, int ldd) {
  if (na <= 0 || nb <= 0) return OK;
  if (d < 0 || lda < d || ldb < d || ldd < na) {
    set_error(E_ARG, "cross distances: bad leading dimensions");
    return E_ARG;
  }
  Ctx *ctx;
  YG_CHECK(ctx_get(&ctx));
  cudaStream_t st = ctx->stream;
  Workspace &ws = ctx->ws;
  float *da, *db, *dout, *an;
  double *bn;
  YG_CHECK(ws_get(ws, WS_H_Q, (size_t)na * d + 1, &da));
  YG_CHECK(ws_get(ws, WS_H_B, (size_t)nb * d + 1, &db));
  YG_CHECK(ws_get(ws, WS_QN64, (size_t)nb, &bn));
  YG_CHECK(ws_get(ws, WS_BN32, (size_t)na, &an));
  if (d > 0) {
    YG_CUDA(cudaMemcpy2DAsync(da, sizeof(float) * d, a, sizeof(float) * lda, sizeof(float) * d,
                              na, cudaMemcpyHostToDevice, st));
    YG_CUDA(cudaMemcpy2DAsync(db, sizeof(float) * d, b, sizeof(float) * ldb, sizeof(float) * d,
                              nb, cudaMemcpyHostToDevice, st));
  }
  if (metric == METRIC_L2 && d > 0) {
    norms_kernel<<<(unsigned)ceil_div(na, 8), 256, 0, st>>>(da, d, na, d, an, nullptr);
    YG_LAUNCH_CHECK();
    norms_kernel<<<(unsigned)ceil_div(nb, 8), 256, 0, st>>>(db, d, nb, d, nullptr, bn);
    YG_LAUNCH_CHECK();
  } else if (metric == METRIC_L2) {
    YG_CUDA(cudaMemsetAsync(an, 0, sizeof(float) * na, st));
    YG_CUDA(cudaMemsetAsync(bn, 0, sizeof(double) * nb, st));
  }
  const size_t smem = sizeof(float) * (kOperandFloats + BM * ST_LD);
  YG_CHECK(ensure_smem((const void *)cross_kernel, smem));
  long jb = (long)(((size_t)1 << 30) / ((size_t)na * 4));
  jb = (jb / BN) * BN;
  if (jb < BN) jb = BN;
  YG_CHECK(ws_get(ws, WS_H_DIS, (size_t)na * (size_t)imin(nb, (int)jb), &dout));
  for (long j0 = 0; j0 < nb; j0 += jb) {
    const int nbc = (int)(nb - j0 < jb ? nb - j0 : jb);
    const int ntj = (int)ceil_div(nbc, BN);
    for (int t0 = 0; t0 < ntj; t0 += 65535) {
      dim3 grid((unsigned)ceil_div(na, BM), (unsigned)imin(65535, ntj - t0));
      cross_kernel<<<grid, NT, smem, st>>>(da, d, na, db + j0 * d, d, nbc, d, an, bn + j0,
                                           metric, dout, na, t0);
      YG_LAUNCH_CHECK();
    }
    YG_CUDA(cudaMemcpy2DAsync(dist2 + j0 * ldd, sizeof(float) * ldd, dout, sizeof(float) * na,
                              sizeof(float) * na, nbc, cudaMemcpyDeviceToHost, st));
  }
  YG_CUDA(cudaStreamSynchronize(st));
  return OK;
}

// ---- short-list re-ranking (nn.c:528-580): FP64 exact distances, stable
// ordering by (distance, list position)
__global__ void reorder_kernel(int nq, int nb, int d, int k, const float *b, const float *v,
                               int *idx, float *dis) {
  extern __shared__ __align__(16) unsigned char sm[];
  double *key = reinterpret_cast<double *>(sm);
  int *pos = reinterpret_cast<int *>(key + k);
  int *ids = pos + k;
  __shared__ int ski;
  const int q = blockIdx.x;
  int *ia = idx + (long)q * k;
  if (threadIdx.x == 0) {
    int j = 0;
    while (j < k && ia[j] >= 0) j++;
    ski = j;
  }
  __syncthreads();
  const int ki = ski;
  for (int i = threadIdx.x; i < ki; i += blockDim.x) {
    if (ia[i] >= nb) {  // ids must index the base (the reference reads b[id*d])
      key[i] = INFINITY;
      pos[i] = i;
      ids[i] = ia[i];
      continue;
    }
    const float *bv = b + (long)ia[i] * d;
    const float *qv = v + (long)q * d;
    double s = 0;
    for (int c = 0; c < d; c++) {
      const double t = (double)qv[c] - (double)bv[c];
      s = add_sq64(s, t);
    }
    key[i] = s;
    pos[i] = i;
    ids[i] = ia[i];
  }
  __syncthreads();
  // rank sort: position of element i = #{j : (key_j, j) < (key_i, i)}
  for (int i = threadIdx.x; i < ki; i += blockDim.x) {
    int r = 0;
    for (int j = 0; j < ki; j++) r += (key[j] < key[i]) || (key[j] == key[i] && j < i);
    ia[r] = ids[i];
    dis[(long)q * k + r] = (float)key[i];
  }
}

__global__ void recompute_kernel(int nq, int nb, int d, int k, const float *b,
                                 const float *v, int label0, int *kp, const int *idx,
                                 float *dis, int *bad) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq) return;
  int i = kp[q];
  for (; i < k; i++) {
    const long j = (long)idx[(long)q * k + i] - label0;
    if (j < 0) { atomicExch(bad, 1); break; }
    if (j >= nb) break;
    double s = 0;
    for (int c = 0; c < d; c++) {
      const double t = (double)v[(long)q * d + c] - (double)b[j * d + c];
      s = add_sq64(s, t);
    }
    dis[(long)q * k + i] = (float)s;
  }
  kp[q] = i;
}

}  // namespace

int cross_distances_host(int metric, int d, int na, int nb, const float *a, int lda,
                         const float *b, int ldb, float *dist2, int ldd) {
  return cross_host(metric, d, na, nb, a, lda, b, ldb, dist2, ldd);
}

static int reorder_host(int n, int nb, int d, int k, const float *b, const float *v, int *idx,
                        float *dis) {
  if (n <= 0 || k <= 0) return OK;
  Ctx *ctx;
  YG_CHECK(ctx_get(&ctx));
  cudaStream_t st = ctx->stream;
  Workspace &ws = ctx->ws;
  float *db, *dv, *ddis;
  int *didx;
  YG_CHECK(ws_get(ws, WS_H_B, (size_t)nb * d + 1, &db));
  YG_CHECK(ws_get(ws, WS_H_Q, (size_t)n * d + 1, &dv));
  YG_CHECK(ws_get(ws, WS_H_IDX, (size_t)n * k, &didx));
  YG_CHECK(ws_get(ws, WS_H_DIS, (size_t)n * k, &ddis));
  YG_CUDA(cudaMemcpyAsync(db, b, sizeof(float) * (size_t)nb * d, cudaMemcpyHostToDevice, st));
  YG_CUDA(cudaMemcpyAsync(dv, v, sizeof(float) * (size_t)n * d, cudaMemcpyHostToDevice, st));
  YG_CUDA(cudaMemcpyAsync(didx, idx, sizeof(int) * (size_t)n * k, cudaMemcpyHostToDevice, st));
  YG_CUDA(cudaMemcpyAsync(ddis, dis, sizeof(float) * (size_t)n * k, cudaMemcpyHostToDevice, st));
  const size_t smem = (size_t)k * 16;
  if (smem > 200 * 1024) {
    set_error(E_UNSUPPORTED, "knn_reorder_shortlist: k=%d too large", k);
    return E_UNSUPPORTED;
  }
  YG_CHECK(ensure_smem((const void *)reorder_kernel, smem));
  reorder_kernel<<<n, 128, smem, st>>>(n, nb, d, k, db, dv, didx, ddis);
  YG_LAUNCH_CHECK();
  YG_CUDA(cudaMemcpyAsync(idx, didx, sizeof(int) * (size_t)n * k, cudaMemcpyDeviceToHost, st));
  YG_CUDA(cudaMemcpyAsync(dis, ddis, sizeof(float) * (size_t)n * k, cudaMemcpyDeviceToHost, st));
  YG_CUDA(cudaStreamSynchronize(st));
  return OK;
}

static int recompute_host(int n, int nb, int d, int k, const float *b, const float *v,
                          int label0, int *kp, const int *idx, float *dis) {
  if (n <= 0) return OK;
  Ctx *ctx;
  YG_CHECK(ctx_get(&ctx));
  cudaStream_t st = ctx->stream;
  Workspace &ws = ctx->ws;
  float *db, *dv, *ddis;
  int *didx, *dkp, *bad;
  YG_CHECK(ws_get(ws, WS_H_B, (size_t)nb * d + 1, &db));
  YG_CHECK(ws_get(ws, WS_H_Q, (size_t)n * d + 1, &dv));
  YG_CHECK(ws_get(ws, WS_H_IDX, (size_t)n * k + 1, &didx));
  YG_CHECK(ws_get(ws, WS_H_DIS, (size_t)n * k + 1, &ddis));
  YG_CHECK(ws_get(ws, WS_H_W, (size_t)n + 1, &dkp));
  YG_CHECK(ws_get(ws, WS_H_EXTRA, 1, &bad));
  YG_CUDA(cudaMemcpyAsync(db, b, sizeof(float) * (size_t)nb * d, cudaMemcpyHostToDevice, st));
  YG_CUDA(cudaMemcpyAsync(dv, v, sizeof(float) * (size_t)n * d, cudaMemcpyHostToDevice, st));
  YG_CUDA(cudaMemcpyAsync(didx, idx, sizeof(int) * (size_t)n * k, cudaMemcpyHostToDevice, st));
  YG_CUDA(cudaMemcpyAsync(ddis, dis, sizeof(float) * (size_t)n * k, cudaMemcpyHostToDevice, st));
  YG_CUDA(cudaMemcpyAsync(dkp, kp, sizeof(int) * (size_t)n, cudaMemcpyHostToDevice, st));
  YG_CUDA(cudaMemsetAsync(bad, 0, sizeof(int), st));
  recompute_kernel<<<(unsigned)ceil_div(n, 128), 128, 0, st>>>(n, nb, d, k, db, dv, label0, dkp,
                                                               didx, ddis, bad);
  YG_LAUNCH_CHECK();
  int hbad = 0;
  YG_CUDA(cudaMemcpyAsync(dis, ddis, sizeof(float) * (size_t)n * k, cudaMemcpyDeviceToHost, st));
  YG_CUDA(cudaMemcpyAsync(kp, dkp, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost, st));
  YG_CUDA(cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, st));
  YG_CUDA(cudaStreamSynchronize(st));
  if (hbad) {
    set_error(E_ARG, "knn_recompute_exact_dists: id below label0 (yael asserts j >= 0)");
    return E_ARG;
  }
  return OK;
}

// ---- the other distance types of compute_cross_distances_alt (alt.cuh):
// one thread per output (a_i, b_j); the coordinates are walked in order
// through 32-wide slices staged in shared memory.
constexpr int AT = 16, AC = 32;  // pairs per block side, coordinates per slice

template <int TYPE, bool SSE>
__global__ void __launch_bounds__(AT * AT)
    alt_kernel(const float *__restrict__ a, int lda, int na, const float *__restrict__ b, int ldb,
               int nb, int d, float *out, int ldo) {
  __shared__ float sa[AT][AC + 1], sb[AT][AC + 1];
  const int ti = threadIdx.x % AT, tj = threadIdx.x / AT;
  const int i = blockIdx.x * AT + ti, j = blockIdx.y * AT + tj;
  AltAcc acc;
  for (int c0 = 0; c0 < d; c0 += AC) {
    const int w = min(AC, d - c0);
    __syncthreads();
    for (int e = threadIdx.x; e < AT * AC; e += AT * AT) {
      const int r = e / AC, c = e % AC;
      const long ia = (long)blockIdx.x * AT + r, jb = (long)blockIdx.y * AT + r;
      sa[r][c] = (c < w && ia < na) ? a[ia * lda + c0 + c] : 0.f;
      sb[r][c] = (c < w && jb < nb) ? b[jb * ldb + c0 + c] : 0.f;
    }
    __syncthreads();
    for (int c = 0; c < w; c++) alt_step<TYPE, SSE>(acc, sa[ti][c], sb[tj][c], c0 + c);
  }
  if (i >= na || j >= nb) return;
  out[(long)j * ldo + i] = alt_finish<SSE>(acc);
}

template <int TYPE, bool SSE>
void alt_launch(const float *a, int na, const float *b, int nb, int d, float *out, int ldo,
                cudaStream_t st) {
  dim3 grid((unsigned)ceil_div(na, AT), (unsigned)ceil_div(nb, AT));
  alt_kernel<TYPE, SSE><<<grid, AT * AT, 0, st>>>(a, d, na, b, d, nb, d, out, ldo);
}

// host arrays in, host matrix out (pitch ldd), chunked over b
int alt_host(int type, int d, int na, int nb, const float *a, int lda, const float *b, int ldb,
             float *dist2, int ldd) {
  if (na <= 0 || nb <= 0) return OK;
  if (d < 0 || lda < d || ldb < d || ldd < na) {
    set_error(E_ARG, "cross distances: bad leading dimensions");
    return E_ARG;
  }
  Ctx *ctx;
  YG_CHECK(ctx_get(&ctx));
  cudaStream_t st = ctx->stream;
  Workspace &ws = ctx->ws;
  float *da, *db, *dout;
  YG_CHECK(ws_get(ws, WS_H_Q, (size_t)na * d + 1, &da));
  YG_CHECK(ws_get(ws, WS_H_B, (size_t)nb * d + 1, &db));
  if (d > 0) {
    YG_CUDA(cudaMemcpy2DAsync(da, sizeof(float) * d, a, sizeof(float) * lda, sizeof(float) * d,
                              na, cudaMemcpyHostToDevice, st));
    YG_CUDA(cudaMemcpy2DAsync(db, sizeof(float) * d, b, sizeof(float) * ldb, sizeof(float) * d,
                              nb, cudaMemcpyHostToDevice, st));
  }
  const bool sse = (type == 1 || type == 3) && d % 4 == 0;
  long jb = (long)(((size_t)1 << 30) / ((size_t)na * 4));
  jb = std::max<long>(AT, jb / AT * AT);
  YG_CHECK(ws_get(ws, WS_H_DIS, (size_t)na * (size_t)imin(nb, (int)std::min<long>(jb, nb)), &dout));
  for (long j0 = 0; j0 < nb; j0 += jb) {
    const int nbc = (int)std::min<long>(jb, nb - j0);
    const float *bj = db + j0 * d;
    switch (type * 2 + (sse ? 1 : 0)) {
      case 2: alt_launch<1, false>(da, na, bj, nbc, d, dout, na, st); break;
      case 3: alt_launch<1, true>(da, na, bj, nbc, d, dout, na, st); break;
      case 4: alt_launch<2, false>(da, na, bj, nbc, d, dout, na, st); break;
      case 6: alt_launch<3, false>(da, na, bj, nbc, d, dout, na, st); break;
      case 7: alt_launch<3, true>(da, na, bj, nbc, d, dout, na, st); break;
      case 8: alt_launch<4, false>(da, na, bj, nbc, d, dout, na, st); break;
      case 10: alt_launch<5, false>(da, na, bj, nbc, d, dout, na, st); break;
      default: alt_launch<6, false>(da, na, bj, nbc, d, dout, na, st); break;
    }
    YG_LAUNCH_CHECK();
    YG_CUDA(cudaMemcpy2DAsync(dist2 + j0 * ldd, sizeof(float) * ldd, dout, sizeof(float) * na,
                              sizeof(float) * na, nbc, cudaMemcpyDeviceToHost, st));
  }
  YG_CUDA(cudaStreamSynchronize(st));
  return OK;
}

}  // namespace yg

using namespace yg;

static int alt_metric(int distance_type) {
  if (distance_type == 2 || distance_type == 12) return METRIC_L2;
  if (distance_type == 16) return METRIC_DOT;
  return -1;
}

extern "C" {

void compute_cross_distances_nonpacked(int d, int na, int nb, const float *a, int lda,
                                       const float *b, int ldb, float *dist2, int ldd) {
  if (cross_distances_host(METRIC_L2, d, na, nb, a, lda, b, ldb, dist2, ldd) != OK)
    fatal_last("compute_cross_distances_nonpacked");
}

void compute_cross_distances(int d, int na, int nb, const float *a, const float *b,
                             float *dist2) {
  compute_cross_distances_nonpacked(d, na, nb, a, d, b, d, dist2, na);
}

void compute_cross_distances_thread(int d, int na, int nb, const float *a, const float *b,
                                    float *dist2, int nt) {
  (void)nt;
  compute_cross_distances(d, na, nb, a, b, dist2);
}

void compute_cross_distances_alt_nonpacked(int distance_type, int d, int na, int nb,
                                           const float *a, int lda, const float *b, int ldb,
                                           float *dist2, int ldd) {
  // types 12 / 16: the expanded form and the plain product (yael/nn.c:321-328);
  // 1-6: per-coordinate sums (yael/nn.c:311-350, SSE forms at 164-259)
  if (distance_type == 12 || distance_type == 16) {
    if (cross_distances_host(alt_metric(distance_type), d, na, nb, a, lda, b, ldb, dist2, ldd) !=
        OK)
      fatal_last("compute_cross_distances_alt");
    return;
  }
  if (distance_type < 1 || distance_type > 6) {
    set_error(E_UNSUPPORTED, "distance_type %d is not one of 1-6, 12, 16", distance_type);
    fatal_last("compute_cross_distances_alt");
  }
  if (alt_host(distance_type, d, na, nb, a, lda, b, ldb, dist2, ldd) != OK)
    fatal_last("compute_cross_distances_alt");
}

void compute_cross_distances_alt(int distance_type, int d, int na, int nb, const float *a,
                                 const float *b, float *dist2) {
  compute_cross_distances_alt_nonpacked(distance_type, d, na, nb, a, d, b, d, dist2, na);
}

void compute_cross_distances_alt_thread(int distance_type, int d, int na, int nb,
                                        const float *a, const float *b, float *dist2, int nt) {
  (void)nt;
  compute_cross_distances_alt(distance_type, d, na, nb, a, b, dist2);
}

void compute_distances_1_nonpacked(int d, int nb, const float *a, const float *b, int ldb,
                                   float *dist2) {
  if (cross_distances_host(METRIC_L2, d, 1, nb, a, d, b, ldb, dist2, 1) != OK)
    fatal_last("compute_distances_1");
}

void compute_distances_1(int d, int nb, const float *a, const float *b, float *dist2) {
  compute_distances_1_nonpacked(d, nb, a, b, d, dist2);
}

void compute_distances_1_thread(int d, int nb, const float *a, const float *b, float *dist2,
                                int n_thread) {
  (void)n_thread;
  compute_distances_1(d, nb, a, b, dist2);
}

void compute_distances_1_nonpacked_thread(int d, int nb, const float *a, const float *b,
                                          int ldb, float *dist2, int n_thread) {
  (void)n_thread;
  compute_distances_1_nonpacked(d, nb, a, b, ldb, dist2);
}

void knn_reorder_shortlist(int n, int nb, int d, int k, const float *b, const float *v,
                           int *idx, float *dis) {
  if (reorder_host(n, nb, d, k, b, v, idx, dis) != OK) fatal_last("knn_reorder_shortlist");
}

void knn_recompute_exact_dists(int n, int nb, int d, int k, const float *b, const float *v,
                               int label0, int *kp, const int *idx, float *dis) {
  if (recompute_host(n, nb, d, k, b, v, label0, kp, idx, dis) != OK)
    fatal_last("knn_recompute_exact_dists");
}

}  // extern "C"
