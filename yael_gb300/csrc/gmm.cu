// Gaussian mixture models with diagonal covariances (yael/gmm.c): EM learning
// seeded by k-means, posteriors p(component | vector), Fisher vectors.
//
// Two device passes carry every cost that grows with the number of vectors:
//   * posteriors: the squared Mahalanobis distance of every (vector,
//     component) pair in direct form, sum_l (x_l - mu_l)^2 / sigma_l (tiles
//     of 32 vectors x 32 components staged in shared memory), then one warp per
//     vector turns its row into log densities and applies the reference's
//     thresholded softmax in place;
//   * moments: sum_i p_ij, sum_i p_ij x_il and sum_i p_ij x_il^2 for every
//     component and dimension (tiles of 32 components x 32 dimensions, FP32
//     within each step of 32 vectors, FP64 across steps and across vector
//     slices, summed in a fixed order: every result is reproducible).
// The EM update of the k x d parameters, the empty-component splits and the
// Fisher-vector formulas are host code over those moments.  The posterior
// matrix (n x k) stays on the device between the passes of an EM iteration.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "../../include/yael_gpu.h"
#include "common.cuh"

namespace yg {
namespace {

constexpr int GT = 32;                // tile edge
constexpr float kNormTo0 = 16.636f;   // log(2^24) (yael/gmm.c:264)
constexpr float kMinSigma = 1e-10f;   // yael/gmm.c:111

// M[i*k + j] = sum_l (v[i*d + l] - mu[j*d + l])^2 * isig[j*d + l]
// block 32 x 8: thread (tx, ty) owns component j0 + tx and vectors
// i0 + ty + 8r (r < 4)
__global__ void __launch_bounds__(256) maha_kernel(const float *__restrict__ v,
                                                   const float *__restrict__ mu,
                                                   const float *__restrict__ isig, long n, int k,
                                                   int d, float *__restrict__ M) {
  __shared__ float vs[GT][GT + 1];  // [vector][dimension]
  __shared__ float ms[GT][GT + 1];  // [dimension][component]
  __shared__ float is[GT][GT + 1];  // [dimension][component]
  const int tx = threadIdx.x, ty = threadIdx.y;
  const long i0 = (long)blockIdx.x * GT;
  const int j0 = blockIdx.y * GT;
  float acc[4] = {0.f, 0.f, 0.f, 0.f};
  for (int l0 = 0; l0 < d; l0 += GT) {
    const int l = l0 + tx;
#pragma unroll
    for (int r = 0; r < 4; r++) {
      const int row = ty + 8 * r;
      const long i = i0 + row;
      vs[row][tx] = (i < n && l < d) ? v[i * d + l] : 0.f;
      const int j = j0 + row;
      const bool ok = j < k && l < d;
      ms[tx][row] = ok ? mu[(long)j * d + l] : 0.f;
      is[tx][row] = ok ? isig[(long)j * d + l] : 0.f;
    }
    __syncthreads();
#pragma unroll 8
    for (int ll = 0; ll < GT; ll++) {
      const float m = ms[ll][tx], s = is[ll][tx];
#pragma unroll
      for (int r = 0; r < 4; r++) {
        const float t = vs[ty + 8 * r][ll] - m;
        acc[r] = fmaf(t * t, s, acc[r]);
      }
    }
    __syncthreads();
  }
  const int j = j0 + tx;
  if (j < k) {
#pragma unroll
    for (int r = 0; r < 4; r++) {
      const long i = i0 + ty + 8 * r;
      if (i < n) M[i * k + j] = acc[r];
    }
  }
}

// one warp per vector, in place on its row of P (squared Mahalanobis
// distances on entry): x_j = logdet_j - 0.5 M_ij + lg_j (yael/gmm.c:349-354),
// then softmax_ref (yael/gmm.c:262-300): x_j below max - 16.636 gives 0, the
// others exp(x_j - max), all divided by their sum
__global__ void softmax_kernel(float *__restrict__ P, const float *__restrict__ logdet,
                               const float *__restrict__ lg, long n, int k) {
  const int lane = threadIdx.x & 31;
  const long i = (long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (i >= n) return;  // whole warps leave together
  float *row = P + i * k;
  float mx = -1e30f;
  for (int j = lane; j < k; j += 32) {
    const float x = (float)((double)logdet[j] - 0.5 * (double)row[j] + (double)lg[j]);
    row[j] = x;
    if (x > mx) mx = x;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  const float thr = mx - kNormTo0;
  float s = 0.f;
  for (int j = lane; j < k; j += 32) {
    const float x = row[j];
    const float e = x >= thr ? expf(x - mx) : 0.f;
    row[j] = e;
    s += e;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (s != 0.f) {
    const float inv = (float)(1.0 / (double)s);
    for (int j = lane; j < k; j += 32) row[j] *= inv;
  }
}

// moments of vector slice z: for components j0.. and columns l0.. of
// [v | 1] (column d is the constant 1, so S1[., d] = sum_i p_ij),
// part1[z][j][l] = sum_i p_ij x_il and part2[z][j][l] = sum_i p_ij x_il^2
// over vectors [z*chunk, min(n, (z+1)*chunk)).  Block 32 x 8: thread (tx, ty)
// owns column l0 + tx and components j0 + ty + 8r (r < 4).
__global__ void __launch_bounds__(256) moments_kernel(const float *__restrict__ P,
                                                      const float *__restrict__ v, long n, int k,
                                                      int d, long chunk,
                                                      double *__restrict__ part1,
                                                      double *__restrict__ part2) {
  __shared__ float ps[GT][GT + 1];  // [vector][component]
  __shared__ float xs[GT][GT + 1];  // [vector][column]
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int l0 = blockIdx.x * GT, j0 = blockIdx.y * GT;
  const long z = blockIdx.z;
  const long ib = z * chunk, ie = min(n, ib + chunk);
  const int dc = d + 1;
  double a1[4] = {0, 0, 0, 0}, a2[4] = {0, 0, 0, 0};
  for (long c0 = ib; c0 < ie; c0 += GT) {
#pragma unroll
    for (int r = 0; r < 4; r++) {
      const int row = ty + 8 * r;
      const long i = c0 + row;
      const bool iok = i < ie;
      ps[row][tx] = (iok && j0 + tx < k) ? P[i * k + j0 + tx] : 0.f;
      const int l = l0 + tx;
      xs[row][tx] = !iok ? 0.f : l < d ? v[i * d + l] : (l == d ? 1.f : 0.f);
    }
    __syncthreads();
    float f1[4] = {0.f, 0.f, 0.f, 0.f}, f2[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll 8
    for (int ii = 0; ii < GT; ii++) {
      const float x = xs[ii][tx];
      const float x2 = x * x;
#pragma unroll
      for (int r = 0; r < 4; r++) {
        const float p = ps[ii][ty + 8 * r];
        f1[r] = fmaf(p, x, f1[r]);
        f2[r] = fmaf(p, x2, f2[r]);
      }
    }
#pragma unroll
    for (int r = 0; r < 4; r++) {
      a1[r] += (double)f1[r];
      a2[r] += (double)f2[r];
    }
    __syncthreads();
  }
  const int l = l0 + tx;
  if (l < dc) {
#pragma unroll
    for (int r = 0; r < 4; r++) {
      const int j = j0 + ty + 8 * r;
      if (j < k) {
        const long o = (z * k + j) * (long)dc + l;
        part1[o] = a1[r];
        part2[o] = a2[r];
      }
    }
  }
}

// out[t] = sum over slices z (in order) of part[z * m + t]
__global__ void sum_slices_kernel(const double *__restrict__ part, int nz, long m,
                                  double *__restrict__ out) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= m) return;
  double s = 0;
  for (int z = 0; z < nz; z++) s += part[(long)z * m + t];
  out[t] = s;
}

// nnz[j] += number of vectors of slice y with P[i*k + j] > 0.  Block 32 x 8:
// thread (tx, ty) counts component j0 + tx over vectors ty, ty + 8, ...
__global__ void nnz_kernel(const float *__restrict__ P, long n, int k, long chunk,
                           int *__restrict__ nnz) {
  __shared__ int red[8][GT];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int j = blockIdx.x * GT + tx;
  const long ib = (long)blockIdx.y * chunk, ie = min(n, ib + chunk);
  int c = 0;
  if (j < k)
    for (long i = ib + ty; i < ie; i += 8) c += P[i * k + j] > 0.f ? 1 : 0;
  red[ty][tx] = c;
  __syncthreads();
  if (ty == 0 && j < k) {
    int t = 0;
    for (int q = 0; q < 8; q++) t += red[q][tx];
    if (t) atomicAdd(nnz + j, t);
  }
}

// the split of gmm_handle_empty (yael/gmm.c:404-411): vectors with
// P[., j2] > 0 and v[., sd] < thr move their posterior from j2 to j
__global__ void transfer_kernel(float *__restrict__ P, const float *__restrict__ v, long n,
                                int k, int d, int j, int j2, int sd, float thr,
                                int *__restrict__ moved) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  int c = 0;
  if (i < n) {
    const float q = P[i * k + j2];
    if (q > 0.f && v[i * d + sd] < thr) {
      P[i * k + j] = q;
      P[i * k + j2] = 0.f;
      c = 1;
    }
  }
  c = __reduce_add_sync(0xffffffffu, c);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(moved, c);
}

[[noreturn]] void die(const char *where) { fatal_last(where); }

void ok(const char *where, cudaError_t e) {
  if (e != cudaSuccess) {
    set_error(E_CUDA, "%s", cudaGetErrorString(e));
    die(where);
  }
}

void launched(const char *where) {
  count_launch();
  ok(where, cudaGetLastError());
}

// The moments of a posterior matrix against a set of vectors, as FP64:
// s0[j] = sum_i p_ij, s1[j*d + l] = sum_i p_ij x_il, s2[j*d + l] = sum_i p_ij x_il^2
struct Moments {
  std::vector<double> s0, s1, s2;
};

// device state of one call: vectors, posteriors, parameters, moments
struct GmmDev {
  const char *where;
  Ctx *ctx = nullptr;
  long n = 0;
  int d = 0, k = 0;
  DevArray<float> v, P, mu, isig, logdet, lg;
  DevArray<double> part1, part2, sum1, sum2;
  DevArray<int> nnz, moved;

  GmmDev(const char *w, long n_, int d_, int k_) : where(w), n(n_), d(d_), k(k_) {
    if (ctx_get(&ctx) != OK) die(where);
  }
  void sync() { ok(where, cudaStreamSynchronize(ctx->stream)); }
  void upload_v(const float *hv) {
    ok(where, cudaMemcpyAsync(v.get(where, n * d), hv, sizeof(float) * (size_t)(n * d),
                              cudaMemcpyHostToDevice, ctx->stream));
  }
  void upload_P(const float *hp) {
    ok(where, cudaMemcpyAsync(P.get(where, n * k), hp, sizeof(float) * (size_t)(n * k),
                              cudaMemcpyHostToDevice, ctx->stream));
  }
  void download_P(float *hp) {
    ok(where, cudaMemcpyAsync(hp, P.p, sizeof(float) * (size_t)(n * k), cudaMemcpyDeviceToHost,
                              ctx->stream));
    sync();
  }

  // P = p(component | vector) for the mixture (w, mu, sigma): gmm_compute_p
  // (yael/gmm.c:305-362); flags & GMM_FLAGS_W adds log w_j
  void posteriors(const gmm_t *g, int flags) {
    std::vector<float> hl((size_t)k), hdet((size_t)k), his((size_t)k * d);
    const long kd = (long)k * d;
    for (long t = 0; t < kd; t++) his[t] = (float)(1.0 / g->sigma[t]);
    for (int j = 0; j < k; j++) {
      float det = (float)(-d / 2.0 * log(2 * M_PI));  // float accumulation as the reference
      for (int l = 0; l < d; l++) det = (float)(det - 0.5 * log(g->sigma[(long)j * d + l]));
      hdet[j] = det;
      hl[j] = (flags & YAEL_GMM_FLAGS_W) ? (float)log(g->w[j]) : 0.f;
    }
    cudaStream_t st = ctx->stream;
    ok(where, cudaMemcpyAsync(mu.get(where, kd), g->mu, sizeof(float) * kd,
                              cudaMemcpyHostToDevice, st));
    ok(where, cudaMemcpyAsync(isig.get(where, kd), his.data(), sizeof(float) * kd,
                              cudaMemcpyHostToDevice, st));
    ok(where, cudaMemcpyAsync(logdet.get(where, k), hdet.data(), sizeof(float) * k,
                              cudaMemcpyHostToDevice, st));
    ok(where, cudaMemcpyAsync(lg.get(where, k), hl.data(), sizeof(float) * k,
                              cudaMemcpyHostToDevice, st));
    P.get(where, n * k);
    const dim3 grid((unsigned)((n + GT - 1) / GT), (unsigned)((k + GT - 1) / GT));
    maha_kernel<<<grid, dim3(GT, 8), 0, st>>>(v.p, mu.p, isig.p, n, k, d, P.p);
    launched(where);
    softmax_kernel<<<(unsigned)((n + 7) / 8), 256, 0, st>>>(P.p, logdet.p, lg.p, n, k);
    launched(where);
    sync();  // the host arrays above are freed on return
  }

  // number of vectors with a positive posterior, per component
  std::vector<int> nonzeros() {
    cudaStream_t st = ctx->stream;
    ok(where, cudaMemsetAsync(nnz.get(where, k), 0, sizeof(int) * k, st));
    const long ny = std::min<long>(std::max<long>(1, (n + 4095) / 4096), 4096);
    const long chunk = (n + ny - 1) / ny;
    nnz_kernel<<<dim3((unsigned)((k + GT - 1) / GT), (unsigned)ny), dim3(GT, 8), 0, st>>>(
        P.p, n, k, chunk, nnz.p);
    launched(where);
    std::vector<int> h((size_t)k);
    ok(where, cudaMemcpyAsync(h.data(), nnz.p, sizeof(int) * k, cudaMemcpyDeviceToHost, st));
    sync();
    return h;
  }

  int transfer(int j, int j2, int sd, float thr) {
    cudaStream_t st = ctx->stream;
    ok(where, cudaMemsetAsync(moved.get(where, 1), 0, sizeof(int), st));
    transfer_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(P.p, v.p, n, k, d, j, j2, sd,
                                                                thr, moved.p);
    launched(where);
    int h = 0;
    ok(where, cudaMemcpyAsync(&h, moved.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    sync();
    return h;
  }

  Moments moments() {
    cudaStream_t st = ctx->stream;
    const int dc = d + 1;
    const long m = (long)k * dc;
    const long tiles = (long)((dc + GT - 1) / GT) * ((k + GT - 1) / GT);
    const long want = (4L * (ctx->num_sms > 0 ? ctx->num_sms : 148) + tiles - 1) / tiles;
    const long nz = std::max(1L, std::min(want, (n + GT - 1) / GT));
    const long chunk = ((n + nz - 1) / nz + GT - 1) / GT * GT;
    part1.get(where, nz * m);
    part2.get(where, nz * m);
    moments_kernel<<<dim3((unsigned)((dc + GT - 1) / GT), (unsigned)((k + GT - 1) / GT),
                          (unsigned)nz),
                     dim3(GT, 8), 0, st>>>(P.p, v.p, n, k, d, chunk, part1.p, part2.p);
    launched(where);
    const unsigned rb = (unsigned)((m + 255) / 256);
    sum_slices_kernel<<<rb, 256, 0, st>>>(part1.p, (int)nz, m, sum1.get(where, m));
    launched(where);
    sum_slices_kernel<<<rb, 256, 0, st>>>(part2.p, (int)nz, m, sum2.get(where, m));
    launched(where);
    std::vector<double> h1((size_t)m), h2((size_t)m);
    ok(where, cudaMemcpyAsync(h1.data(), sum1.p, sizeof(double) * m, cudaMemcpyDeviceToHost, st));
    ok(where, cudaMemcpyAsync(h2.data(), sum2.p, sizeof(double) * m, cudaMemcpyDeviceToHost, st));
    sync();
    Moments r;
    r.s0.resize((size_t)k);
    r.s1.resize((size_t)k * d);
    r.s2.resize((size_t)k * d);
    for (int j = 0; j < k; j++) {
      r.s0[j] = h1[(size_t)j * dc + d];
      for (int l = 0; l < d; l++) {
        r.s1[(size_t)j * d + l] = h1[(size_t)j * dc + l];
        r.s2[(size_t)j * d + l] = h2[(size_t)j * dc + l];
      }
    }
    return r;
  }
};

gmm_t *gmm_alloc(int d, int k) {
  gmm_t *g = (gmm_t *)malloc(sizeof(gmm_t));
  g->d = d;
  g->k = k;
  g->w = (float *)malloc(sizeof(float) * (size_t)(k > 0 ? k : 1));
  g->mu = (float *)malloc(sizeof(float) * (size_t)((long)k * d + 1));
  g->sigma = (float *)malloc(sizeof(float) * (size_t)((long)k * d + 1));
  return g;
}

void print_fvec(const float *v, int n) {  // fvec_print (yael/vector.c:1587-1594)
  printf("[");
  for (int i = 0; i < n; i++) printf("%g ", v[i]);
  printf("]\n");
}

// gmm_handle_empty (yael/gmm.c:366-433): each component without any positive
// posterior takes, from the next component in steps of 1000003 (mod k) that
// has some and holds at least n / k vectors, the vectors below that
// component's mean along its dimension of largest variance
void handle_empty(GmmDev &dev, const gmm_t *g) {
  const long n = dev.n;
  const int k = dev.k, d = dev.d;
  const std::vector<int> nnz = dev.nonzeros();
  long nz = 0;
  for (int j = 0; j < k; j++) nz += n - nnz[j];
  printf("nb of 0 probabilities: %ld / (%ld*%ld) = %.1f %%\n", nz, (long)k, n,
         nz * 100.0 / ((double)k * n));
  // the reference's w[j] (a float sum of non-negative posteriors) is positive
  // exactly when the component has a positive posterior; -1 after a split
  std::vector<int> state((size_t)k);
  for (int j = 0; j < k; j++) state[j] = nnz[j] > 0 ? 1 : 0;
  const int bigprime = 1000003;
  for (int j = 0; j < k; j++) {
    if (state[j] != 0) continue;
    printf("center %d is empty....", j);
    fflush(stdout);
    int j2 = j, tries = 0;
    for (;;) {
      int i;
      for (i = 0; i < k; i++) {
        j2 = (int)(((long)j2 + bigprime) % k);
        if (state[j2] > 0) break;
      }
      if (i == k || ++tries > k) {
        set_error(E_ARG, "gmm_learn: could not find a component to split");
        die("gmm_learn");
      }
      printf("try share with cent %d...", j2);
      fflush(stdout);
      // a component is split once and never receives: its count is still nnz
      if (nnz[j2] < n / k) {
        printf("has too few pts (%d)...", nnz[j2]);
        fflush(stdout);
        continue;
      }
      break;
    }
    const float *sj2 = g->sigma + (long)d * j2;
    int sd = 0;  // fvec_arg_max: first maximum
    for (int l = 1; l < d; l++)
      if (sj2[l] > sj2[sd]) sd = l;
    const int nt = dev.transfer(j, j2, sd, g->mu[(long)j2 * d + sd]);
    printf("split %d at dim %d (variance %g, transferred %d/%d pts)\n", j2, sd, sj2[sd], nt,
           nnz[j2]);
    if (nt == nnz[j2] || nt == 0) printf("  still not balanced !!! (expect crash)\n");
    state[j2] = -1;
  }
}

// gmm_compute_params (yael/gmm.c:114-199) from the moments of the posteriors
void compute_params(GmmDev &dev, gmm_t *g, int flags) {
  const int k = dev.k, d = dev.d;
  const Moments m = dev.moments();
  const std::vector<float> mu_old(g->mu, g->mu + (long)k * d);
  for (int j = 0; j < k; j++) {
    g->w[j] = (float)m.s0[j];
    for (int l = 0; l < d; l++) {
      const size_t t = (size_t)j * d + l;
      const double mo = mu_old[t];
      g->mu[t] = (float)m.s1[t];
      // sum_i p_ij (x_il - mu_old_jl)^2, expanded around the previous means
      g->sigma[t] = (float)(m.s2[t] - 2.0 * mo * m.s1[t] + mo * mo * m.s0[j]);
    }
  }
  if (flags & YAEL_GMM_FLAGS_1SIGMA) {
    for (int j = 0; j < k; j++) {
      float *sj = g->sigma + (long)j * d;
      double s = 0;
      for (int l = 0; l < d; l++) s += sj[l];
      const float var = (float)(s / d);
      for (int l = 0; l < d; l++) sj[l] = var;
    }
  }
  long nz = 0;
  for (long t = 0; t < (long)k * d; t++)
    if (g->sigma[t] < kMinSigma) {
      g->sigma[t] = kMinSigma;
      nz++;
    }
  if (nz) printf("WARN %ld sigma diagonals are too small (set to %g)\n", nz, kMinSigma);
  double msum = 0;
  for (long t = 0; t < (long)k * d; t++) msum += g->mu[t];
  if (!isfinite(msum)) {
    set_error(E_ARG, "gmm_learn: non-finite means");
    die("gmm_learn");
  }
  for (int j = 0; j < k; j++) {  // fvec_div_by: times 1 / w in double
    const double inv = 1.0 / g->w[j];
    for (int l = 0; l < d; l++) {
      g->mu[(long)j * d + l] = (float)(g->mu[(long)j * d + l] * inv);
      g->sigma[(long)j * d + l] = (float)(g->sigma[(long)j * d + l] * inv);
    }
  }
  double wn = 0;  // fvec_normalize(w, k, 1)
  for (int j = 0; j < k; j++) wn += fabs((double)g->w[j]);
  for (int j = 0; j < k; j++) g->w[j] = (float)(g->w[j] * (1.0 / wn));
  printf("w = ");
  print_fvec(g->w, k);
  double ss = 0;
  for (int j = 0; j < k; j++) ss += (double)g->w[j] * g->w[j];
  printf(" imfac = %.3f\n", k * ss);
}

// gmm_fisher_from_posteriors (yael/gmm.c:527-725) from the moments
void fisher_from_moments(const Moments &m, long n, const gmm_t *g, int flags, float *out) {
  const long d = g->d, k = g->k;
  long ii = 0;
  auto MU = [&](long l, long j) { return (double)g->mu[j * d + l]; };
  auto SG = [&](long l, long j) { return (double)g->sigma[j * d + l]; };
  if (flags & YAEL_GMM_FLAGS_W) {
    for (long j = 1; j < k; j++) {
      const double accu = m.s0[j] / g->w[j] - m.s0[0] / g->w[0];
      const double f = n * (1.0 / g->w[j] + 1.0 / g->w[0]);
      out[ii++] = (float)(accu / sqrt(f));
    }
  }
  if (flags & YAEL_GMM_FLAGS_MU) {
    float *dmu = out + ii;
    for (long j = 0; j < k; j++)
      for (long l = 0; l < d; l++) {
        double x = (m.s1[j * d + l] - MU(l, j) * m.s0[j]) / SG(l, j);
        if (!(flags & YAEL_GMM_FLAGS_NO_NORM)) {
          const double nf = sqrt(n * (double)g->w[j] / SG(l, j));
          if (nf > 0) x /= nf;
        }
        dmu[j * d + l] = (float)x;
      }
    ii += d * k;
  }
  if (flags & (YAEL_GMM_FLAGS_SIGMA | YAEL_GMM_FLAGS_1SIGMA)) {
    // sum_i p_ij (x_il - mu_jl)^2
    auto dev2 = [&](long l, long j) {
      const double mu = MU(l, j);
      return m.s2[j * d + l] - 2.0 * mu * m.s1[j * d + l] + mu * mu * m.s0[j];
    };
    if (flags & YAEL_GMM_FLAGS_1SIGMA) {
      for (long j = 0; j < k; j++) {
        double accu2 = 0;
        for (long l = 0; l < d; l++) {
          const double sg = SG(l, j);
          const double accu = (dev2(l, j) / sg - m.s0[j]) / sqrt(sg);
          if (flags & YAEL_GMM_FLAGS_SIGMA) {
            const double f = (flags & YAEL_GMM_FLAGS_NO_NORM) ? 1.0 : 2 * n * (double)g->w[j] / sg;
            out[ii++] = (float)(accu / sqrt(f));
          }
          accu2 += accu;
        }
        const double f =
            (flags & YAEL_GMM_FLAGS_NO_NORM) ? 1.0 : 2 * d * n * (double)g->w[j] / SG(0, j);
        out[ii++] = (float)(accu2 / sqrt(f));
      }
    } else {
      float *dsg = out + ii;
      for (long j = 0; j < k; j++)
        for (long l = 0; l < d; l++) {
          const double sg = SG(l, j);
          const double accu = dev2(l, j) - m.s0[j] * sg;
          const double f = (flags & YAEL_GMM_FLAGS_NO_NORM)
                               ? pow(sg, -1.5)
                               : 1 / (sg * sqrt(2 * n * (double)g->w[j]));
          dsg[l + j * d] = (float)(accu * f);
        }
      ii += d * k;
    }
  }
}

}  // namespace
}  // namespace yg

using namespace yg;

extern "C" {

void gmm_delete(gmm_t *g) {
  free(g->w);
  free(g->mu);
  free(g->sigma);
  free(g);
}

gmm_t *gmm_learn(int di, int ni, int ki, int niter, const float *v, int nt, int seed, int nredo,
                 int flags) {
  const long d = di, k = ki, n = ni;
  niter = niter == 0 ? 10000 : niter;
  gmm_t *g = gmm_alloc(di, ki);
  // initialisation: k-means, weights 1 / k, one variance for every diagonal
  std::vector<int> nassign((size_t)(k > 0 ? k : 1));
  std::vector<float> dis((size_t)(n > 0 ? n : 1));
  kmeans(di, ni, ki, niter, v, nt, seed, nredo, g->mu, dis.data(), nullptr, nassign.data());
  fflush(stderr);
  fprintf(stderr, "assign = ");
  fflush(stderr);
  printf("[");
  for (long j = 0; j < k; j++) printf("%d ", nassign[j]);
  printf("]\n");
  fprintf(stderr, "\n");
  for (long j = 0; j < k; j++) g->w[j] = (float)(1.0 / k);
  double sig = 0;
  for (long i = 0; i < n; i++) sig += dis[i];
  sig /= n;
  printf("sigma at initialization = %.3f\n", sig);
  for (long t = 0; t < k * d; t++) g->sigma[t] = (float)sig;
  fprintf(stdout, "<><><><> GMM  <><><><><>\n");
  if (flags & YAEL_GMM_FLAGS_PURE_KMEANS) niter = 0;
  if (niter > 0 && n > 0) {
    GmmDev dev("gmm_learn", n, di, ki);
    dev.upload_v(v);
    double key = 666, old_key;
    for (int iter = 1; iter <= niter; iter++) {
      dev.posteriors(g, flags);
      fflush(stdout);
      handle_empty(dev, g);
      compute_params(dev, g, flags);
      fflush(stdout);
      old_key = key;
      key = 0;
      for (long t = 0; t < k * d; t++) key += g->mu[t];
      printf("keys %5d: %.6f -> %.6f\n", iter, old_key, key);
      fflush(stdout);
      if (key == old_key) break;
    }
  }
  fprintf(stderr, "\n");
  return g;
}

void gmm_compute_p(int n, const float *v, const gmm_t *g, float *p, int flags) {
  if (n == 0) return;
  GmmDev dev("gmm_compute_p", n, g->d, g->k);
  dev.upload_v(v);
  dev.posteriors(g, flags);
  dev.download_P(p);
}

void gmm_compute_p_thread(int n, const float *v, const gmm_t *g, float *p, int flags,
                          int n_thread) {
  (void)n_thread;
  gmm_compute_p(n, v, g, p, flags);
}

size_t gmm_fisher_sizeof(const gmm_t *g, int flags) {
  int sz = 0;
  if (flags & YAEL_GMM_FLAGS_W) sz += g->k - 1;
  if (flags & YAEL_GMM_FLAGS_MU) sz += g->d * g->k;
  if (flags & YAEL_GMM_FLAGS_1SIGMA) sz += g->k;
  if (flags & YAEL_GMM_FLAGS_SIGMA) sz += g->d * g->k;
  return sz;
}

void gmm_fisher(int n, const float *v, const gmm_t *g, int flags, float *dp_dlambda) {
  GmmDev dev("gmm_fisher", n, g->d, g->k);
  Moments m;
  if (n > 0) {
    dev.upload_v(v);
    dev.posteriors(g, flags | YAEL_GMM_FLAGS_W);
    m = dev.moments();
  } else {
    m.s0.assign((size_t)g->k, 0.0);
    m.s1.assign((size_t)g->k * g->d, 0.0);
    m.s2.assign((size_t)g->k * g->d, 0.0);
  }
  fisher_from_moments(m, n, g, flags, dp_dlambda);
}

void gmm_fisher_from_posteriors(int n, const float *v, const gmm_t *g, int flags,
                                const float *p, float *dp_dlambda) {
  GmmDev dev("gmm_fisher_from_posteriors", n, g->d, g->k);
  Moments m;
  if (n > 0) {
    dev.upload_v(v);
    dev.upload_P(p);
    m = dev.moments();
  } else {
    m.s0.assign((size_t)g->k, 0.0);
    m.s1.assign((size_t)g->k * g->d, 0.0);
    m.s2.assign((size_t)g->k * g->d, 0.0);
  }
  fisher_from_moments(m, n, g, flags, dp_dlambda);
}

void gmm_fisher_spatial(int N, int K, int D, const float *Q, const float *sgmm, const float *ll,
                        float *sdesc) {
  // ll is D x N (coordinate d of vector i at ll[d * N + i]): transposed to
  // the vector-major layout of the moments pass
  std::vector<float> llt((size_t)N * D + 1);
  for (long i = 0; i < N; i++)
    for (long c = 0; c < D; c++) llt[i * D + c] = ll[c * N + i];
  GmmDev dev("gmm_fisher_spatial", N, D, K);
  Moments m;
  if (N > 0) {
    dev.upload_v(llt.data());
    dev.upload_P(Q);
    m = dev.moments();
  } else {
    m.s0.assign((size_t)K, 0.0);
    m.s1.assign((size_t)K * D, 0.0);
    m.s2.assign((size_t)K * D, 0.0);
  }
  const float *mm = sgmm, *S = sgmm + D;
  float *d_mm = sdesc, *d_S = sdesc + (long)K * D;
  for (long c = 0; c < D; c++)
    for (long j = 0; j < K; j++) {
      const double qs = m.s0[j] / N, ql = m.s1[j * D + c] / N, ql2 = m.s2[j * D + c] / N;
      d_mm[c + j * D] = (float)(ql - qs * mm[c]);
      d_S[c + j * D] = (float)(-ql2 + 2 * ql * mm[c] + qs * ((double)S[c] - (double)mm[c] * mm[c]));
    }
}

void gmm_print(const gmm_t *g) {
  printf("gmm (%d gaussians in %d dim)=[\n", g->k, g->d);
  for (int i = 0; i < g->k; i++) {
    printf("   w=%g, mu=[", g->w[i]);
    for (int j = 0; j < g->d; j++) printf("%g ", g->mu[(long)i * g->d + j]);
    printf("], sigma=diag([");
    for (int j = 0; j < g->d; j++) printf("%g ", g->sigma[(long)i * g->d + j]);
    printf("])\n");
  }
  printf("]\n");
}

// gmm_write / gmm_read (yael/gmm.c:810-850): d, k, w, mu, sigma as raw int32
// and float32; an I/O error prints and aborts
static void write_or_abort(const void *a, size_t sz, size_t n, FILE *f) {
  if (fwrite(a, sz, n, f) != n) {
    perror("gmm_write");
    abort();
  }
}

static void read_or_abort(void *a, size_t sz, size_t n, FILE *f) {
  if (fread(a, sz, n, f) != n) {
    perror("gmm_read");
    abort();
  }
}

void gmm_write(const gmm_t *g, FILE *f) {
  write_or_abort(&g->d, sizeof(int), 1, f);
  write_or_abort(&g->k, sizeof(int), 1, f);
  write_or_abort(g->w, sizeof(float), (size_t)g->k, f);
  write_or_abort(g->mu, sizeof(float), (size_t)g->k * g->d, f);
  write_or_abort(g->sigma, sizeof(float), (size_t)g->k * g->d, f);
}

gmm_t *gmm_read(FILE *f) {
  int d, k;
  read_or_abort(&d, sizeof(int), 1, f);
  read_or_abort(&k, sizeof(int), 1, f);
  gmm_t *g = gmm_alloc(d, k);
  read_or_abort(g->w, sizeof(float), (size_t)k, f);
  read_or_abort(g->mu, sizeof(float), (size_t)k * d, f);
  read_or_abort(g->sigma, sizeof(float), (size_t)k * d, f);
  return g;
}

}  // extern "C"
