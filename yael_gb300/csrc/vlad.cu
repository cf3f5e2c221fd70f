// VLAD and bag-of-features descriptors (yael/vlad.c:10-139) on the exact
// nearest-centroid assignment of the k-NN pipeline.
//
// A VLAD sum is float arithmetic in a fixed order: the reference adds the
// residuals (v_i - c) of a cluster's points in increasing point order (list
// order for the subset form).  Here the point indices are sorted stably by
// cluster (radix sort: equal keys keep their order), and one thread per
// (cluster, coordinate) walks its cluster's points in that order with
// round-to-nearest adds and multiplies that the compiler may not fuse, so each
// output is the reference's own sequence of float operations.  Bag-of-features
// counts are integer (or exact float) histograms.
#include <limits.h>
#include <string.h>

#include <cub/device/device_radix_sort.cuh>

#include "knn.cuh"

namespace yg {
namespace {

enum VladSlot : int {
  VS_V = 220, VS_C, VS_ASSIGN, VS_DIS, VS_KEYS, VS_KEYS2, VS_VALS, VS_VALS2, VS_OFFS, VS_TMP,
  VS_DESC, VS_W, VS_SUBIDX, VS_SUBEND,
};

template <typename T>
int vs_get(Workspace &ws, int slot, size_t count, T **p) {
  void *v = nullptr;
  YG_CHECK(ws.get(slot, (count ? count : 1) * sizeof(T), &v));
  *p = reinterpret_cast<T *>(v);
  return OK;
}

// sort key of element e: cluster of point idx[e] (or e), with the subset
// index above it; points without a nearest centroid (all-NaN rows) go past
// every segment
__global__ void keys_kernel(const int *assign, const int *idx, const int *sub_of, long n, int k,
                            int *keys, int *vals) {
  const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const int i = idx ? idx[e] : (int)e;
  const int a = assign[i];
  const int s = sub_of ? sub_of[e] : 0;
  keys[e] = a < 0 ? INT_MAX : s * k + a;
  vals[e] = i;
}

// offs[g] = first sorted element of segment g (g < nseg), offs[nseg] = end
__global__ void offsets_kernel(const int *sorted, long n, int nseg, int *offs) {
  const long g = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g > nseg) return;
  long lo = 0, hi = n;
  while (lo < hi) {
    const long mid = (lo + hi) / 2;
    if (sorted[mid] < g) lo = mid + 1; else hi = mid;
  }
  offs[g] = (int)lo;
}

// desc[g][j], g = subset * k + c: the ordered sum of (v_i[j] - C[c][j]) (* w_i)
__global__ void vlad_sum_kernel(const int *perm, const int *offs, const float *v, int d,
                                const float *C, const float *w, int k, long nseg, float *desc) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nseg * d) return;
  const long g = t / d;
  const int j = (int)(t - g * d), c = (int)(g % k);
  const float cj = C[(long)c * d + j];
  float s = 0.f;
  for (int e = offs[g]; e < offs[g + 1]; e++) {
    const int i = perm[e];
    float r = __fsub_rn(v[(long)i * d + j], cj);
    if (w) r = __fmul_rn(r, w[i]);
    s = __fadd_rn(s, r);
  }
  desc[t] = s;
}

__global__ void hist_int_kernel(const int *assign, long n, int k, int *desc) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int a = assign[i];
  if (a >= 0 && a < k) atomicAdd(desc + a, 1);
}

// subset s of the list: elements [ends[s-1], ends[s]) (integer counts, stored
// as float: exact below 2^24)
__global__ void hist_sub_kernel(const int *assign, const int *idx, const int *sub_of, long n, int k,
                                float *desc) {
  const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const int a = assign[idx[e]];
  if (a >= 0 && a < k) atomicAdd(desc + (long)sub_of[e] * k + a, 1.f);
}

__global__ void subset_of_kernel(const int *ends, int nsub, long n, int *sub_of) {
  const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  int lo = 0, hi = nsub - 1;  // first subset whose end is past e
  while (lo < hi) {
    const int mid = (lo + hi) / 2;
    if (ends[mid] > e) hi = mid; else lo = mid + 1;
  }
  sub_of[e] = lo;
}

struct Assigned {
  Ctx *ctx = nullptr;
  cudaStream_t st = nullptr;
  float *dv = nullptr, *dc = nullptr;
  int *assign = nullptr;
};

// the ma nearest centroids of every point (yael's nn / knn_thread semantics)
int assign_points(int k, int d, const float *centroids, int n, const float *v, int ma,
                  Assigned *A) {
  YG_CHECK(ctx_get(&A->ctx));
  A->st = A->ctx->stream;
  Workspace &ws = A->ctx->ws;
  float *dis;
  YG_CHECK(vs_get(ws, VS_V, (size_t)n * d, &A->dv));
  YG_CHECK(vs_get(ws, VS_C, (size_t)k * d, &A->dc));
  YG_CHECK(vs_get(ws, VS_ASSIGN, (size_t)n * ma, &A->assign));
  YG_CHECK(vs_get(ws, VS_DIS, (size_t)n * ma, &dis));
  YG_CUDA(cudaMemcpyAsync(A->dv, v, sizeof(float) * n * (size_t)d, cudaMemcpyHostToDevice, A->st));
  YG_CUDA(cudaMemcpyAsync(A->dc, centroids, sizeof(float) * k * (size_t)d, cudaMemcpyHostToDevice,
                          A->st));
  KnnJob job;
  job.nq = n; job.nb = k; job.d = d; job.k = ma; job.metric = METRIC_L2;
  job.prec = default_precision();
  job.q = A->dv; job.ldq = d; job.b = A->dc; job.ldb = d;
  job.out_idx = A->assign; job.out_dis = dis;
  return knn_device(job, A->ctx, A->st);
}

// the sorted (segment, point) order of n elements and the segment offsets
int sort_segments(Assigned &A, const int *idx, const int *sub_of, long n, int k, int nseg,
                  int **perm, int **offs) {
  Workspace &ws = A.ctx->ws;
  int *keys, *keys2, *vals, *vals2;
  YG_CHECK(vs_get(ws, VS_KEYS, n, &keys));
  YG_CHECK(vs_get(ws, VS_KEYS2, n, &keys2));
  YG_CHECK(vs_get(ws, VS_VALS, n, &vals));
  YG_CHECK(vs_get(ws, VS_VALS2, n, &vals2));
  YG_CHECK(vs_get(ws, VS_OFFS, (size_t)nseg + 1, offs));
  if (n > 0) {
    keys_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, A.st>>>(A.assign, idx, sub_of, n, k, keys,
                                                               vals);
    YG_LAUNCH_CHECK();
    size_t tb = 0;
    YG_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tb, keys, keys2, vals, vals2, (int)n, 0, 32,
                                            A.st));
    void *tmp;
    YG_CHECK(A.ctx->ws.get(VS_TMP, tb ? tb : 1, &tmp));
    YG_CUDA(cub::DeviceRadixSort::SortPairs(tmp, tb, keys, keys2, vals, vals2, (int)n, 0, 32,
                                            A.st));
  }
  offsets_kernel<<<(unsigned)ceil_div((long)nseg + 1, 256), 256, 0, A.st>>>(keys2, n, nseg, *offs);
  YG_LAUNCH_CHECK();
  *perm = vals2;
  return OK;
}

int vlad_run(int k, int d, const float *centroids, int n, const float *v, const float *weights,
             int n_subset, const int *subset_indexes, const int *subset_ends, float *desc) {
  if (k < 1 || d < 1 || n < 0 || n_subset < 0) {
    set_error(E_ARG, "vlad: invalid sizes k=%d d=%d n=%d", k, d, n);
    return E_ARG;
  }
  const bool subsets = subset_indexes != nullptr;
  const int nsub = subsets ? n_subset : 1;
  const long nseg = (long)nsub * k;
  if (nseg > INT_MAX - 1 || (long)n * d > ((long)1 << 40)) {
    set_error(E_UNSUPPORTED, "vlad: sizes too large");
    return E_UNSUPPORTED;
  }
  if (n == 0 || (subsets && (nsub == 0 || subset_ends[nsub - 1] == 0))) {
    memset(desc, 0, sizeof(float) * nseg * d);
    return OK;
  }
  Assigned A;
  YG_CHECK(assign_points(k, d, centroids, n, v, 1, &A));
  Workspace &ws = A.ctx->ws;
  const float *dw = nullptr;
  if (weights) {
    float *w;
    YG_CHECK(vs_get(ws, VS_W, n, &w));
    YG_CUDA(cudaMemcpyAsync(w, weights, sizeof(float) * n, cudaMemcpyHostToDevice, A.st));
    dw = w;
  }
  const int *didx = nullptr, *dsub = nullptr;
  long ne = n;
  if (subsets) {
    ne = subset_ends[nsub - 1];
    int *ix, *ends, *so;
    YG_CHECK(vs_get(ws, VS_SUBIDX, ne, &ix));
    YG_CHECK(vs_get(ws, VS_SUBEND, (size_t)nsub + ne, &ends));
    so = ends + nsub;
    YG_CUDA(cudaMemcpyAsync(ix, subset_indexes, sizeof(int) * ne, cudaMemcpyHostToDevice, A.st));
    YG_CUDA(cudaMemcpyAsync(ends, subset_ends, sizeof(int) * nsub, cudaMemcpyHostToDevice, A.st));
    subset_of_kernel<<<(unsigned)ceil_div(ne, 256), 256, 0, A.st>>>(ends, nsub, ne, so);
    YG_LAUNCH_CHECK();
    didx = ix;
    dsub = so;
  }
  int *perm, *offs;
  YG_CHECK(sort_segments(A, didx, dsub, ne, k, (int)nseg, &perm, &offs));
  float *ddesc;
  YG_CHECK(vs_get(ws, VS_DESC, (size_t)nseg * d, &ddesc));
  vlad_sum_kernel<<<(unsigned)ceil_div(nseg * d, 256), 256, 0, A.st>>>(perm, offs, A.dv, d, A.dc,
                                                                       dw, k, nseg, ddesc);
  YG_LAUNCH_CHECK();
  YG_CUDA(cudaMemcpyAsync(desc, ddesc, sizeof(float) * nseg * d, cudaMemcpyDeviceToHost, A.st));
  YG_CUDA(cudaStreamSynchronize(A.st));
  return OK;
}

int bof_run(int k, int d, const float *centroids, int n, const float *v, int ma, int n_subset,
            const int *subset_indexes, const int *subset_ends, int *desc_i, float *desc_f) {
  if (k < 1 || d < 1 || n < 0 || ma < 1 || ma > k) {
    set_error(E_ARG, "bof: invalid sizes k=%d d=%d n=%d ma=%d", k, d, n, ma);
    return E_ARG;
  }
  const bool subsets = subset_indexes != nullptr;
  if (!subsets) memset(desc_i, 0, sizeof(int) * (size_t)k);
  else memset(desc_f, 0, sizeof(float) * (size_t)k * n_subset);
  const long ne = subsets ? (n_subset > 0 ? subset_ends[n_subset - 1] : 0) : (long)n * ma;
  if (n == 0 || ne == 0) return OK;
  Assigned A;
  YG_CHECK(assign_points(k, d, centroids, n, v, ma, &A));
  Workspace &ws = A.ctx->ws;
  if (!subsets) {
    int *dd;
    YG_CHECK(vs_get(ws, VS_DESC, k, &dd));
    YG_CUDA(cudaMemsetAsync(dd, 0, sizeof(int) * k, A.st));
    hist_int_kernel<<<(unsigned)ceil_div(ne, 256), 256, 0, A.st>>>(A.assign, ne, k, dd);
    YG_LAUNCH_CHECK();
    YG_CUDA(cudaMemcpyAsync(desc_i, dd, sizeof(int) * k, cudaMemcpyDeviceToHost, A.st));
  } else {
    int *ix, *ends;
    float *dd;
    YG_CHECK(vs_get(ws, VS_SUBIDX, ne, &ix));
    YG_CHECK(vs_get(ws, VS_SUBEND, (size_t)n_subset + ne, &ends));
    YG_CHECK(vs_get(ws, VS_DESC, (size_t)k * n_subset, &dd));
    YG_CUDA(cudaMemcpyAsync(ix, subset_indexes, sizeof(int) * ne, cudaMemcpyHostToDevice, A.st));
    YG_CUDA(cudaMemcpyAsync(ends, subset_ends, sizeof(int) * n_subset, cudaMemcpyHostToDevice,
                            A.st));
    subset_of_kernel<<<(unsigned)ceil_div(ne, 256), 256, 0, A.st>>>(ends, n_subset, ne,
                                                                    ends + n_subset);
    YG_LAUNCH_CHECK();
    YG_CUDA(cudaMemsetAsync(dd, 0, sizeof(float) * (size_t)k * n_subset, A.st));
    hist_sub_kernel<<<(unsigned)ceil_div(ne, 256), 256, 0, A.st>>>(A.assign, ix, ends + n_subset,
                                                                   ne, k, dd);
    YG_LAUNCH_CHECK();
    YG_CUDA(cudaMemcpyAsync(desc_f, dd, sizeof(float) * (size_t)k * n_subset,
                            cudaMemcpyDeviceToHost, A.st));
  }
  YG_CUDA(cudaStreamSynchronize(A.st));
  return OK;
}

}  // namespace
}  // namespace yg

using namespace yg;

extern "C" {

void vlad_compute(int k, int d, const float *centroids, int n, const float *v, float *desc) {
  if (vlad_run(k, d, centroids, n, v, nullptr, 0, nullptr, nullptr, desc) != OK)
    fatal_last("vlad_compute");
}

void vlad_compute_weighted(int k, int d, const float *centroids, int n, const float *v,
                           const float *weights, float *desc) {
  if (vlad_run(k, d, centroids, n, v, weights, 0, nullptr, nullptr, desc) != OK)
    fatal_last("vlad_compute_weighted");
}

void vlad_compute_subsets(int k, int d, const float *centroids, int n, const float *v,
                          int n_subset, const int *subset_indexes, const int *subset_ends,
                          float *desc) {
  if (vlad_run(k, d, centroids, n, v, nullptr, n_subset, subset_indexes, subset_ends, desc) != OK)
    fatal_last("vlad_compute_subsets");
}

void bof_compute(int k, int d, const float *centroids, int n, const float *v, int *desc) {
  if (bof_run(k, d, centroids, n, v, 1, 0, nullptr, nullptr, desc, nullptr) != OK)
    fatal_last("bof_compute");
}

void bof_compute_ma(int k, int d, const float *centroids, int n, const float *v, int *desc, int ma,
                    float alpha, int nt) {
  (void)alpha;  // unused by the reference too (yael/vlad.c:124-139)
  (void)nt;
  if (bof_run(k, d, centroids, n, v, ma, 0, nullptr, nullptr, desc, nullptr) != OK)
    fatal_last("bof_compute_ma");
}

void bof_compute_subsets(int k, int d, const float *centroids, int n, const float *v,
                         int n_subset, const int *subset_indexes, const int *subset_ends,
                         float *desc) {
  if (bof_run(k, d, centroids, n, v, 1, n_subset, subset_indexes, subset_ends, nullptr, desc) != OK)
    fatal_last("bof_compute_subsets");
}

}  // extern "C"
