// K-means LSH (yael/kmlsh.c): nhash k-means partitions ("hash functions") of
// the space; a query's neighbours are searched exactly among the base vectors
// of its cell in each partition, and the per-partition lists are merged into
// one list of k per query.
//
// The GPU does the work that scales: each partition's clustering is the
// drop-in kmeans, each cell assignment one k = 1 search over all the vectors,
// and all the per-cell searches of a partition one batched k-NN call
// (yael_gpu_knn_batch) over the occupied cells, whose rows are uploaded once,
// cell after cell.  With the BF16 precision and k >= 9 that call is the grouped
// persistent pass, otherwise the concurrent per-cell pool.  Sampling, cell
// ordering and the merge are host code that follows the reference step for
// step, so every list comes out in the reference's order.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "../../include/yael_gpu.h"
#include "common.cuh"

namespace {

[[noreturn]] void die(const char *where, const char *what) {
  yg::set_error(yg::E_ARG, "%s", what);
  yg::fatal_last(where);
}

void check_type(const char *where, int vec_type) {
  if (vec_type != YAEL_KMLSH_VECTYPE_FVEC && vec_type != YAEL_KMLSH_VECTYPE_BVEC)
    die(where, "vec_type must be KMLSH_VECTYPE_FVEC or KMLSH_VECTYPE_BVEC");
}

// ivec_new_random_idx (yael/vector.c:221-243): the first k entries of a
// partial Fisher-Yates shuffle of 0..n-1, rand_r seeded by one lrand48()
std::vector<int> random_idx(int n, int k) {
  unsigned int seed = (unsigned int)lrand48();
  std::vector<int> idx(n > 0 ? n : 1);
  for (int i = 0; i < n; i++) idx[i] = i;
  for (int i = 0; i < k; i++) {
    const int j = i + rand_r(&seed) % (n - i);
    std::swap(idx[i], idx[j]);
  }
  return idx;
}

// rows idx[0..m) of v (floats, or bytes cast to float) into out (m x d):
// fvec_cpy_subvectors / b2fvec_cpy_subvectors (yael/vector.c:2478-2497)
void gather_rows(const void *v, int vec_type, const int *idx, long m, int d, float *out) {
  if (vec_type == YAEL_KMLSH_VECTYPE_FVEC) {
    const float *vf = (const float *)v;
    for (long i = 0; i < m; i++)
      memcpy(out + i * d, vf + (long)idx[i] * d, sizeof(float) * (size_t)d);
  } else {
    const unsigned char *vb = (const unsigned char *)v;
    for (long i = 0; i < m; i++)
      for (int j = 0; j < d; j++) out[i * d + j] = vb[(long)idx[i] * d + j];
  }
}

long round_up(long x, long a) { return (x + a - 1) / a * a; }

// nnlist_add (yael/kmlsh.c:60-84): slot 0 holds the largest distance of the
// list; a new (id, distance) not above it and not already listed replaces it,
// then the new largest is swapped into slot 0 (the first one on ties).
void nnlist_add(nnlist_t *l, int lno, int elidx, float eldis) {
  int *idx = l->idx + (long)lno * l->k;
  float *dis = l->dis + (long)lno * l->k;
  if (eldis > dis[0]) return;
  for (long i = 0; i < l->k; i++)
    if (idx[i] == elidx) return;
  idx[0] = elidx;
  dis[0] = eldis;
  long posmax = 0;  // fvec_arg_max (yael/sorting.c:764-775)
  float m = dis[0];
  for (long i = 1; i < l->k; i++)
    if (dis[i] > m) {
      m = dis[i];
      posmax = i;
    }
  if (posmax == 0) return;
  idx[0] = idx[posmax];
  dis[0] = dis[posmax];
  idx[posmax] = elidx;
  dis[posmax] = eldis;
}

// exact k-NN of every occupied cell of one partition: cells[] gives each
// cell's base / query counts, the rows' positions in the gathered arrays
// and its outputs' position; one batched call per distinct k2
struct Cell {
  int c, nb, nq, k2;
  long boff, qoff, ooff;
};

void cuda_ok(const char *where, cudaError_t e) {
  if (e != cudaSuccess) {
    yg::set_error(yg::E_CUDA, "%s", cudaGetErrorString(e));
    yg::fatal_last(where);
  }
}

void search_cells(const std::vector<Cell> &cells, int d, const float *hb, long bt,
                  const float *hq, long qt, int *hi, float *hd, long ot) {
  const char *where = "kmlsh_match_xvec";
  yg::DevArray<float> db, dq, dd;
  yg::DevArray<int> di;
  db.get(where, bt);
  dq.get(where, qt);
  di.get(where, ot);
  dd.get(where, ot);
  cuda_ok(where, cudaMemcpy(db.p, hb, sizeof(float) * (size_t)bt, cudaMemcpyHostToDevice));
  cuda_ok(where, cudaMemcpy(dq.p, hq, sizeof(float) * (size_t)qt, cudaMemcpyHostToDevice));
  std::vector<int> ks;
  for (const Cell &x : cells) ks.push_back(x.k2);
  std::sort(ks.begin(), ks.end());
  ks.erase(std::unique(ks.begin(), ks.end()), ks.end());
  std::vector<yael_gpu_knn_pair> pairs;
  for (int k2 : ks) {
    pairs.clear();
    for (const Cell &x : cells)
      if (x.k2 == k2)
        pairs.push_back({x.nq, x.nb, dq.p + x.qoff, db.p + x.boff, di.p + x.ooff, dd.p + x.ooff});
    yael_gpu_knn_opts o;
    memset(&o, 0, sizeof(o));
    o.precision = YAEL_GPU_PREC_ENV;
    o.metric = 2;
    o.device_ptrs = 1;
    if (yael_gpu_knn_batch((int)pairs.size(), pairs.data(), d, k2, &o) != 0)
      yg::fatal_last(where);
  }
  cuda_ok(where, cudaMemcpy(hi, di.p, sizeof(int) * (size_t)ot, cudaMemcpyDeviceToHost));
  cuda_ok(where, cudaMemcpy(hd, dd.p, sizeof(float) * (size_t)ot, cudaMemcpyDeviceToHost));
}

}  // namespace

extern "C" {

nnlist_t *nnlist_new_noalloc(int n, int k) {
  nnlist_t *l = (nnlist_t *)malloc(sizeof(nnlist_t));
  l->n = n;
  l->k = k;
  l->idx = nullptr;
  l->dis = nullptr;
  return l;
}

nnlist_t *nnlist_new(int n, int k) {
  nnlist_t *l = nnlist_new_noalloc(n, k);
  const long nk = (long)n * k;
  l->idx = (int *)malloc(sizeof(int) * (size_t)(nk > 0 ? nk : 1));
  l->dis = (float *)malloc(sizeof(float) * (size_t)(nk > 0 ? nk : 1));
  for (long i = 0; i < nk; i++) {
    l->idx[i] = -1;
    l->dis[i] = 1e30f;
  }
  return l;
}

void nnlist_delete(nnlist_t *l) {
  free(l->dis);
  free(l->idx);
  free(l);
}

void nnlist_addn(nnlist_t *l, int lno, int n, int *idx, float *dis) {
  for (int i = 0; i < n; i++) nnlist_add(l, lno, idx[i], dis[i]);
}

kmlsh_t *kmlsh_new(int nhash, int nclust, int d) {
  kmlsh_t *lsh = (kmlsh_t *)malloc(sizeof(kmlsh_t));
  lsh->d = d;
  lsh->nhash = nhash;
  lsh->nclust = nclust;
  lsh->centroids = (float **)malloc(sizeof(float *) * (size_t)(nhash > 0 ? nhash : 1));
  for (int h = 0; h < nhash; h++)
    lsh->centroids[h] = (float *)malloc(sizeof(float) * (size_t)((long)d * nclust + 1));
  return lsh;
}

void kmlsh_delete(kmlsh_t *lsh) {
  for (int h = 0; h < lsh->nhash; h++) free(lsh->centroids[h]);
  free(lsh->centroids);
  free(lsh);
}

void kmlsh_learn_xvec(kmlsh_t *lsh, int n, int nlearn, const void *v, int flags,
                      int vec_type) {
  check_type("kmlsh_learn_xvec", vec_type);
  const int d = lsh->d, nclust = lsh->nclust;
  int kmeans_flags = (flags & YAEL_KMLSH_NT) | YAEL_KMEANS_INIT_RANDOM;
  const bool verbose = !(flags & YAEL_KMLSH_QUIET);
  if (nlearn == 0) {
    nlearn = nclust * 50;
    if (nlearn > n) nlearn = (n * 3) / 4;
  }
  if (nlearn > n) die("kmlsh_learn_xvec", "nlearn > n");
  if (verbose)
    fprintf(stderr, "n=%d  nlearn=%d  nclust=%d\n", n, nlearn, nclust);
  else
    kmeans_flags |= YAEL_KMEANS_QUIET;
  std::vector<float> vlearn((size_t)nlearn * d + 1);
  for (int h = 0; h < lsh->nhash; h++) {
    const std::vector<int> perm = random_idx(n, nlearn);
    gather_rows(v, vec_type, perm.data(), nlearn, d, vlearn.data());
    if (verbose) fprintf(stderr, "Learn K-means using %d vectors\n", nlearn);
    kmeans(d, nlearn, nclust, YAEL_KMLSH_NB_ITER_MAX, vlearn.data(), kmeans_flags, 0, 1,
           lsh->centroids[h], nullptr, nullptr, nullptr);
    if (flags & YAEL_KMLSH_WRITE_INTER_NHASH) {
      char name[256];
      snprintf(name, sizeof(name), "tmp/nhash-intermediate_%d.kmlsh", h + 1);
      kmlsh_write(name, lsh);
    }
  }
}

kmlsh_t *kmlsh_new_learn_bvec(int nhash, int nclust, int d, int n, int nlearn,
                              const unsigned char *v, int flags) {
  kmlsh_t *lsh = kmlsh_new(nhash, nclust, d);
  kmlsh_learn_xvec(lsh, n, nlearn, v, flags, YAEL_KMLSH_VECTYPE_BVEC);
  return lsh;
}

kmlsh_t *kmlsh_new_learn_fvec(int nhash, int nclust, int d, int n, int nlearn,
                              const float *v, int flags) {
  kmlsh_t *lsh = kmlsh_new(nhash, nclust, d);
  kmlsh_learn_xvec(lsh, n, nlearn, v, flags, YAEL_KMLSH_VECTYPE_FVEC);
  return lsh;
}

void kmeans_cohash_xvec(const kmlsh_t *lsh, int h, const void *v, int n, int *perm,
                        int *boundaries, int flags, int vec_type) {
  check_type("kmeans_cohash_xvec", vec_type);
  const int d = lsh->d, nclust = lsh->nclust;
  std::vector<int> idx(n > 0 ? n : 1);
  std::vector<float> dis(n > 0 ? n : 1);
  // the nearest centroid of every vector: one k = 1 search (the reference
  // searches blocks of 256 vectors; each vector's result is its own)
  if (vec_type == YAEL_KMLSH_VECTYPE_FVEC) {
    if (n > 0)
      knn_full(2, n, nclust, d, 1, lsh->centroids[h], (const float *)v, nullptr, idx.data(),
               dis.data());
  } else {
    const long block = 1L << 18;
    std::vector<float> buf((size_t)std::min<long>(block, n > 0 ? n : 1) * d);
    const unsigned char *vb = (const unsigned char *)v;
    for (long i0 = 0; i0 < n; i0 += block) {
      const long m = std::min<long>(block, n - i0);
      for (long j = 0; j < m * d; j++) buf[j] = vb[i0 * d + j];
      knn_full(2, (int)m, nclust, d, 1, lsh->centroids[h], buf.data(), nullptr,
               idx.data() + i0, dis.data() + i0);
    }
  }
  if (!(flags & YAEL_KMLSH_QUIET)) {
    if (n > 0) fprintf(stdout, "\rQuantize %d descriptors. %6.2f%%", n, 100.0);
    printf("\n");
  }
  // cells' starts (exclusive prefix sums of the cell counts), then the
  // vector ids in increasing order within each cell (yael/kmlsh.c:252-273)
  std::vector<int> start(nclust + 1, 0), nocc(nclust > 0 ? nclust : 1, 0);
  for (long i = 0; i < n; i++) {
    if (idx[i] < 0 || idx[i] >= nclust) die("kmeans_cohash_xvec", "vector without a cell");
    start[idx[i] + 1]++;
  }
  for (int c = 0; c < nclust; c++) start[c + 1] += start[c];
  for (long i = 0; i < n; i++) {
    const int cell = idx[i];
    perm[start[cell] + nocc[cell]++] = (int)i;
  }
  memcpy(boundaries, start.data(), sizeof(int) * (size_t)(nclust + 1));
}

void kmeans_cohash_bvec(const kmlsh_t *lsh, int h, const unsigned char *v, int n, int *perm,
                        int *boundaries, int flags) {
  kmeans_cohash_xvec(lsh, h, v, n, perm, boundaries, flags, YAEL_KMLSH_VECTYPE_BVEC);
}

void kmeans_cohash_fvec(const kmlsh_t *lsh, int h, const float *v, int n, int *perm,
                        int *boundaries, int flags) {
  kmeans_cohash_xvec(lsh, h, v, n, perm, boundaries, flags, YAEL_KMLSH_VECTYPE_FVEC);
}

kmlsh_idx_t *kmlsh_idx_new(const kmlsh_t *lsh, int n) {
  kmlsh_idx_t *x = (kmlsh_idx_t *)malloc(sizeof(kmlsh_idx_t));
  x->nhash = lsh->nhash;
  x->n = n;
  x->nclust = lsh->nclust;
  x->perm = (int *)malloc(sizeof(int) * (size_t)((long)lsh->nhash * n + 1));
  x->boundaries = (int *)malloc(sizeof(int) * (size_t)((long)lsh->nhash * (lsh->nclust + 1)));
  return x;
}

void kmlsh_idx_delete(kmlsh_idx_t *lshidx) {
  free(lshidx->perm);
  free(lshidx->boundaries);
  free(lshidx);
}

kmlsh_idx_t *kmlsh_idx_new_compile_xvec(const kmlsh_t *lsh, const void *v, int n, int flags,
                                        int vec_type) {
  kmlsh_idx_t *x = kmlsh_idx_new(lsh, n);
  const int nt = flags & YAEL_KMLSH_NT;
  for (int h = 0; h < lsh->nhash; h++) {
    // the thread count alone is passed on: the assignment reports progress
    kmeans_cohash_xvec(lsh, h, v, n, x->perm + (long)h * n,
                       x->boundaries + (long)h * (lsh->nclust + 1), nt, vec_type);
    if (flags & YAEL_KMLSH_WRITE_INTER_NHASH) {
      char name[256];
      snprintf(name, sizeof(name), "tmp/nhash-intermediate_%d.kmlshidx", h + 1);
      kmlsh_idx_write(name, x);
    }
  }
  return x;
}

kmlsh_idx_t *kmlsh_idx_new_compile_bvec(const kmlsh_t *lsh, const unsigned char *v, int n,
                                        int flags) {
  return kmlsh_idx_new_compile_xvec(lsh, v, n, flags, YAEL_KMLSH_VECTYPE_BVEC);
}

kmlsh_idx_t *kmlsh_idx_new_compile_fvec(const kmlsh_t *lsh, const float *v, int n, int flags) {
  return kmlsh_idx_new_compile_xvec(lsh, v, n, flags, YAEL_KMLSH_VECTYPE_FVEC);
}

int kmlsh_idx_get_nvec(const kmlsh_idx_t *lshidx, int h, int c) {
  const int *b = lshidx->boundaries + (long)h * (lshidx->nclust + 1);
  return b[c + 1] - b[c];
}

int kmlsh_idx_get_maxincell(const kmlsh_idx_t *lshidx, int h) {
  int m = 0;
  for (int c = 0; c < lshidx->nclust; c++) m = std::max(m, kmlsh_idx_get_nvec(lshidx, h, c));
  return m;
}

int *kmlsh_idx_get_vecids(const kmlsh_idx_t *lshidx, int h, int c) {
  return lshidx->perm + (long)lshidx->n * h +
         lshidx->boundaries[(long)h * (lshidx->nclust + 1) + c];
}

nnlist_t *kmlsh_match_xvec(const kmlsh_t *lsh, const kmlsh_idx_t *lshidx_b, const void *vb,
                           int nb, const kmlsh_idx_t *lshidx_q, const void *vq, int nq, int k,
                           int nt, int vec_type) {
  (void)nt;
  check_type("kmlsh_match_xvec", vec_type);
  const int d = lsh->d, nclust = lsh->nclust;
  nnlist_t *nnlist = nnlist_new(nq, k);
  for (int h = 0; h < lsh->nhash; h++) {
    const long maxb = kmlsh_idx_get_maxincell(lshidx_b, h);
    const long maxq = kmlsh_idx_get_maxincell(lshidx_q, h);
    printf("max in histo: base=%ld  query=%ld  (nclust=%d, nb=%d, nq=%d)\n", maxb, maxq,
           nclust, nb, nq);
    printf("Group the vectors based on cell %d / %d, then exact search\n", h + 1, lsh->nhash);
    // the cells holding both base vectors and queries; each slice starts on a
    // 256-byte boundary, as a separate allocation would
    std::vector<Cell> cells;
    long bt = 0, qt = 0, ot = 0;
    for (int c = 0; c < nclust; c++) {
      const int nbc = kmlsh_idx_get_nvec(lshidx_b, h, c);
      const int nqc = kmlsh_idx_get_nvec(lshidx_q, h, c);
      if (nqc == 0 || nbc == 0) continue;
      const Cell x{c, nbc, nqc, std::min(k, nbc), bt, qt, ot};
      bt += round_up((long)nbc * d, 64);
      qt += round_up((long)nqc * d, 64);
      ot += round_up((long)nqc * x.k2, 64);
      cells.push_back(x);
    }
    if (cells.empty()) continue;
    std::vector<float> hb((size_t)bt), hq((size_t)qt), hd((size_t)ot);
    std::vector<int> hi((size_t)ot);
    for (const Cell &x : cells) {
      gather_rows(vb, vec_type, kmlsh_idx_get_vecids(lshidx_b, h, x.c), x.nb, d,
                  hb.data() + x.boff);
      gather_rows(vq, vec_type, kmlsh_idx_get_vecids(lshidx_q, h, x.c), x.nq, d,
                  hq.data() + x.qoff);
    }
    search_cells(cells, d, hb.data(), bt, hq.data(), qt, hi.data(), hd.data(), ot);
    // merge in the reference's order: cells ascending, queries in cell order
    for (const Cell &x : cells) {
      const int *vidx_b = kmlsh_idx_get_vecids(lshidx_b, h, x.c);
      const int *vidx_q = kmlsh_idx_get_vecids(lshidx_q, h, x.c);
      int *ids = hi.data() + x.ooff;
      float *ds = hd.data() + x.ooff;
      for (long i = 0; i < (long)x.nq * x.k2; i++) ids[i] = ids[i] >= 0 ? vidx_b[ids[i]] : -1;
      for (int i = 0; i < x.nq; i++)
        nnlist_addn(nnlist, vidx_q[i], x.k2, ids + (long)i * x.k2, ds + (long)i * x.k2);
    }
  }
  return nnlist;
}

nnlist_t *kmlsh_match_bvec(const kmlsh_t *lsh, const kmlsh_idx_t *lshidx_b,
                           const unsigned char *vb, int nb, const kmlsh_idx_t *lshidx_q,
                           const unsigned char *vq, int nq, int k, int nt) {
  return kmlsh_match_xvec(lsh, lshidx_b, vb, nb, lshidx_q, vq, nq, k, nt,
                          YAEL_KMLSH_VECTYPE_BVEC);
}

nnlist_t *kmlsh_match_fvec(const kmlsh_t *lsh, const kmlsh_idx_t *lshidx_b, const float *vb,
                           int nb, const kmlsh_idx_t *lshidx_q, const float *vq, int nq, int k,
                           int nt) {
  return kmlsh_match_xvec(lsh, lshidx_b, vb, nb, lshidx_q, vq, nq, k, nt,
                          YAEL_KMLSH_VECTYPE_FVEC);
}

nnlist_t *kmlsh_ann_xvec(const void *vb, int nb, const void *vq, int nq, int d, int k,
                         int nhash, int flags, int vec_type) {
  const int nclust = (int)sqrt((double)nb);
  int nlearn = nclust * 100;
  if (nlearn > nb) {
    fprintf(stderr, "Warning: should use more vector in learning set\n");
    nlearn = nb;
  }
  kmlsh_t *lsh = kmlsh_new(nhash, nclust, d);
  kmlsh_learn_xvec(lsh, nb, nlearn, vb, flags, vec_type);
  kmlsh_idx_t *lshidx_b = kmlsh_idx_new_compile_xvec(lsh, vb, nb, flags, vec_type);
  kmlsh_idx_t *lshidx_q = kmlsh_idx_new_compile_xvec(lsh, vq, nq, flags, vec_type);
  nnlist_t *nnlist =
      kmlsh_match_xvec(lsh, lshidx_b, vb, nb, lshidx_q, vq, nq, k, flags, vec_type);
  kmlsh_delete(lsh);
  kmlsh_idx_delete(lshidx_b);
  kmlsh_idx_delete(lshidx_q);
  return nnlist;
}

nnlist_t *kmlsh_ann_bvec(const unsigned char *vb, int nb, const unsigned char *vq, int nq,
                         int d, int k, int nhash, int flags) {
  return kmlsh_ann_xvec(vb, nb, vq, nq, d, k, nhash, flags, YAEL_KMLSH_VECTYPE_BVEC);
}

nnlist_t *kmlsh_ann_fvec(const float *vb, int nb, const float *vq, int nq, int d, int k,
                         int nhash, int flags) {
  return kmlsh_ann_xvec(vb, nb, vq, nq, d, k, nhash, flags, YAEL_KMLSH_VECTYPE_FVEC);
}

// I/O (yael/kmlsh.c:526-611): a partition is one .fvecs record of nclust * d
// floats; an index one .ivecs record of the ids then one of the nclust + 1
// cell starts per partition.  An I/O error prints and exits(1).
static void io_fail(const char *who, const char *filename) {
  fprintf(stderr, "# %s: I/O error with file %s\n", who, filename);
  exit(1);
}

void kmlsh_write(const char *filename, const kmlsh_t *lsh) {
  FILE *f = fopen(filename, "w");
  if (!f) io_fail("kmlsh_write", filename);
  for (int h = 0; h < lsh->nhash; h++)
    if (fvec_fwrite(f, lsh->centroids[h], lsh->nclust * lsh->d) != 0)
      io_fail("kmlsh_write", filename);
  fclose(f);
}

void kmlsh_read(const char *filename, const kmlsh_t *lsh) {
  FILE *f = fopen(filename, "r");
  if (!f) io_fail("kmlsh_read", filename);
  for (int h = 0; h < lsh->nhash; h++) {
    // a fresh array per partition, as the reference does
    lsh->centroids[h] = (float *)malloc(sizeof(float) * (size_t)((long)lsh->d * lsh->nclust + 1));
    if (fvec_fread(f, lsh->centroids[h], lsh->d * lsh->nclust) != lsh->nclust * lsh->d)
      io_fail("kmlsh_read", filename);
  }
  fclose(f);
}

void kmlsh_idx_write(const char *filename, const kmlsh_idx_t *lshidx) {
  FILE *f = fopen(filename, "w");
  if (!f) io_fail("kmlsh_idx_write", filename);
  for (long h = 0; h < lshidx->nhash; h++) {
    if (ivec_fwrite(f, lshidx->perm + h * lshidx->n, lshidx->n) != 0)
      io_fail("kmlsh_idx_write", filename);
    if (ivec_fwrite(f, lshidx->boundaries + h * (lshidx->nclust + 1), lshidx->nclust + 1) != 0)
      io_fail("kmlsh_idx_write", filename);
  }
  fclose(f);
}

void kmlsh_idx_read(const char *filename, kmlsh_idx_t *lshidx) {
  FILE *f = fopen(filename, "r");
  if (!f) io_fail("kmlsh_idx_read", filename);
  for (long h = 0; h < lshidx->nhash; h++) {
    if (ivec_fread(f, lshidx->perm + h * lshidx->n, lshidx->n) != lshidx->n)
      io_fail("kmlsh_idx_read", filename);
    if (ivec_fread(f, lshidx->boundaries + h * (lshidx->nclust + 1), lshidx->nclust + 1) !=
        lshidx->nclust + 1)
      io_fail("kmlsh_idx_read", filename);
  }
  fclose(f);
}

}  // extern "C"
