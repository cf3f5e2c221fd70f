/*
 * yael_oracle.c -- TEST INFRASTRUCTURE ONLY (the checker, never the product).
 *
 * CPU restatement of yael's distance-GEMM path.  See yael_oracle.h for the two
 * arithmetic modes.  Every function names the reference lines it restates
 * (paths relative to the reference project).  Written from the reference's
 * documented behaviour; the heap, RNG and update orders are kept step-for-step
 * alike because the reference's results (tie order, random streams) depend on
 * them.
 */
#define _GNU_SOURCE
#include "yael_oracle.h"

#include <assert.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

int sgemv_(const char *trans, const int *m, const int *n, const float *alpha,
           const float *a, const int *lda, const float *x, const int *incx,
           const float *beta, float *y, const int *incy);
int sgemm_(const char *ta, const char *tb, const int *m, const int *n,
           const int *k, const float *alpha, const float *a, const int *lda,
           const float *b, const int *ldb, const float *beta, float *c,
           const int *ldc);

#define TILE 256 /* yael/nn.c:371-372 BLOCK_N1 / BLOCK_N2 */

/* ------------------------------------------------------------------ */
/* bounded max-heap with yael's tie behaviour (yael/binheap.c:11-211)  */

typedef struct {
  int cnt, cap;
  float *val; /* 1-based */
  int *lab;   /* 1-based */
} oheap;

static void oheap_push(oheap *h, int lab, float v)
{
  /* sift up, stopping as soon as the parent is >= v (yael/binheap.c:89-103) */
  int i = ++h->cnt;
  while (i > 1) {
    int f = i >> 1;
    if (h->val[f] >= v) break;
    h->val[i] = h->val[f];
    h->lab[i] = h->lab[f];
    i = f;
  }
  h->val[i] = v;
  h->lab[i] = lab;
}

static void oheap_pop(oheap *h)
{
  /* remove the root; the last element sinks from the root.  The child test
   * counts the not-yet-removed last slot (yael/binheap.c:55-86). */
  float last = h->val[h->cnt];
  int i = 1;
  for (;;) {
    int l = i << 1, r = l + 1, c;
    if (l > h->cnt) break;
    if (r == h->cnt + 1 || h->val[l] > h->val[r]) c = l; else c = r;
    if (last > h->val[c]) break;
    h->val[i] = h->val[c];
    h->lab[i] = h->lab[c];
    i = c;
  }
  h->val[i] = h->val[h->cnt];
  h->lab[i] = h->lab[h->cnt];
  h->cnt--;
}

/* fill with the first non-NaN values, then replace the root only on a strict
 * improvement (yael/binheap.c:139-156) */
static void oheap_add_range(oheap *h, int n, int label0, const float *v)
{
  int i = 0;
  for (; i < n && h->cnt < h->cap; i++)
    if (!isnan(v[i])) oheap_push(h, label0 + i, v[i]);
  if (i >= n) return;
  float lim = h->val[1];
  for (; i < n; i++)
    if (v[i] < lim) {
      oheap_pop(h);
      oheap_push(h, label0 + i, v[i]);
      lim = h->val[1];
    }
}

/* sort by (value, heap slot) -- fvec_sort_index semantics (yael/sorting.c:286-317) */
static int cmp_slot(const void *a, const void *b, void *ctx)
{
  const float *key = (const float *)ctx;
  int ia = *(const int *)a, ib = *(const int *)b;
  float dt = key[ia] - key[ib];
  if (dt) return dt > 0 ? 1 : -1;
  return ia - ib;
}

static void sort_index_f(const float *key, int n, int *perm)
{
  for (int i = 0; i < n; i++) perm[i] = i;
  qsort_r(perm, n, sizeof(int), cmp_slot, (void *)key);
}

static void oheap_sort_out(oheap *h, int *lab_out, float *val_out)
{
  int *perm = malloc(sizeof(int) * (h->cnt + 1));
  sort_index_f(h->val + 1, h->cnt, perm);
  for (int i = 0; i < h->cnt; i++) {
    int p = perm[i] + 1;
    lab_out[i] = h->lab[p];
    val_out[i] = h->val[p];
  }
  free(perm);
}

/* ------------------------------------------------------------------ */
/* expanded-form distances (yael/nn.c:54-67, 100-129, 266-275)         */

void orc_cross_distances_port(int d, int na, int nb, const float *a, int lda,
                              const float *b, int ldb, float *dist2, int ldd)
{
  float *sa = malloc(sizeof(float) * (na > 0 ? na : 1));
  for (long i = 0; i < na; i++) { /* float accumulation for a */
    float s = 0;
    const float *x = a + (long)lda * i;
    for (long j = 0; j < d; j++) s += x[j] * x[j];
    sa[i] = s;
  }
  for (long i = 0; i < nb; i++) { /* double accumulation for b, rounded on store */
    double s = 0;
    const float *x = b + (long)ldb * i;
    for (long j = 0; j < d; j++) s += x[j] * x[j];
    float *row = dist2 + i * (long)ldd;
    for (long j = 0; j < na; j++) row[j] = s + sa[j];
  }
  float m2 = -2, one = 1;
  sgemm_("Transposed", "Not trans", &na, &nb, &d, &m2, a, &lda, b, &ldb, &one,
         dist2, &ldd);
  free(sa);
}

static void dot_products_port(int d, int na, int nb, const float *a, const float *b,
                              float *dist2)
{
  float one = 1, zero = 0;
  sgemm_("Trans", "Not", &na, &nb, &d, &one, a, &d, b, &d, &zero, dist2, &na);
}

/* the SSE2 forms of yael/nn.c:172-210 (used when d % 4 == 0 in builds with
 * SSE2): four float lanes, lane l adding the terms of coordinates l, l+4, ...,
 * then lane0 + lane1 + lane2 + lane3; chi2 terms where the coordinates differ */
static float alt_lanes(int dt, const float *a, const float *b, int d)
{
  float acc[4] = {0, 0, 0, 0};
  for (int i = 0; i < d; i += 4)
    for (int l = 0; l < 4; l++) {
      float ai = a[i + l], bi = b[i + l];
      float diff = ai - bi;
      if (dt == 1) {
        acc[l] += fabsf(diff);
      } else if (ai != bi) {
        float sum = ai + bi;
        acc[l] += (diff * diff) / sum;
      }
    }
  return acc[0] + acc[1] + acc[2] + acc[3];
}

/* compute_cross_distances_alt_nonpacked (yael/nn.c:280-350):
 * dist2[i + ldd*j] = distance(a_i, b_j) */
void orc_cross_distances_alt(int dt, int d, int na, int nb, const float *a, int lda,
                             const float *b, int ldb, float *dist2, int ldd)
{
#ifdef __SSE2__
  if (d % 4 == 0 && (dt == 1 || dt == 3)) {
    for (long j = 0; j < nb; j++)
      for (long i = 0; i < na; i++)
        dist2[j * ldd + i] = alt_lanes(dt, a + i * lda, b + j * ldb, d);
    return;
  }
#endif
  if (dt == 12) {
    orc_cross_distances_port(d, na, nb, a, lda, b, ldb, dist2, ldd);
    return;
  }
  if (dt == 16) {
    float one = 1, zero = 0;
    sgemm_("Trans", "Not", &na, &nb, &d, &one, a, &lda, b, &ldb, &zero, dist2, &ldd);
    return;
  }
  for (long j = 0; j < nb; j++) {
    const float *bl = b + (long)ldb * j;
    for (long i = 0; i < na; i++) {
      const float *al = a + (long)lda * i;
      double sum = 0;
      for (int c = 0; c < d; c++) {
        float av = al[c], bv = bl[c];
        if (dt == 1) {
          sum += fabs(av - bv);
        } else if (dt == 2) {
          double t = av - bv;
          sum += t * t;
        } else if (dt == 3) {
          double t = av - bv;
          sum += av + bv == 0 ? 0 : t * t / (av + bv);
        } else if (dt == 4) {
          float den = fabs(av + bv);
          double t = av - bv;
          sum += den == 0 ? 0 : t * t / den;
        } else if (dt == 5) {
          sum += av < bv ? av : bv;
        } else if (dt == 6) {
          sum += av * bv;
        } else {
          fprintf(stderr, "oracle: distance_type %d not restated\n", dt);
          abort();
        }
      }
      dist2[j * ldd + i] = (float)sum;
    }
  }
}

static void tile_distances(int dt, int d, int na, int nb, const float *a,
                           const float *b, float *out)
{
  /* knn_full / nn_single_full (yael/nn.c:414-417, 491-496): type 2 through
   * compute_cross_distances, every other through the _alt dispatch */
  if (dt == 2 || dt == 12)
    orc_cross_distances_port(d, na, nb, a, d, b, d, out, na);
  else if (dt == 16)
    dot_products_port(d, na, nb, a, b, out);
  else
    orc_cross_distances_alt(dt, d, na, nb, a, d, b, d, out, na);
}

/* nn_single_full (yael/nn.c:383-446): blocked argmin, strict '<' */
static void nn_single_port(int dt, int n1, int n2, int d, const float *b,
                           const float *q, const float *w, int *vw, float *vwdis)
{
  int s1 = n1 < TILE ? n1 : TILE, s2 = n2 < TILE ? n2 : TILE;
  float *dists = malloc(sizeof(float) * (size_t)(s1 > 0 ? s1 : 1) * (s2 > 0 ? s2 : 1));
  for (long i1 = 0; i1 < n1; i1 += s1) {
    int m1 = n1 - i1 < s1 ? n1 - i1 : s1;
    for (long j = 0; j < m1; j++) { vw[i1 + j] = -1; vwdis[i1 + j] = 1e30f; }
    for (long i2 = 0; i2 < n2; i2 += s2) {
      int m2 = n2 - i2 < s2 ? n2 - i2 : s2;
      tile_distances(dt, d, m2, m1, b + i2 * d, q + i1 * d, dists);
      if (w)
        for (long j1 = 0; j1 < m1; j1++)
          for (long j2 = 0; j2 < m2; j2++) dists[j1 * m2 + j2] *= w[j2 + i2];
      for (long j1 = 0; j1 < m1; j1++) {
        const float *row = dists + j1 * m2;
        int im = vw[i1 + j1];
        float dm = vwdis[i1 + j1];
        for (long j2 = 0; j2 < m2; j2++)
          if (row[j2] < dm) { im = j2 + i2; dm = row[j2]; }
        vw[i1 + j1] = im;
        vwdis[i1 + j1] = dm;
      }
    }
  }
  free(dists);
}

/* knn_full (yael/nn.c:451-525) */
static void knn_full_port(int dt, int n1, int n2, int d, int k, const float *b,
                          const float *q, const float *w, int *vw, float *vwdis)
{
  assert(k <= n2);
  if (k == 1) { nn_single_port(dt, n1, n2, d, b, q, w, vw, vwdis); return; }
  int s1 = n1 < TILE ? n1 : TILE, s2 = n2 < TILE ? n2 : TILE;
  if (s1 <= 0) return;
  float *dists = malloc(sizeof(float) * (size_t)s1 * s2);
  oheap *hs = malloc(sizeof(oheap) * s1);
  float *hv = malloc(sizeof(float) * (size_t)s1 * (k + 1));
  int *hl = malloc(sizeof(int) * (size_t)s1 * (k + 1));
  for (int j = 0; j < s1; j++) {
    hs[j].cap = k;
    hs[j].val = hv + (size_t)j * (k + 1);
    hs[j].lab = hl + (size_t)j * (k + 1);
  }
  for (long i1 = 0; i1 < n1; i1 += s1) {
    int m1 = n1 - i1 < s1 ? n1 - i1 : s1;
    for (int j = 0; j < m1; j++) hs[j].cnt = 0;
    for (long i2 = 0; i2 < n2; i2 += s2) {
      int m2 = n2 - i2 < s2 ? n2 - i2 : s2;
      tile_distances(dt, d, m2, m1, b + i2 * d, q + i1 * d, dists);
      if (w)
        for (long j1 = 0; j1 < m1; j1++)
          for (long j2 = 0; j2 < m2; j2++) dists[j1 * m2 + j2] *= w[j2 + i2];
      for (long j1 = 0; j1 < m1; j1++)
        oheap_add_range(&hs[j1], m2, (int)i2, dists + j1 * m2);
    }
    for (long j1 = 0; j1 < m1; j1++) {
      oheap *h = &hs[j1];
      oheap_sort_out(h, vw + (i1 + j1) * k, vwdis + (i1 + j1) * k);
      if (h->cnt < k) { /* NaN-short heaps: -1 ids, all-ones distance bits (nn.c:515-518) */
        memset(vw + (i1 + j1) * k + h->cnt, 0xff, sizeof(int) * (k - h->cnt));
        memset(vwdis + (i1 + j1) * k + h->cnt, 0xff, sizeof(float) * (k - h->cnt));
      }
    }
  }
  free(dists); free(hs); free(hv); free(hl);
}

/* knn_full_thread (yael/nn.c:665-699): nt contiguous query slices */
void orc_knn_port(int dt, int nq, int nb, int d, int k, const float *b,
                  const float *q, const float *w, int *assign, float *dis, int nt)
{
  if (nq < nt || nt <= 1) { knn_full_port(dt, nq, nb, d, k, b, q, w, assign, dis); return; }
#pragma omp parallel for schedule(dynamic) num_threads(nt)
  for (int i = 0; i < nt; i++) {
    long n0 = (long)nq * i / nt, n1 = (long)nq * (i + 1) / nt;
    knn_full_port(dt, (int)(n1 - n0), nb, d, k, b, q + n0 * d, w, assign + n0 * k,
                  dis + n0 * k);
  }
}

/* ------------------------------------------------------------------ */
/* FP64 brute force (distance form of yael/vector.c:2348-2358)          */

static double dist64(const float *x, const float *y, int d)
{
  double s = 0;
  for (int i = 0; i < d; i++) { double a = (double)x[i] - (double)y[i]; s += a * a; }
  return s;
}

/* lexicographic (distance, id) max-heap, 0-based */
static int lex_gt(double da, int ia, double db, int ib)
{
  return da > db || (da == db && ia > ib);
}

static void lexheap_sift_down(double *v, int *id, int n, int i)
{
  for (;;) {
    int l = 2 * i + 1, r = l + 1, m = i;
    if (l < n && lex_gt(v[l], id[l], v[m], id[m])) m = l;
    if (r < n && lex_gt(v[r], id[r], v[m], id[m])) m = r;
    if (m == i) return;
    double tv = v[i]; v[i] = v[m]; v[m] = tv;
    int ti = id[i]; id[i] = id[m]; id[m] = ti;
    i = m;
  }
}

void orc_knn_exact(int nq, int nb, int d, int k, const float *b, const float *q,
                   int *assign, float *dis, double *dis64, int nt)
{
  if (nt <= 0) nt = 1;
#pragma omp parallel num_threads(nt)
  {
    double *hv = malloc(sizeof(double) * (k + 1));
    int *hi = malloc(sizeof(int) * (k + 1));
#pragma omp for schedule(dynamic, 4)
    for (long iq = 0; iq < nq; iq++) {
      const float *x = q + iq * (long)d;
      int n = 0;
      for (int j = 0; j < nb; j++) {
        double v = dist64(x, b + (long)j * d, d);
        if (isnan(v)) continue;
        if (n < k) {
          hv[n] = v; hi[n] = j; n++;
          if (n == k)
            for (int s = k / 2 - 1; s >= 0; s--) lexheap_sift_down(hv, hi, k, s);
        } else if (lex_gt(hv[0], hi[0], v, j)) {
          hv[0] = v; hi[0] = j;
          lexheap_sift_down(hv, hi, k, 0);
        }
      }
      if (n < k)
        for (int s = n / 2 - 1; s >= 0; s--) lexheap_sift_down(hv, hi, n, s);
      /* heap-sort ascending */
      int m = n;
      while (m > 1) {
        double tv = hv[0]; hv[0] = hv[m - 1]; hv[m - 1] = tv;
        int ti = hi[0]; hi[0] = hi[m - 1]; hi[m - 1] = ti;
        m--;
        lexheap_sift_down(hv, hi, m, 0);
      }
      for (int r = 0; r < k; r++) {
        if (r < n) {
          assign[iq * k + r] = hi[r];
          dis[iq * k + r] = (float)hv[r];
          if (dis64) dis64[iq * k + r] = hv[r];
        } else {
          assign[iq * k + r] = -1;
          memset(&dis[iq * k + r], 0xff, sizeof(float));
          if (dis64) dis64[iq * k + r] = NAN;
        }
      }
    }
    free(hv); free(hi);
  }
}

void orc_cross_distances_exact(int d, int na, int nb, const float *a,
                               const float *b, double *dist2)
{
#pragma omp parallel for schedule(static)
  for (long j = 0; j < nb; j++)
    for (long i = 0; i < na; i++)
      dist2[i + (long)na * j] = dist64(a + i * d, b + j * d, d);
}

/* argmin in FP64, ties to the lowest index (the k=1 rule of yael/nn.c:431-435) */
static void assign_exact(int d, int n, int k, const float *v, const float *c,
                         int *assign, float *dis, int nt)
{
#pragma omp parallel for schedule(static) num_threads(nt > 0 ? nt : 1)
  for (long i = 0; i < n; i++) {
    double best = INFINITY;
    int bi = -1;
    for (int j = 0; j < k; j++) {
      double t = dist64(v + i * d, c + (long)j * d, d);
      if (t < best) { best = t; bi = j; }
    }
    assign[i] = bi;
    dis[i] = bi >= 0 ? (float)best : 1e30f;
  }
}

/* FP64 argmin of point x over all k centroids (assign_exact's rule) */
static int argmin64(int d, int k, const float *x, const float *c)
{
  double best = INFINITY;
  int bi = -1;
  for (int j = 0; j < k; j++) {
    double t = dist64(x, c + (long)j * d, d);
    if (t < best) { best = t; bi = j; }
  }
  return bi;
}

long orc_assign_check(int d, int n, int k, const float *v, const float *c, const int *assign,
                      int nt, long *first_bad)
{
  enum { PB = 64, CB = 2048, CAP = 32 };
  double *cn = malloc(sizeof(double) * (size_t)k);
  for (long j = 0; j < k; j++) {
    double s = 0;
    for (int i = 0; i < d; i++) s += (double)c[j * d + i] * c[j * d + i];
    cn[j] = s;
  }
  const double rel = (d + 4) * 5.9604644775390625e-08;
  long bad = 0, first = -1;
#pragma omp parallel num_threads(nt > 0 ? nt : 1)
  {
    float *dot = malloc(sizeof(float) * PB * CB);
    int *cj = malloc(sizeof(int) * PB * CAP);
    double *clo = malloc(sizeof(double) * PB * CAP);
    long my_bad = 0, my_first = -1;
#pragma omp for schedule(dynamic)
    for (long p0 = 0; p0 < n; p0 += PB) {
      const int np = (int)(n - p0 < PB ? n - p0 : PB);
      double xn2[PB], xn[PB], m[PB];
      int cnt[PB];
      for (int i = 0; i < np; i++) {
        double s = 0;
        for (int t = 0; t < d; t++) s += (double)v[(p0 + i) * d + t] * v[(p0 + i) * d + t];
        xn2[i] = s;
        xn[i] = sqrt(s);
        m[i] = INFINITY;
        cnt[i] = 0;
      }
      for (int j0 = 0; j0 < k; j0 += CB) {
        const int nc = k - j0 < CB ? k - j0 : CB;
        float one = 1, zero = 0;
        sgemm_("Trans", "Not", &np, &nc, &d, &one, v + p0 * d, &d, c + (long)j0 * d, &d, &zero,
               dot, &np);
        for (int jj = 0; jj < nc; jj++) {
          const long j = j0 + jj;
          const double cnj = sqrt(cn[j]);
          for (int i = 0; i < np; i++) {
            if (cnt[i] < 0) continue;  /* overflowed: full FP64 scan later */
            const double a = xn2[i] + cn[j] - 2.0 * (double)dot[i + (long)np * jj];
            const double b = rel * (xn[i] + cnj) * (xn[i] + cnj);
            if (!(a - b <= m[i])) continue;  /* NaN never enters */
            if (a + b < m[i]) {
              m[i] = a + b;
              int w = 0; /* drop the listed ones now above the new bound */
              for (int t = 0; t < cnt[i]; t++)
                if (clo[i * CAP + t] <= m[i]) {
                  clo[i * CAP + w] = clo[i * CAP + t];
                  cj[i * CAP + w] = cj[i * CAP + t];
                  w++;
                }
              cnt[i] = w;
            }
            if (cnt[i] == CAP) { cnt[i] = -1; continue; }
            clo[i * CAP + cnt[i]] = a - b;
            cj[i * CAP + cnt[i]] = (int)j;
            cnt[i]++;
          }
        }
      }
      for (int i = 0; i < np; i++) {
        const float *x = v + (p0 + i) * d;
        int bi = -1;
        if (cnt[i] <= 0) {
          bi = argmin64(d, k, x, c);
        } else {
          double best = INFINITY;
          for (int t = 0; t < cnt[i]; t++) {
            const int j = cj[i * CAP + t];
            const double e = dist64(x, c + (long)j * d, d);
            if (e < best || (e == best && j < bi)) { best = e; bi = j; }
          }
        }
        if (assign[p0 + i] != bi) {
          my_bad++;
          if (my_first < 0 || p0 + i < my_first) my_first = p0 + i;
        }
      }
    }
#pragma omp critical
    {
      bad += my_bad;
      if (my_first >= 0 && (first < 0 || my_first < first)) first = my_first;
    }
    free(dot); free(cj); free(clo);
  }
  free(cn);
  if (first_bad) *first_bad = first;
  return bad;
}

/* k-th smallest (0-based) of a[0..n) in place (Hoare partitions) */
static double select_kth(double *a, long n, long kth)
{
  long lo = 0, hi = n - 1;
  while (lo < hi) {
    const double piv = a[lo + (hi - lo) / 2];
    long i = lo, j = hi;
    while (i <= j) {
      while (a[i] < piv) i++;
      while (a[j] > piv) j--;
      if (i <= j) { double t = a[i]; a[i] = a[j]; a[j] = t; i++; j--; }
    }
    if (kth <= j) hi = j;
    else if (kth >= i) lo = i;
    else break;
  }
  return a[kth];
}

typedef struct { double d; int j; } dist_id;

static int cmp_dist_id(const void *x, const void *y)
{
  const dist_id *a = x, *b = y;
  if (a->d < b->d) return -1;
  if (a->d > b->d) return 1;
  return (a->j > b->j) - (a->j < b->j);
}

long orc_knn_check(int d, int nq, int nb, int k, const float *b, const float *q, const int *idx,
                   int nt, long *first_bad)
{
  enum { QB = 8 };
  double *bn = malloc(sizeof(double) * (size_t)nb);
  int bfinite = 1;
  for (long j = 0; j < nb; j++) {
    double s = 0;
    for (int i = 0; i < d; i++) s += (double)b[j * d + i] * b[j * d + i];
    bn[j] = sqrt(s);
    if (!isfinite(s)) bfinite = 0;
  }
  const double rel = (d + 4) * 5.9604644775390625e-08;
  long bad = 0, first = -1;
#pragma omp parallel num_threads(nt > 0 ? nt : 1)
  {
    float *dot = malloc(sizeof(float) * (size_t)QB * nb);
    double *up = malloc(sizeof(double) * (size_t)nb);
    dist_id *cand = malloc(sizeof(dist_id) * (size_t)nb);
    int *ei = malloc(sizeof(int) * (size_t)k);
    float *ed = malloc(sizeof(float) * (size_t)k);
    long my_bad = 0, my_first = -1;
#pragma omp for schedule(dynamic)
    for (long q0 = 0; q0 < nq; q0 += QB) {
      const int nqb = (int)(nq - q0 < QB ? nq - q0 : QB);
      float one = 1, zero = 0;
      sgemm_("Trans", "Not", &nqb, &nb, &d, &one, q + q0 * d, &d, b, &d, &zero, dot, &nqb);
      for (int i = 0; i < nqb; i++) {
        const float *x = q + (q0 + i) * d;
        double qs = 0;
        for (int t = 0; t < d; t++) qs += (double)x[t] * x[t];
        const double qn = sqrt(qs);
        int ok = 1;
        if (!bfinite || !isfinite(qs)) {
          /* non-finite values: the exact brute force itself */
          orc_knn_exact(1, nb, d, k, b, x, ei, ed, NULL, 1);
          for (int t = 0; t < k; t++) ok &= ei[t] == idx[(q0 + i) * (long)k + t];
        } else {
          for (long j = 0; j < nb; j++) {
            const double a = qs + bn[j] * bn[j] - 2.0 * (double)dot[i + (long)nqb * j];
            up[j] = a + rel * (qn + bn[j]) * (qn + bn[j]);
          }
          const double U = select_kth(up, nb, k - 1);
          long nc = 0;
          for (long j = 0; j < nb; j++) {
            const double a = qs + bn[j] * bn[j] - 2.0 * (double)dot[i + (long)nqb * j];
            if (a - rel * (qn + bn[j]) * (qn + bn[j]) <= U) {
              cand[nc].d = dist64(x, b + j * d, d);
              cand[nc].j = (int)j;
              nc++;
            }
          }
          qsort(cand, (size_t)nc, sizeof(dist_id), cmp_dist_id);
          for (int t = 0; t < k; t++)
            ok &= t < nc && cand[t].j == idx[(q0 + i) * (long)k + t];
        }
        if (!ok) {
          my_bad++;
          if (my_first < 0 || q0 + i < my_first) my_first = q0 + i;
        }
      }
    }
#pragma omp critical
    {
      bad += my_bad;
      if (my_first >= 0 && (first < 0 || my_first < first)) first = my_first;
    }
    free(dot); free(up); free(cand); free(ei); free(ed);
  }
  free(bn);
  if (first_bad) *first_bad = first;
  return bad;
}

double orc_objective64(int d, int n, const float *v, const float *c, const int *assign, int nt)
{
  double tot = 0;
#pragma omp parallel for schedule(static) reduction(+ : tot) num_threads(nt > 0 ? nt : 1)
  for (long i = 0; i < n; i++)
    if (assign[i] >= 0) tot += dist64(v + i * d, c + (long)assign[i] * d, d);
  return tot;
}

/* ------------------------------------------------------------------ */
/* RNG replay (yael/vector.c:134-155, 184-189, 226-253; kmeans.c:15-24) */

static double drand_r(unsigned int *seed) { return rand_r(seed) / ((double)RAND_MAX + 1.0); }

/* Kinderman-Monahan ratio-of-uniforms normal deviate with the reference's
 * float/double roundings (u1, u2 and zz held in float). */
double orc_gaussrand_r(unsigned int *seed)
{
  const double magic = 1.71552776992141; /* 4 exp(-1/2) / sqrt(2) */
  double z;
  for (;;) {
    float u1 = (float)drand_r(seed);
    float u2 = (float)drand_r(seed);
    z = magic * (u1 - .5) / u2;
    float zz = (float)(z * z / 4.0);
    if (zz < -log(u2)) break;
  }
  return z;
}

/* first k entries of the partial Fisher-Yates permutation */
void orc_random_init(int n, int k, unsigned int seed, int *sel)
{
  int *idx = malloc(sizeof(int) * (size_t)n);
  for (int i = 0; i < n; i++) idx[i] = i;
  for (int i = 0; i < k && i < n; i++) {
    int j = i + rand_r(&seed) % (n - i);
    int t = idx[i]; idx[i] = idx[j]; idx[j] = t;
  }
  memcpy(sel, idx, sizeof(int) * (size_t)k);
  free(idx);
}

static double norm_l1(const float *v, long n)
{
  double s = 0;
  for (long i = 0; i < n; i++) s += fabs(v[i]);
  return s;
}

static double norm_l2(const float *v, long n)
{
  double s = 0;
  for (long i = 0; i < n; i++) s += v[i] * v[i];
  return sqrt(s);
}

static void mul_by(float *v, long n, double s)
{
  for (long i = 0; i < n; i++) v[i] *= s;
}

/* kmeans_reassign_empty (yael/kmeans.c:166-209) */
static int reassign_empty(int d, int k, float *C, const int *nassign, unsigned int seed)
{
  int nre = 0;
  float *p = malloc(sizeof(float) * k);
  float *eps = malloc(sizeof(float) * d);
  for (int c = 0; c < k; c++) {
    /* nassign^2 - 1 in int arithmetic; large clusters wrap like the reference */
    unsigned int sq = (unsigned int)nassign[c] * (unsigned int)nassign[c] - 1u;
    p[c] = nassign[c] < 2 ? 0 : (float)(int)sq;
  }
  mul_by(p, k, 1. / norm_l1(p, k));
  for (int c = 0; c < k; c++) {
    if (nassign[c] != 0) continue;
    nre++;
    double rd = drand_r(&seed);
    int j;
    for (j = 0; j < k - 1; j++) {
      rd -= p[j];
      if (rd < 0) break;
    }
    memcpy(C + (long)c * d, C + (long)j * d, sizeof(float) * d);
    double s = norm_l2(C + (long)j * d, d) * 0.0000001;
    unsigned int s2 = rand_r(&seed);
    for (int i = 0; i < d; i++) eps[i] = (float)orc_gaussrand_r(&s2);
    mul_by(eps, d, s);
    for (int i = 0; i < d; i++) C[(long)j * d + i] += eps[i];
    for (int i = 0; i < d; i++) C[(long)c * d + i] -= eps[i];
    p[j] = 0;
    mul_by(p, k, 1. / norm_l1(p, k));
  }
  free(p); free(eps);
  return nre;
}

int orc_reassign_empty(int d, int k, float *C, const int *nassign, unsigned int seed)
{
  return reassign_empty(d, k, C, nassign, seed);
}

/* ------------------------------------------------------------------ */
/* exact fixed-point centroid sums                                     */

int orc_fixed_shift(long n, long d, const float *v)
{
  /* largest |x| < 2^e; n terms of |x| 2^S stay below 2^62 */
  float m = 0;
  for (long i = 0; i < n * d; i++) {
    float a = fabsf(v[i]);
    if (a > m) m = a;
  }
  int e = 0;
  if (m > 0) frexp((double)m, &e);
  int lg = 0;
  while ((1L << lg) < n) lg++;
  return 62 - lg - e;
}

static void update_exact(int d, int n, int k, const float *v, const int *assign,
                         const int *nassign, float *C, int S)
{
  int64_t *acc = calloc((size_t)k * d, sizeof(int64_t));
  double sc = ldexp(1.0, S), inv = ldexp(1.0, -S);
  for (long i = 0; i < n; i++) {
    int a = assign[i];
    if (a < 0) continue;
    for (int j = 0; j < d; j++) acc[(long)a * d + j] += llrint((double)v[i * d + j] * sc);
  }
  for (long c = 0; c < k; c++) {
    double r = 1.0 / nassign[c];
    for (int j = 0; j < d; j++)
      C[c * d + j] = (float)((double)acc[c * d + j] * inv * r);
  }
  free(acc);
}

void orc_kmeans_step_exact(int d, int n, int k, const float *v, const float *c_in,
                           int *assign, float *dis, int *nassign, float *c_out,
                           int S)
{
  assign_exact(d, n, k, v, c_in, assign, dis, 8);
  memset(nassign, 0, sizeof(int) * k);
  for (int i = 0; i < n; i++)
    if (assign[i] >= 0) nassign[assign[i]]++;
  update_exact(d, n, k, v, assign, nassign, c_out, S);
}

/* compute_distances_1_nonpacked (yael/nn.c:132-154): double norms + sgemv */
static void distances_1_port(int d, int nb, const float *a, const float *b, int ldb,
                             float *dist2)
{
  double sa = 0;
  for (int j = 0; j < d; j++) sa += a[j] * a[j];
  for (long i = 0; i < nb; i++) {
    double s = 0;
    const float *x = b + ldb * i;
    for (int j = 0; j < d; j++) s += x[j] * x[j];
    dist2[i] = s + sa;
  }
  float m2 = -2, one = 1;
  int ione = 1;
  sgemv_("Transposed", &d, &nb, &m2, b, &ldb, a, &ione, &one, dist2, &ione);
}

/* kmeanspp_init (yael/kmeans.c:27-82); the port computes the distances as
 * compute_distances_1_thread does (yael/nn.c:840-860), the exact mode as
 * FP64 rounded to float */
static void kmeanspp_init(int d, int n, int k, const float *v, int *sel, unsigned int seed,
                          int nt, int mode)
{
  float *best = malloc(sizeof(float) * (size_t)n);
  float *tmp = malloc(sizeof(float) * (size_t)n);
  for (long j = 0; j < n; j++) best[j] = HUGE_VAL;
  sel[0] = rand_r(&seed) % k;
  for (int i = 1; i < k; i++) {
    int ns = sel[i - 1];
    if (mode == ORC_PORT) {
#pragma omp parallel for num_threads(nt > 0 ? nt : 1)
      for (int t = 0; t < nt; t++) {
        int i0 = t * n / nt, i1 = (t + 1) * n / nt;
        distances_1_port(d, i1 - i0, v + (long)d * ns, v + (long)i0 * d, d, tmp + i0);
      }
    } else {
#pragma omp parallel for schedule(static)
      for (long j = 0; j < n; j++) tmp[j] = (float)dist64(v + j * d, v + (long)ns * d, d);
    }
    for (long j = 0; j < n; j++)
      if (tmp[j] < best[j]) best[j] = tmp[j];
    memcpy(tmp, best, sizeof(float) * (size_t)n);
    mul_by(tmp, n, 1. / norm_l1(tmp, n));
    double rd = drand_r(&seed);
    long j;
    for (j = 0; j < n - 1; j++) {
      rd -= tmp[j];
      if (rd < 0) break;
    }
    sel[i] = (int)j;
  }
  free(best);
  free(tmp);
}

/* ------------------------------------------------------------------ */
/* kmeans (yael/kmeans.c:213-447), L2 only                              */

static int cmp_float(const void *a, const void *b)
{
  float x = *(const float *)a, y = *(const float *)b;
  return x < y ? -1 : x > y;
}

/* fvec_median (yael/sorting.c:676-703): an order statistic, so the value of
 * a sorted copy equals the reference's in-place selection (non-NaN data) */
static float median_port(const float *f, int n, float *work)
{
  if (n == 0) return 0.0f / 0.0f;
  if (n == 1) return f[0];
  memcpy(work, f, sizeof(float) * (size_t)n);
  qsort(work, (size_t)n, sizeof(float), cmp_float);
  int halfn = n / 2;
  if (n % 2 == 1) return work[halfn];
  return (float)(0.5 * (work[halfn] + work[halfn - 1]));
}

/* minimize_sum_chi2 (yael/kmeans.c:95-158): Newton steps in float over a[]
 * in the order given */
static float chi2_port(const float *a, int n)
{
  if (n == 0) return 0.0f / 0.0f;
  if (n == 1) return a[0];
  float x, prev_x = 0, mag = 0;
  for (int i = 0; i < n; i++) mag += a[i];
  mag /= n;
  x = 0;
  int niter = 0;
  do {
    float dv = 0, dd = 0;
    for (int i = 0; i < n; i++) {
      float sum2 = (x + a[i]) * (x + a[i]);
      float sum3 = (x + a[i]) * sum2;
      if (sum2 == 0) continue;
      dv += (x - a[i]) * (x + 3 * a[i]) / sum2;
      dd += 8 * a[i] * a[i] / sum3;
    }
    if (dv == 0) break;
    prev_x = x;
    x -= dv / dd;
    if (x < 0) x = (float)(prev_x / 2.0);
    if (++niter == 1000) break;
  } while (fabs(x - prev_x) > 1e-4 * mag);
  return x;
}

/* the L1 / chi2 centroid update of kmeans_core (yael/kmeans.c:253-275): each
 * cluster's coordinates gathered column by column, the cluster's points in
 * decreasing index order, then the median / the chi2 minimiser of each */
static void update_alt_port(int d, int n, int k, const float *v, const int *assign,
                            const int *nassign, int l1, float *C)
{
  float *tmp_v = malloc(sizeof(float) * ((size_t)n * d + 1));
  float *work = malloc(sizeof(float) * ((size_t)n + 1));
  int *cum = malloc(sizeof(int) * (size_t)k);
  int run = 0;
  for (int c = 0; c < k; c++) { run += nassign[c]; cum[c] = run; }
  for (long i = 0; i < n; i++) {
    int w = --cum[assign[i]];
    for (long j = 0; j < d; j++) tmp_v[w + j * n] = v[i * d + j];
  }
  for (long c = 0; c < k; c++)
    for (long j = 0; j < d; j++) {
      const float *col = tmp_v + cum[c] + j * n;
      C[c * d + j] = l1 ? median_port(col, nassign[c], work) : chi2_port(col, nassign[c]);
    }
  free(cum); free(work); free(tmp_v);
}

static int kmeans_core(int d, int n, int k, int niter, int nt, int flags, float *C,
                       const float *v, unsigned int seed, int *assign, int *nassign,
                       float *dis, double *qerr_out, long *iter_tot, int mode, int S)
{
  const int alt = (flags & (ORC_KMEANS_L1 | ORC_KMEANS_CHI2)) != 0;
  const int l1 = (flags & ORC_KMEANS_L1) != 0;
  if (alt && mode != ORC_PORT) {
    fprintf(stderr, "oracle: L1 / chi2 k-means is restated in port mode only\n");
    abort();
  }
  double qerr = HUGE_VAL, qerr_old;
  int tot_re = 0;
  for (int iter = 1; iter <= niter; iter++) {
    (*iter_tot)++;
    if (mode == ORC_PORT)
      orc_knn_port(alt ? (l1 ? 1 : 3) : 2, n, k, d, 1, C, v, NULL, assign, dis, nt);
    else
      assign_exact(d, n, k, v, C, assign, dis, nt);
    memset(nassign, 0, sizeof(int) * k);
    for (int i = 0; i < n; i++) nassign[assign[i]]++;
    if (alt) {
      update_alt_port(d, n, k, v, assign, nassign, l1, C);
    } else if (mode == ORC_PORT) {
      memset(C, 0, sizeof(float) * (size_t)k * d);
      for (long i = 0; i < n; i++) {
        float *c = C + (long)assign[i] * d;
        for (int j = 0; j < d; j++) c[j] += v[i * d + j];
      }
      for (long c = 0; c < k; c++) mul_by(C + c * d, d, 1.0 / nassign[c]);
    } else {
      update_exact(d, n, k, v, assign, nassign, C, S);
    }
    if (flags & ORC_KMEANS_NORMALIZE_CENTS)
      for (long c = 0; c < k; c++)
        mul_by(C + c * d, d, 1. / (l1 ? norm_l1(C + c * d, d) : norm_l2(C + c * d, d)));
    int nre = reassign_empty(d, k, C, nassign, rand_r(&seed));
    tot_re += nre;
    if (tot_re > n / 100 && tot_re > 1000) return -1;
    qerr_old = qerr;
    qerr = 0;
    for (long i = 0; i < n; i++) qerr += dis[i];
    if (qerr_old == qerr && nre == 0) break;
  }
  *qerr_out = qerr;
  return 0;
}

float orc_kmeans(int d, int n, int k, int niter, const float *v, int flags,
                 long seed_in, int redo, float *C_out, float *dis_out,
                 int *assign_out, int *nassign_out, int mode, long *iters_out)
{
  int nt = flags & 0xffff;
  if (nt == 0) nt = 1;
  niter = niter == 0 ? 1000000 : niter;
  int user = (flags & ORC_KMEANS_INIT_USER) != 0;
  if (user) redo = 1;
  if (k > n) return -2; /* the reference asserts (kmeans.c:377) */
  float *C = malloc(sizeof(float) * (size_t)k * d);
  float *dis = malloc(sizeof(float) * (size_t)n);
  int *assign = malloc(sizeof(int) * (size_t)n);
  int *nassign = malloc(sizeof(int) * (size_t)k);
  int *sel = malloc(sizeof(int) * (size_t)k);
  double qerr = 0, best = HUGE_VAL;
  long iter_tot = 0;
  int S = mode == ORC_EXACT ? orc_fixed_shift(n, d, v) : 0;
  if (seed_in == 0) seed_in = lrand48();
  unsigned int seed = (unsigned int)seed_in;
  int ret = 0;
  for (int run = 0; run < redo; run++) {
    if (user) {
      memcpy(C, C_out, sizeof(float) * (size_t)k * d);
    } else {
      if (flags & ORC_KMEANS_INIT_BERKELEY) {
        int nsub = n;
        if (n > k * 8 && n > 8192) nsub = k * 8;
        kmeanspp_init(d, nsub, k, v, sel, rand_r(&seed), nt, mode);
      } else {
        orc_random_init(n, k, rand_r(&seed), sel);
      }
      for (long i = 0; i < k; i++) memcpy(C + i * d, v + (long)sel[i] * d, sizeof(float) * d);
    }
    ret = kmeans_core(d, n, k, niter, nt, flags, C, v, rand_r(&seed), assign, nassign,
                      dis, &qerr, &iter_tot, mode, S);
    if (ret < 0) break;
    if (qerr < best) {
      best = qerr;
      if (C_out) memcpy(C_out, C, sizeof(float) * (size_t)k * d);
      if (dis_out) memcpy(dis_out, dis, sizeof(float) * (size_t)n);
      if (assign_out) memcpy(assign_out, assign, sizeof(int) * (size_t)n);
      if (nassign_out) memcpy(nassign_out, nassign, sizeof(int) * (size_t)k);
    }
  }
  if (iters_out) *iters_out = iter_tot;
  free(C); free(dis); free(assign); free(nassign); free(sel);
  return ret < 0 ? -1 : (float)(best / n);
}

/* ------------------------------------------------------------------ */
/* hierarchical k-means (yael/hkm.c:36-150)                             */

static int cmp_key_then_index(const void *a, const void *b, void *ctx)
{
  const int *key = (const int *)ctx;
  int ia = *(const int *)a, ib = *(const int *)b;
  if (key[ia] != key[ib]) return key[ia] < key[ib] ? -1 : 1;
  return ia - ib;
}

int orc_hkm_learn(int n, int d, int nlevel, int bf, const float *points,
                  int nb_iter_max, float *centroids_out, int *assign_out, int mode)
{
  int *node = calloc((size_t)n, sizeof(int));
  int *perm = malloc(sizeof(int) * (size_t)n);
  float *v = malloc(sizeof(float) * (size_t)n * d);
  long k = 1, off = 0;
  int rc = 0;
  for (int l = 0; l < nlevel && rc == 0; l++) {
    for (int i = 0; i < n; i++) perm[i] = i;
    qsort_r(perm, n, sizeof(int), cmp_key_then_index, node);
    for (long i = 0; i < n; i++) memcpy(v + i * d, points + (long)perm[i] * d, sizeof(float) * d);
    long pos = 0;
    for (long parent = 0; parent < k; parent++) {
      int na = 0;
      while (pos + na < n && node[perm[pos + na]] == parent) na++;
      const int small = na < bf && (mode & ORC_HKM_SMALL_NODES);
      if (na == 0 || (na < bf && !small)) { rc = -1; break; }
      int *ca = malloc(sizeof(int) * (size_t)na);
      float *C = malloc(sizeof(float) * (size_t)bf * d);
      if (small) {
        /* one child per point (later children repeat the last point); the
         * kmeans() seed draw is still made, so later seeds stay in step */
        (void)lrand48();
        for (int j = 0; j < bf; j++)
          memcpy(C + (long)j * d, v + (pos + (j < na ? j : na - 1)) * d, sizeof(float) * d);
        for (int i = 0; i < na; i++) ca[i] = i;
      } else {
        orc_kmeans(d, na, bf, nb_iter_max, v + pos * d,
                   8 | ORC_KMEANS_INIT_RANDOM | ORC_KMEANS_QUIET, 0, 1, C, NULL, ca,
                   NULL, mode & 1, NULL);
      }
      memcpy(centroids_out + off + parent * bf * d, C, sizeof(float) * (size_t)bf * d);
      for (int i = 0; i < na; i++) {
        int t = perm[pos + i];
        node[t] = node[t] * bf + ca[i];
      }
      free(ca); free(C);
      pos += na;
    }
    off += k * bf * d;
    k *= bf;
  }
  if (assign_out) memcpy(assign_out, node, sizeof(int) * (size_t)n);
  free(node); free(perm); free(v);
  return rc;
}

void orc_hkm_quantize(int nlevel, int bf, int d, const float *centroids, int npt,
                      const float *v, int *idx, int mode)
{
#pragma omp parallel for schedule(static)
  for (long i = 0; i < npt; i++) {
    long vw = 0, off = 0, k = bf;
    for (int l = 0; l < nlevel; l++) {
      const float *C = centroids + off + vw * d * bf;
      int t;
      float dd;
      if (mode == ORC_PORT)
        knn_full_port(2, 1, bf, d, 1, C, v + i * d, NULL, &t, &dd);
      else
        assign_exact(d, 1, bf, v + i * d, C, &t, &dd, 1);
      vw = vw * bf + t;
      off += k * d;
      k *= bf;
    }
    idx[i] = (int)vw;
  }
}

/* ------------------------------------------------------------------ */
/* k-means LSH (yael/kmlsh.c)                                           */

/* nnlist_add (yael/kmlsh.c:60-84) on one list of k */
static void orc_nnlist_add(int *idx, float *dis, int k, int elidx, float eldis)
{
  if (eldis > dis[0]) return;
  for (int i = 0; i < k; i++)
    if (idx[i] == elidx) return;
  idx[0] = elidx;
  dis[0] = eldis;
  int posmax = 0; /* fvec_arg_max (yael/sorting.c:764-775) */
  float m = dis[0];
  for (int i = 1; i < k; i++)
    if (dis[i] > m) { m = dis[i]; posmax = i; }
  if (posmax == 0) return;
  idx[0] = idx[posmax];
  dis[0] = dis[posmax];
  idx[posmax] = elidx;
  dis[posmax] = eldis;
}

/* fvec_cpy_subvectors / b2fvec_cpy_subvectors (yael/vector.c:2478-2497) */
static void orc_rows(const void *v, int vec_type, const int *ids, long m, int d, float *out)
{
  for (long i = 0; i < m; i++)
    for (int j = 0; j < d; j++)
      out[i * d + j] = vec_type == 0 ? ((const float *)v)[(long)ids[i] * d + j]
                                     : (float)((const unsigned char *)v)[(long)ids[i] * d + j];
}

/* kmeans_cohash_xvec (yael/kmlsh.c:210-279): nearest centroid of every vector
 * in blocks of KMLSH_BLOCK_SIZE, then the ids ordered by cell and the cell
 * starts */
static void orc_cohash(const float *C, int nclust, int d, const void *v, int n, int vec_type,
                       int mode, int nt, int *perm, int *bnd)
{
  int *idx = malloc(sizeof(int) * (size_t)(n + 1));
  float *dis = malloc(sizeof(float) * (size_t)(n + 1));
  float *buf = malloc(sizeof(float) * 256 * (size_t)d);
  int *ids = malloc(sizeof(int) * 256);
  for (long i = 0; i < n; i += 256) {
    int m = n - i < 256 ? (int)(n - i) : 256;
    for (int j = 0; j < m; j++) ids[j] = (int)(i + j);
    orc_rows(v, vec_type, ids, m, d, buf);
    if (mode == ORC_PORT)
      orc_knn_port(2, m, nclust, d, 1, C, buf, NULL, idx + i, dis + i, nt);
    else
      orc_knn_exact(m, nclust, d, 1, C, buf, idx + i, dis + i, NULL, nt);
  }
  int *nocc = calloc((size_t)nclust + 1, sizeof(int));
  for (int c = 0; c <= nclust; c++) bnd[c] = 0;
  for (long i = 0; i < n; i++) bnd[idx[i] + 1]++;
  for (int c = 0; c < nclust; c++) bnd[c + 1] += bnd[c];
  for (long i = 0; i < n; i++) perm[bnd[idx[i]] + nocc[idx[i]]++] = (int)i;
  free(nocc); free(ids); free(buf); free(dis); free(idx);
}

void orc_kmlsh_ann(const void *vb, int nb, const void *vq, int nq, int d, int k, int nhash,
                   int vec_type, int mode, int nt, int *idx_out, float *dis_out)
{
  /* kmlsh_ann_xvec (yael/kmlsh.c:479-500); nt threads as its knn_full_thread
   * and kmeans calls use them */
  if (nt < 1) nt = 1;
  int nclust = (int)sqrt(nb);
  int nlearn = nclust * 100;
  if (nlearn > nb) nlearn = nb;
  long cs = (long)nclust * d;
  float *C = malloc(sizeof(float) * (size_t)(cs * nhash + 1));
  /* kmlsh_learn_xvec (yael/kmlsh.c:133-185) */
  float *vlearn = malloc(sizeof(float) * ((size_t)nlearn * d + 1));
  int *sel = malloc(sizeof(int) * (size_t)(nlearn + 1));
  for (int h = 0; h < nhash; h++) {
    orc_random_init(nb, nlearn, (unsigned int)lrand48(), sel);
    orc_rows(vb, vec_type, sel, nlearn, d, vlearn);
    orc_kmeans(d, nlearn, nclust, 8, vlearn, nt | ORC_KMEANS_INIT_RANDOM, 0, 1, C + h * cs,
               NULL, NULL, NULL, mode, NULL);
  }
  free(sel);
  free(vlearn);
  /* kmlsh_idx_new_compile_xvec (yael/kmlsh.c:319-338) for base and queries */
  int *pb = malloc(sizeof(int) * ((size_t)nb * nhash + 1));
  int *pq = malloc(sizeof(int) * ((size_t)nq * nhash + 1));
  int *bb = malloc(sizeof(int) * (size_t)(nclust + 1) * nhash);
  int *bq = malloc(sizeof(int) * (size_t)(nclust + 1) * nhash);
  for (int h = 0; h < nhash; h++) {
    orc_cohash(C + h * cs, nclust, d, vb, nb, vec_type, mode, nt, pb + (long)h * nb,
               bb + (long)h * (nclust + 1));
    orc_cohash(C + h * cs, nclust, d, vq, nq, vec_type, mode, nt, pq + (long)h * nq,
               bq + (long)h * (nclust + 1));
  }
  /* kmlsh_match_xvec (yael/kmlsh.c:376-456) */
  for (long i = 0; i < (long)nq * k; i++) { idx_out[i] = -1; dis_out[i] = 1e30f; }
  float *vbuf_b = malloc(sizeof(float) * ((size_t)nb * d + 1));
  float *vbuf_q = malloc(sizeof(float) * ((size_t)nq * d + 1));
  int *it = malloc(sizeof(int) * ((size_t)nq * k + 1));
  float *dt = malloc(sizeof(float) * ((size_t)nq * k + 1));
  for (int h = 0; h < nhash; h++) {
    const int *hb = bb + (long)h * (nclust + 1), *hq = bq + (long)h * (nclust + 1);
    for (int c = 0; c < nclust; c++) {
      int nbc = hb[c + 1] - hb[c], nqc = hq[c + 1] - hq[c];
      if (nbc == 0 || nqc == 0) continue;
      const int *vidx_b = pb + (long)h * nb + hb[c];
      const int *vidx_q = pq + (long)h * nq + hq[c];
      orc_rows(vb, vec_type, vidx_b, nbc, d, vbuf_b);
      orc_rows(vq, vec_type, vidx_q, nqc, d, vbuf_q);
      int k2 = k < nbc ? k : nbc;
      if (mode == ORC_PORT)
        orc_knn_port(2, nqc, nbc, d, k2, vbuf_b, vbuf_q, NULL, it, dt, nt);
      else
        orc_knn_exact(nqc, nbc, d, k2, vbuf_b, vbuf_q, it, dt, NULL, nt);
      for (long i = 0; i < (long)k2 * nqc; i++) it[i] = vidx_b[it[i]];
      for (int i = 0; i < nqc; i++)
        for (int j = 0; j < k2; j++)
          orc_nnlist_add(idx_out + (long)vidx_q[i] * k, dis_out + (long)vidx_q[i] * k, k,
                         it[(long)i * k2 + j], dt[(long)i * k2 + j]);
    }
  }
  free(dt); free(it); free(vbuf_q); free(vbuf_b);
  free(bq); free(bb); free(pq); free(pb); free(C);
}

/* ------------------------------------------------------------------ */
/* Gaussian mixtures (yael/gmm.c) in the reference's arithmetic: the   */
/* expanded sgemm forms, float / double roundings and slice order      */

/* softmax_ref (yael/gmm.c:262-300), in place on k x n */
static void gmm_softmax_port(int k, long n, float *p)
{
  const float norm_to_0 = 16.636f;
  for (long i = 0; i < n; i++) {
    float *f = p + i * k;
    float maxval = -1e30f;
    for (int l = 0; l < k; l++)
      if (f[l] > maxval) maxval = f[l];
    float s = 0.0f;
    for (int l = 0; l < k; l++) {
      if (f[l] >= maxval - norm_to_0) {
        f[l] = (float)exp(f[l] - maxval);
        s += f[l];
      } else {
        f[l] = 0;
      }
    }
    if (s != 0) {
      float is = (float)(1.0 / s);
      for (int l = 0; l < k; l++) f[l] *= is;
    }
  }
}

/* gmm_compute_p (yael/gmm.c:305-362) with compute_mahalanobis_sqr (212-259) */
static void gmm_compute_p_port(int ni, const float *v, int di, int ki, const float *w,
                               const float *mu, const float *sigma, float *p, int flags)
{
  if (ni == 0) return;
  long n = ni, d = di, k = ki;
  float *logdetnr = malloc(sizeof(float) * k);
  for (long j = 0; j < k; j++) {
    logdetnr[j] = (float)(-d / 2.0 * log(2 * M_PI));
    for (long i = 0; i < d; i++) logdetnr[j] = (float)(logdetnr[j] - 0.5 * log(sigma[j * d + i]));
  }
  for (long j = 0; j < k; j++) {
    double dtmp = 0;
    for (long l = 0; l < d; l++) {
      double m = mu[j * d + l];
      dtmp += m * m / sigma[j * d + l];
    }
    float m2 = (float)dtmp;
    for (long i = 0; i < n; i++) p[i * k + j] = m2;
  }
  float *v2 = malloc(sizeof(float) * (size_t)(n * d));
  for (long i = 0; i < n * d; i++) v2[i] = v[i] * v[i];
  float *tmp = malloc(sizeof(float) * (size_t)(k * d));
  for (long i = 0; i < k * d; i++) tmp[i] = (float)(1.0 / sigma[i]);
  float one = 1, minus_two = -2;
  sgemm_("Transposed", "Not transposed", &ki, &ni, &di, &one, tmp, &di, v2, &di, &one, p, &ki);
  free(v2);
  for (long i = 0; i < k * d; i++) tmp[i] = mu[i] / sigma[i];
  sgemm_("Transposed", "Not transposed", &ki, &ni, &di, &minus_two, tmp, &di, v, &di, &one, p,
         &ki);
  free(tmp);
  float *lg = malloc(sizeof(float) * k);
  for (long j = 0; j < k; j++) lg[j] = (flags & 1) ? (float)log(w[j]) : 0.0f;
  for (long i = 0; i < n; i++)
    for (long j = 0; j < k; j++)
      p[i * k + j] = (float)(logdetnr[j] - 0.5 * p[i * k + j] + lg[j]);
  free(lg);
  gmm_softmax_port(ki, n, p);
  free(logdetnr);
}

void orc_gmm_compute_p(int n, const float *v, int d, int k, const float *w, const float *mu,
                       const float *sigma, float *p, int flags, int nt)
{
  /* gmm_compute_p_thread (yael/gmm.c:854-870): nt slices of the vectors */
  if (nt < 1) nt = 1;
#pragma omp parallel for schedule(static) num_threads(nt)
  for (int t = 0; t < nt; t++) {
    long n0 = (long)t * n / nt, n1 = (long)(t + 1) * n / nt;
    gmm_compute_p_port((int)(n1 - n0), v + n0 * d, d, k, w, mu, sigma, p + n0 * k, flags);
  }
}

/* compute_sum_dcov (yael/gmm.c:72-103) */
static void gmm_sum_dcov_port(int ni, int ki, int di, const float *v, const float *mu_old,
                              const float *p, float *mu, float *sigma, float *w)
{
  long n = ni, k = ki, d = di;
  for (long j = 0; j < k; j++) {
    double dtmp = 0;
    for (long i = 0; i < n; i++) dtmp += p[i * k + j];
    w[j] = (float)dtmp;
  }
  float zero = 0, one = 1;
  sgemm_("Not transposed", "Transposed", &di, &ki, &ni, &one, v, &di, p, &ki, &zero, mu, &di);
  float *v2 = malloc(sizeof(float) * (size_t)(n * d + 1));
  for (long i = 0; i < n * d; i++) v2[i] = v[i] * v[i];
  sgemm_("Not transposed", "Transposed", &di, &ki, &ni, &one, v2, &di, p, &ki, &zero, sigma,
         &di);
  free(v2);
  for (long j = 0; j < k; j++)
    for (long l = 0; l < d; l++) {
      float mo = mu_old[j * d + l];
      sigma[j * d + l] += mo * (mo * w[j] - 2 * mu[j * d + l]);
    }
}

/* gmm_compute_params (yael/gmm.c:114-199) with compute_sum_dcov_thread
 * (880-930) for nt > 1 */
static void gmm_compute_params_port(int n, const float *v, const float *p, int d, int k,
                                    float *w, float *mu, float *sigma, int flags, int nt)
{
  long kd = (long)k * d;
  float *mu_old = malloc(sizeof(float) * (size_t)kd);
  memcpy(mu_old, mu, sizeof(float) * (size_t)kd);
  if (nt <= 1) {
    gmm_sum_dcov_port(n, k, d, v, mu_old, p, mu, sigma, w);
  } else {
    float *tm = malloc(sizeof(float) * (size_t)(nt * kd));
    float *ts = malloc(sizeof(float) * (size_t)(nt * kd));
    float *tw = malloc(sizeof(float) * (size_t)(nt * k));
#pragma omp parallel for schedule(static) num_threads(nt)
    for (int t = 0; t < nt; t++) {
      long n0 = (long)t * n / nt, n1 = (long)(t + 1) * n / nt;
      gmm_sum_dcov_port((int)(n1 - n0), k, d, v + d * n0, mu_old, p + n0 * k, tm + t * kd,
                        ts + t * kd, tw + (long)t * k);
    }
    memcpy(mu, tm, sizeof(float) * (size_t)kd);
    memcpy(sigma, ts, sizeof(float) * (size_t)kd);
    memcpy(w, tw, sizeof(float) * (size_t)k);
    for (int t = 1; t < nt; t++) {
      for (long i = 0; i < kd; i++) mu[i] += tm[t * kd + i];
      for (long i = 0; i < kd; i++) sigma[i] += ts[t * kd + i];
      for (long i = 0; i < k; i++) w[i] += tw[(long)t * k + i];
    }
    free(tm); free(ts); free(tw);
  }
  if (flags & 4) { /* GMM_FLAGS_1SIGMA */
    for (long j = 0; j < k; j++) {
      double s = 0;
      for (long l = 0; l < d; l++) s += sigma[j * d + l];
      float var = (float)(s / d);
      for (long l = 0; l < d; l++) sigma[j * d + l] = var;
    }
  }
  for (long i = 0; i < kd; i++)
    if (sigma[i] < 1e-10f) sigma[i] = 1e-10f;
  for (long j = 0; j < k; j++) { /* fvec_div_by: times 1. / w in double */
    double inv = 1. / w[j];
    for (long l = 0; l < d; l++) {
      mu[j * d + l] = (float)(mu[j * d + l] * inv);
      sigma[j * d + l] = (float)(sigma[j * d + l] * inv);
    }
  }
  double nr = 0; /* fvec_normalize(w, k, 1) */
  for (long j = 0; j < k; j++) nr += fabs(w[j]);
  for (long j = 0; j < k; j++) w[j] = (float)(w[j] * (1. / nr));
  free(mu_old);
}

/* gmm_handle_empty (yael/gmm.c:366-433); returns -1 where the reference
 * asserts or loops for ever */
static int gmm_handle_empty_port(long n, const float *v, int d, int k, const float *mu,
                                 const float *sigma, float *p)
{
  float *w = calloc((size_t)k, sizeof(float));
  for (long i = 0; i < n; i++)
    for (int j = 0; j < k; j++) w[j] += p[j + i * k];
  const int bigprime = 1000003;
  for (int j = 0; j < k; j++) {
    if (w[j] != 0) continue;
    int j2 = j, tries = 0, nnz;
    for (;;) {
      int i;
      for (i = 0; i < k; i++) {
        j2 = (j2 + bigprime) % k;
        if (w[j2] > 0) break;
      }
      if (i == k || ++tries > k) { free(w); return -1; }
      nnz = 0;
      for (long t = 0; t < n; t++)
        if (p[j2 + t * k] > 0) nnz++;
      if (nnz < n / k) continue;
      break;
    }
    int sd = 0;
    for (int l = 1; l < d; l++)
      if (sigma[(long)d * j2 + l] > sigma[(long)d * j2 + sd]) sd = l;
    for (long t = 0; t < n; t++)
      if (p[j2 + t * k] > 0 && v[t * d + sd] < mu[(long)j2 * d + sd]) {
        p[j + t * k] = p[j2 + t * k];
        p[j2 + t * k] = 0;
      }
    w[j2] = -1;
  }
  free(w);
  return 0;
}

int orc_gmm_em_step(int n, const float *v, int d, int k, float *w, float *mu, float *sigma,
                    int flags, int nt)
{
  /* one iteration of gmm_learn's loop (yael/gmm.c:472-484) */
  float *p = malloc(sizeof(float) * ((size_t)n * k + 1));
  orc_gmm_compute_p(n, v, d, k, w, mu, sigma, p, flags, nt);
  int ret = gmm_handle_empty_port(n, v, d, k, mu, sigma, p);
  if (ret == 0) gmm_compute_params_port(n, v, p, d, k, w, mu, sigma, flags, nt);
  free(p);
  return ret;
}

int orc_gmm_learn(int d, int n, int k, int niter, const float *v, int nt, int seed, int nredo,
                  int flags, float *w, float *mu, float *sigma, int *iters_out)
{
  /* gmm_learn (yael/gmm.c:436-502): the reference's k-means, then EM */
  niter = niter == 0 ? 10000 : niter;
  float *dis = malloc(sizeof(float) * (size_t)(n + 1));
  orc_kmeans(d, n, k, niter, v, nt, seed, nredo, mu, dis, NULL, NULL, ORC_PORT, NULL);
  for (int j = 0; j < k; j++) w[j] = (float)(1.0 / k);
  double sig = 0;
  for (long i = 0; i < n; i++) sig += dis[i];
  sig /= n;
  for (long t = 0; t < (long)k * d; t++) sigma[t] = (float)sig;
  free(dis);
  if (flags & 32) niter = 0; /* GMM_FLAGS_PURE_KMEANS */
  float *p = malloc(sizeof(float) * ((size_t)n * k + 1));
  double key = 666, old_key;
  int iter, ret = 0;
  for (iter = 1; iter <= niter; iter++) {
    orc_gmm_compute_p(n, v, d, k, w, mu, sigma, p, flags, nt);
    if (gmm_handle_empty_port(n, v, d, k, mu, sigma, p) < 0) { ret = -1; break; }
    gmm_compute_params_port(n, v, p, d, k, w, mu, sigma, flags, nt);
    old_key = key;
    key = 0;
    for (long t = 0; t < (long)k * d; t++) key += mu[t];
    if (key == old_key) break;
  }
  if (iters_out) *iters_out = iter > niter ? niter : iter;
  free(p);
  return ret;
}

/* vlad_compute (yael/vlad.c:10-27): nearest centroid by nn (the blocked
 * argmin of knn_full, split over nt query slices as knn_full_thread does;
 * each vector's result is its own), then the residuals added in float, in
 * vector order */
void orc_vlad_compute(int k, int d, const float *centroids, int n, const float *v, float *desc,
                      int nt)
{
  int *assign = malloc(sizeof(int) * (size_t)(n + 1));
  float *dis = malloc(sizeof(float) * (size_t)(n + 1));
  orc_knn_port(2, n, k, d, 1, centroids, v, NULL, assign, dis, nt);
  memset(desc, 0, sizeof(float) * (size_t)k * d);
  for (long i = 0; i < n; i++)
    for (long j = 0; j < d; j++)
      desc[(long)assign[i] * d + j] += v[i * d + j] - centroids[(long)assign[i] * d + j];
  free(dis);
  free(assign);
}
