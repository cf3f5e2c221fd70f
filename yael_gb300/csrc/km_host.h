// Host side of the k-means control flow that replays the reference's
// random draws: its RNG helpers (yael/vector.c:134-155, yael/kmeans.c:15-24),
// the random initialisation's partial Fisher-Yates shuffle, and the
// empty-cluster split (yael/kmeans.c:166-209), planned from the counts and
// applied to just the centroid rows it touches.  Plain C++ (no CUDA), so the
// tests compile it on its own against the oracle.
#pragma once

#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

namespace yg {

// ---- reference RNG usage (yael/vector.c:134-155, yael/kmeans.c:15-24) --------

inline double drand_r_(unsigned *seed) { return rand_r(seed) / ((double)RAND_MAX + 1.0); }

// Kinderman-Monahan ratio of uniforms, with the reference's float / double
// roundings: u1, u2 and zz are held in float.
inline double gaussrand_r_(unsigned *seed) {
  const double magic = 1.71552776992141;  // 4 exp(-1/2) / sqrt(2)
  double z;
  for (;;) {
    const float u1 = (float)drand_r_(seed);
    const float u2 = (float)drand_r_(seed);
    z = magic * (u1 - .5) / u2;
    const float zz = (float)(z * z / 4.0);
    if (zz < -log(u2)) break;
  }
  return z;
}

// the first k entries of the partial Fisher-Yates shuffle of 0..n-1 that
// ivec_new_random_perm_r performs (only the first k swaps reach them)
inline void random_init_first_k(int n, int k, unsigned seed, long *sel) {
  // the permuted positions, in an open-addressing table (keys >= 0, -1 free):
  // at most k entries, so 4k slots stay sparse
  int cap = 16;
  while (cap < 4 * k) cap <<= 1;
  std::vector<int> key(cap, -1), val(cap);
  auto slot = [&](int i) {
    unsigned h = (unsigned)i * 2654435761u & (unsigned)(cap - 1);
    while (key[h] != -1 && key[h] != i) h = (h + 1) & (unsigned)(cap - 1);
    return h;
  };
  auto at = [&](int i) {
    const unsigned h = slot(i);
    return key[h] == i ? val[h] : i;
  };
  for (int i = 0; i < k && i < n; i++) {
    const int j = i + rand_r(&seed) % (n - i);
    const int vi = at(i), vj = at(j);
    sel[i] = vj;
    const unsigned h = slot(j);
    key[h] = j;
    val[h] = vi;
  }
}

inline double l1(const float *v, long n) {
  double s = 0;
  for (long i = 0; i < n; i++) s += fabs(v[i]);
  return s;
}
inline double l2(const float *v, long n) {
  double s = 0;
  for (long i = 0; i < n; i++) s += v[i] * v[i];
  return sqrt(s);
}
inline void mul_by(float *v, long n, double s) {
  for (long i = 0; i < n; i++) v[i] *= s;
}

// kmeans_reassign_empty (yael/kmeans.c:166-209) in two halves.  Which row
// each empty cluster copies depends on the counts and the random stream
// alone, so the plan (the draws, in the reference's order) comes first; the
// centroid arithmetic then runs on just the rows the plan touches (gathered
// from the device by the caller), not on a copy of all k rows.
struct SplitStep {
  int c, j;     // the empty cluster and the row it copies
  unsigned s2;  // the seed of its perturbation's Gaussian draws
};

inline int split_plan(int k, const int *nassign, unsigned seed,
                      std::vector<SplitStep> &plan) {
  int nre = 0;
  std::vector<float> p(k);
  for (int c = 0; c < k; c++) {
    // nassign^2 - 1 in int arithmetic (wraps for large clusters, like the reference)
    const unsigned sq = (unsigned)nassign[c] * (unsigned)nassign[c] - 1u;
    p[c] = nassign[c] < 2 ? 0.f : (float)(int)sq;
  }
  mul_by(p.data(), k, 1. / l1(p.data(), k));
  for (int c = 0; c < k; c++) {
    if (nassign[c] != 0) continue;
    nre++;
    double rd = drand_r_(&seed);
    int j;
    for (j = 0; j < k - 1; j++) {
      rd -= p[j];
      if (rd < 0) break;
    }
    plan.push_back(SplitStep{c, j, (unsigned)rand_r(&seed)});
    p[j] = 0;
    mul_by(p.data(), k, 1. / l1(p.data(), k));
  }
  return nre;
}

// One instance's steps on its rows: row r of the instance at R + slot[r] * d
// (every row a step names has a slot).  The same operations, in the same
// order, as on the full array: copy, norm of the source, perturbation
// added to the source and subtracted from the copy.
inline void split_apply(int d, const SplitStep *st, int nst, float *R, const int *slot) {
  std::vector<float> eps(d);
  for (int t = 0; t < nst; t++) {
    float *rc = R + (long)slot[st[t].c] * d, *rj = R + (long)slot[st[t].j] * d;
    if (rc != rj) memcpy(rc, rj, sizeof(float) * d);
    const double s = l2(rj, d) * 0.0000001;
    unsigned s2 = st[t].s2;
    for (int i = 0; i < d; i++) eps[i] = (float)gaussrand_r_(&s2);
    mul_by(eps.data(), d, s);
    for (int i = 0; i < d; i++) rj[i] += eps[i];
    for (int i = 0; i < d; i++) rc[i] -= eps[i];
  }
}

// Several instances' plans at once (instance pinst[b]'s steps from pat[b]
// to pat[b + 1]): rows, the global rows they touch (instance-major, k rows an
// instance), instance b's from first[b] on, each once, in the order its
// steps name them.
struct SplitRows {
  std::vector<long> rows;
  std::vector<int> first;
};

inline void split_rows(int k, const std::vector<SplitStep> &plan, const std::vector<int> &pinst,
                       const std::vector<int> &pat, SplitRows &sr) {
  std::vector<int> slot((size_t)k, -1);
  sr.rows.clear();
  sr.first.assign(pinst.size() + 1, 0);
  for (size_t b = 0; b < pinst.size(); b++) {
    sr.first[b] = (int)sr.rows.size();
    const int e = b + 1 < pinst.size() ? pat[b + 1] : (int)plan.size();
    for (int t = pat[b]; t < e; t++)
      for (int r : {plan[t].c, plan[t].j})
        if (slot[r] < 0) {
          slot[r] = (int)sr.rows.size() - sr.first[b];
          sr.rows.push_back((long)pinst[b] * k + r);
        }
    for (int t = pat[b]; t < e; t++) slot[plan[t].c] = slot[plan[t].j] = -1;
  }
  sr.first[pinst.size()] = (int)sr.rows.size();
}

// Every instance's steps on R, the rows of sr gathered in order (d floats each).
inline void split_apply_rows(int d, int k, const std::vector<SplitStep> &plan,
                             const std::vector<int> &pinst, const std::vector<int> &pat,
                             const SplitRows &sr, float *R) {
  std::vector<int> slot((size_t)k, -1);
  for (size_t b = 0; b < pinst.size(); b++) {
    const int e = b + 1 < pinst.size() ? pat[b + 1] : (int)plan.size();
    const long base = (long)pinst[b] * k;
    for (int r = sr.first[b]; r < sr.first[b + 1]; r++) slot[sr.rows[r] - base] = r - sr.first[b];
    split_apply(d, plan.data() + pat[b], e - pat[b], R + (size_t)sr.first[b] * d, slot.data());
    for (int r = sr.first[b]; r < sr.first[b + 1]; r++) slot[sr.rows[r] - base] = -1;
  }
}

}  // namespace yg
