// Candidate re-ranking, the exactness certificate, and the exhaustive FP64
// fallback.
//
// Contract (all distances in "dist space", ||q-b||^2 for L2, q.b for dot):
//   approx a(q,j)  -- value from the distance pass plus ||q||^2,
//                     |a - exact| <= eps[q]   (eps[q] = 0 for exact-class data)
//   exact e(q,j)   -- FP32 direct difference sum (q_c - b_c)^2, relative error
//                     <= rho; adjacent values closer than their error bound
//                     are re-evaluated in FP64 and ordered by (FP64, id)
//                     (for k = 1, L2, a near tie of the best two alone is
//                     first tried by the exact sign of their difference).
// The k results of a query are the k smallest (exact, id).  A query whose
// candidate set cannot be proven to contain them is re-computed by the
// exhaustive path (FP64 distances to every base row, radix select).
#pragma once
#include "prep.cuh"
#include "scan.cuh"

namespace yg {

struct RerankArgs {
  int nq = 0, nb = 0, d = 0, k = 0, metric = METRIC_L2;
  const float *q = nullptr;
  long ldq = 0;
  const float *b = nullptr;
  long ldb = 0;
  const double *qn64 = nullptr;  // ||q||^2 (L2)
  const float *eps = nullptr;    // per query, dist space
  const unsigned char *qexact = nullptr;  // per query: approx values are exact
  const SetStats *bstats = nullptr;       // base set statistics (device)
  ScanSel sel;                   // how the candidates were produced
  int *out_idx = nullptr;
  float *out_dis = nullptr;
  int *fail_list = nullptr;      // device list of failed queries
  int *fail_cnt = nullptr;       // device counter
  unsigned long long *n_cand = nullptr;  // device stats (may be null)
  int use_query_list = 0;        // when set, row r of the pass is query qlist[r]
  const int *qlist = nullptr;
  // optional: for each rejected query, an upper bound of its k-th smallest
  // exact distance (INFINITY when none was found), for the band pass
  float *kth_out = nullptr;
  // THRESH: expected candidates per query (0: unknown); shared memory is
  // sized for a few times this rather than for every region's capacity, and a
  // query with more candidates fails its certificate (the band pass follows)
  int m_expect = 0;
  // grouped re-rank (many pairs, THRESH): row q belongs to pair qpair[q], whose
  // table entry gives its candidate regions, base rows, statistics and outputs
  // (q, qn64, eps, qexact, thr, fail_list and kth_out stay indexed by q)
  const int *qpair = nullptr;
  const GroupPair *gpairs = nullptr;
  int max_candidates = 0;        // grouped: shared memory is sized for this many
};

int rerank(const RerankArgs &a, cudaStream_t st);

// eps[q] in dist space for the FP32 path (prec 0) or the BF16 path (prec 1),
// computed from the query's norm / residual and the base set statistics
// (grouped: those of the query's pair, gpairs[qpair[q]].bs).
// qexact[q] = query exact class and every base row exact class.
int compute_eps(int nq, int d, int prec, int metric, const double *qn64,
                const float *qres, const unsigned char *qflag, const SetStats *bstats,
                float *eps, unsigned char *qexact, cudaStream_t st,
                const int *qpair = nullptr, const GroupPair *gpairs = nullptr);

// eps[q] for the 3xBF16 split pass: the left-out q_lo.b_lo and residual
// terms plus the FP32 accumulation of 3*Kp1 + 16 products.
int compute_eps_split(int nq, int d, int metric, const double *qn64, const float *qlo,
                      const float *qres2, const unsigned char *qflag, const SetStats *bstats,
                      float *eps, unsigned char *qexact, cudaStream_t st);

// THRESH thresholds from a TOPC pass over a sample: thr[q] (v space) = the
// c-th smallest sampled value + 2 eps[q], rounded up.
int thresh_from_sample(int nq, int nchunk, int C, int c, const float *topv,
                       const float *eps, float *thr, cudaStream_t st);

// Band-pass thresholds: thr[q] (v space) such that every base row whose exact
// distance is <= kth[q] has approx value <= thr[q] (kth: an upper bound of the
// k-th exact distance of query q), widened so that the THRESH certificate
// (k-th <= thr + ||q||^2 - eps, with its relative slack) then holds.
int band_thresholds(int nq, int metric, const float *kth, const double *qn64, const float *eps,
                    float *thr, cudaStream_t st);

// Exhaustive exact path for the queries in qlist[0..nlist): FP64 distances to
// all nb base rows (optionally multiplied by weights), k smallest by
// (distance, id); NaN distances are skipped and short results padded the way
// yael/nn.c:511-519 does (k > 1) or with (-1, 1e30) (k == 1, nn.c:404-407).
// Row i of the output belongs to query qlist[i] (or i when qlist is null).
int exhaustive(int nlist, const int *qlist_dev, int nb, int d, int k, int metric,
               const float *q, long ldq, const float *b, long ldb, const float *w,
               int *out_idx, float *out_dis, void *scratch, size_t scratch_bytes,
               cudaStream_t st);

// scratch bytes per query for exhaustive()
inline size_t exhaustive_bytes_per_query(int nb) { return (size_t)nb * 8 + 64; }

constexpr int kMaxK = 4096;        // largest k the selection supports
constexpr int kMaxCandidates = 8192;  // largest candidate list re-ranked in one block

}  // namespace yg
