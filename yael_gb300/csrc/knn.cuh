// Device-level exact k-NN driver shared by the drop-in entry points, the
// k-means assignment step and the batched calls.
#pragma once
#include "select.cuh"
#include "../../include/yael_gpu.h"

namespace yg {

// A base that arrives part by part (host -> device upload overlapped with the
// passes): part i is rows [row0[i], row0[i+1]); ready[i] is recorded on the
// copy stream once it has landed.  The pipeline packs each part after waiting
// for it, samples the thresholds from part 0 and runs the main pass part by
// part; error bounds for the re-rank are taken over the whole base.
struct BaseUpload {
  static constexpr int kMaxParts = 8;
  int nparts = 0;
  long row0[kMaxParts + 1] = {};
  cudaEvent_t ready[kMaxParts] = {};
  bool packed[kMaxParts] = {};
};

struct KnnJob {
  int nq = 0, nb = 0, d = 0, k = 1;
  int metric = METRIC_L2;
  int prec = PREC_FP32;
  const float *q = nullptr;  // device, nq x d (row stride ldq)
  long ldq = 0;
  const float *b = nullptr;  // device, nb x d (row stride ldb)
  long ldb = 0;
  const float *w = nullptr;  // device base weights or null
  int *out_idx = nullptr;    // device nq x k
  float *out_dis = nullptr;  // device nq x k
  // band pass (internal): when set, a THRESH pass with per-query thresholds
  // from band_kth[q], an upper bound of the query's k-th exact distance
  const float *band_kth = nullptr;
  // Known before the pass (the k-means assignment from its second iteration
  // on): per query an upper bound of its k-th exact distance, here its exact
  // distance to its previous centroid, which has moved.  The pass is then a
  // THRESH pass with thresholds from these bounds (no sample pass; short
  // candidate regions, whose overflow sends the query to the band pass).
  const float *prior_kth = nullptr;
  int level = 0;  // nesting depth of the later-chance passes (workspace slots)
  BaseUpload *upload = nullptr;  // base arriving part by part (BF16 pass only)
  // CUDA-event timing of the passes (optional)
  int timing = 0;
  float ms_scan = 0, ms_sample = 0, ms_rerank = 0;
  float ms_second = 0;  // all later-chance passes (band, split, exhaustive)
  int scan_launches = 0;
  // filled on return
  int n_fallback = 0;   // queries recomputed by the exhaustive FP64 path
  int n_band = 0;       // rejected queries re-run through a band pass
  int n_second = 0;     // queries re-run through the 3xBF16 split pass
  long long n_cand = 0;
  int exact_class = 0;
  // Deferred certificate check (the k-means assignment): with defer = 1 a call
  // whose queries fit one batch (and that runs no autotuner trial) returns
  // right after the re-rank with pending = 1, its status block on its way to
  // the context's pinned buffer; knn_resolve() settles the rejected queries
  // once the caller has synchronised the stream.
  int defer = 0;
  int pending = 0;
  int *fail_dev = nullptr;  // device list of the rejected queries (pending)
};

// Runs the whole pipeline on stream st using the calling thread's workspace.
int knn_device(KnnJob &job, Ctx *ctx, cudaStream_t st);

// For a pending job (defer): reads its status (st must have been synchronised
// since the call), runs the rejected queries through the whole pipeline and
// writes their results; n_band counts them.  No-op when nothing is pending.
int knn_resolve(KnnJob &job, Ctx *ctx, cudaStream_t st);

// One k-NN call on the calling thread's context: host arrays (copied in and
// out) or, with opts->device_ptrs, device arrays on opts->stream (NULL = the
// thread's stream); fills opts' counters.
int knn_host(int metric, int nq, int nb, int d, int k, const float *b, const float *q,
             const float *w, int *assign, float *dis, int prec, yael_gpu_knn_opts *opts);

// Grouped batched k-NN (group.cu): every pair of a batch through one launch
// per pass.  Eligible: device arrays, the BF16 pass, k >= 9 (the threshold
// form of the selection); YAEL_GPU_BATCH_GROUPED=0 turns it off.
struct GroupCounters {
  long long n_band = 0, n_second = 0, n_fallback = 0, n_cand = 0;
  int all_exact = 1;
};
bool knn_grouped_eligible(int d, int k, int prec, int device_ptrs);
int knn_grouped(int npairs, const yael_gpu_knn_pair *pairs, int d, int k, int metric,
                cudaStream_t st, GroupCounters *gc);

// workspace slots (each slot is one grow-only device buffer per host thread)
enum WsSlot : int {
  WS_QN64 = 0, WS_QFLAG, WS_QRES, WS_BN32, WS_SMALL, WS_EPS, WS_QEXACT,
  WS_TOPV, WS_TOPI, WS_THR, WS_CNT, WS_FAIL, WS_STOPV, WS_STOPI, WS_EXH,
  WS_QPACK, WS_BPACK, WS_QNORMP, WS_BNORMP, WS_BRES,
  WS_QLO = 24, WS_BPACK3, WS_BNORMP3, WS_BRES3, WS_KTH,
  WS_H_B = 40, WS_H_Q, WS_H_W, WS_H_IDX, WS_H_DIS, WS_H_EXTRA,
  WS_KM0 = 60,  // k-means / hkm slots start here
  // compacted queries of a later-chance pass, per nesting level
  WS_SC0 = 100,
  WS_SC_PER_LEVEL = 5,  // + 0 map, 1 rows, 2 ids, 3 distances, 4 k-th bounds
  WS_DEF0 = 130,        // knn_resolve: + 0 map, 1 rows, 2 ids, 3 distances
};

}  // namespace yg
