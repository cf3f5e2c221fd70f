// The fused "distance tile + per-query selection" pass.  Two producers of
// distance tiles share the selection contract:
//   * simt_scan  -- FP32 FFMA tiles on the CUDA cores (the plain path)
//   * tc_scan    -- BF16 tcgen05 tiles with FP32 accumulation in TMEM
// Both evaluate, for query row q and base row j,
//     v(q, j) = ||b_j||^2 - 2 q.b_j        (L2; ||q||^2 is added later)
//     v(q, j) = q.b_j                       (dot product)
// and never write the nq x nb matrix.  Selection modes:
//   TOPC   -- every (query, base chunk) keeps its C smallest (v, j) in
//             lexicographic order (strict '<' over increasing j), written to
//             topv/topi[(chunk * nq + q) * C + s], ascending.
//   THRESH -- every (q, j) with v <= thr[q] is appended to a candidate
//             region owned by one thread: region r = chunk * halves + column
//             half (halves = 2 for the CUDA-core producer, whose two threads
//             of a row split the columns; 1 for the tensor-core one), slots
//             candv/candi[(r * nq + q) * cap + s], count cnt[r * nq + q] (all
//             hits, including those that did not fit in cap).  No atomics:
//             each (region, query) has exactly one writer.
#pragma once
#include "common.cuh"

namespace yg {

// SCAN_TOPV is SCAN_TOPC without ids (only the values are kept and written;
// used where a rank statistic of the distances is all that is needed).
enum ScanMode : int { SCAN_TOPC = 0, SCAN_THRESH = 1, SCAN_TOPV = 2 };
enum Metric : int { METRIC_L2 = 2, METRIC_DOT = 16 };

struct ScanSel {
  int mode = SCAN_TOPC;
  int C = 1;
  int nchunk = 1;           // base chunks
  int tiles_per_chunk = 1;  // base tiles per chunk
  float *topv = nullptr;
  int *topi = nullptr;
  const float *thr = nullptr;
  int *cnt = nullptr;
  float *candv = nullptr;
  int *candi = nullptr;
  int cap = 0;              // THRESH: slots per (region, query)
  int halves = 2;           // THRESH: regions per chunk (column halves of a row)
  int id_off = 0;           // added to every emitted base id (a pass over a base slice)
  __host__ __device__ int nregion() const { return nchunk * halves; }
};

// FP32 CUDA-core producer.  q: nq rows (stride ldq floats); b: nb rows (stride
// ldb floats); bn: ||b||^2 as float with stride bn_stride (L2 only).
// Base tiles are 128 rows.  Reported base ids are j (row index in this view).
constexpr int SIMT_TILE_N = 128;
int simt_scan(const float *q, long ldq, int nq, const float *b, long ldb, int nb,
              int d, const float *bn, long bn_stride, int metric, const ScanSel &sel,
              cudaStream_t st);

// number of base chunks that gives enough CTAs for the GPU
int choose_chunks(int n_query_tiles, int n_base_tiles, int num_sms, int ctas_per_sm,
                  int min_tiles_per_chunk);

}  // namespace yg
