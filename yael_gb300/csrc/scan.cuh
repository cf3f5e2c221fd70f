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

struct SetStats;

// Grouped passes (tc_scan only): many (queries, base) pairs in one persistent
// launch.  The pairs' packed queries are concatenated, and so are their packed
// bases, each pair's base padded so that its tiles (in the view the pass
// reads) start at a tile boundary.  A unit is one query tile of one pair
// against a range of that pair's base tiles.
struct GroupUnit {
  int q0;              // first query row of the tile (concatenated rows)
  int qend;            // end of the pair's query rows
  int t_begin, t_end;  // base tiles of this view of the concatenated base
  int bend;            // end of the pair's valid columns in this view
  int pair;            // index into the pair table
  int chunk;           // chunk of the pair's base (THRESH region; 0 for lists)
  int pad_;
};

// Per pair: where its candidates go (THRESH) and what the re-rank needs.
struct GroupPair {
  long cnt_off;   // region counters: cnt[cnt_off + r * nq + (row - qoff)]
  long cand_off;  // slots: candv/candi[cand_off + (r * nq + (row - qoff)) * cap + s]
  int qoff, nq;   // the pair's rows in the concatenated queries
  int boff;       // first row of the pair in the concatenated base (ids are relative)
  int nb;
  int nreg;       // THRESH regions per query (chunks * halves)
  int cap;        // THRESH slots per region
  const float *q;           // the pair's query rows (FP32, stride d): exact re-rank
  const float *b;           // the pair's base rows (FP32, stride d)
  int *out_idx;             // the pair's outputs, nq x k
  float *out_dis;
  const SetStats *bs;       // the pair's base statistics
};

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
  // grouped pass (units != null): the work units, in launch order, and the
  // pair table; the pass's nq / nb are those of the concatenated operands
  const GroupUnit *units = nullptr;
  int nunits = 0;
  const GroupPair *gpairs = nullptr;
  int max_ctas = 0;         // persistent passes: grid limit (0 = one CTA per SM)
  int f16 = 0;              // tensor-core passes: fp16 operands (else bf16)
  // tensor-core passes: bound of every wait (0: kWaitLimitNs), and a test
  // switch under which the producer issues no load, so that the consumers'
  // bounded waits expire (wait_limit_ns / test_withhold_loads in common.cuh)
  unsigned long long wait_ns = 0;
  int withhold = 0;
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
