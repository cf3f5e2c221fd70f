// 16-bit tensor-core (tcgen05 kind::f16) producer of distance tiles with the
// fused selection of scan.cuh: bf16 operands, or fp16 ones (same layout, 8x
// finer rounding, the same tensor rate) where the data range allows.
//
// Operands are packed once per call: queries as bf16(-2 q) (L2) or bf16(q)
// (dot), base rows as bf16(b); both padded to Kp = 64*ceil(d/64) columns.  For
// L2 a 16-column side block carries ||b||^2 as three bf16 parts (hi, mid, lo;
// their exact sum is the FP32 norm) and a matching block of ones on the query
// side, so the MMA itself produces v = ||b||^2 - 2 q.b in FP32.
#pragma once
#include <cuda_bf16.h>

#include "prep.cuh"
#include "scan.cuh"

namespace yg {

constexpr int TC_TILE_M = 128;  // query rows per tile (TMEM lanes)
constexpr int TC_TILE_N = 256;  // base rows per tile (TMEM columns)

struct TcOperands {
  int d = 0, Kp = 0, metric = METRIC_L2;
  const __nv_bfloat16 *q = nullptr;   // [nq][Kp]
  const __nv_bfloat16 *qn = nullptr;  // [nq][16]   (L2)
  const __nv_bfloat16 *b = nullptr;   // [rows][Kp]
  const __nv_bfloat16 *bn = nullptr;  // [rows][16] (L2)
  long b_rows = 0;                    // packed base rows
  long b_step = 1;                    // scan row j reads packed row j*b_step
  int split = 0;                      // 1: 3xBF16 split packing (Kp = 3 * Kp1)
  int f16 = 0;                        // 1: IEEE fp16 operands (the same layout as bf16)
  int *err = nullptr;                 // device flag set when a bounded wait expires
};

// true when the tensor-core pass handles this dimension (any d: a query tile
// of Kp <= 256 stays resident in shared memory, larger ones are streamed)
bool tc_supported(int d);

// split = 0: bf16 packing; split = 1: 3xBF16 split packing (prep.cuh); lonorm
// (split only) receives ||lo|| per row.  f16 = 1 (not with split): fp16 packing
// (prep_rows), for data whose range fp16 holds; both operands of a pass must
// use the same encoding.
int tc_prepare_queries(const float *q, long ldq, int nq, int d, int metric, Workspace &ws,
                       int slot_pack, int slot_norm, TcOperands *op, double *qn64,
                       unsigned char *qflag, float *qres, int split, float *lonorm,
                       cudaStream_t st, int f16 = 0);

int tc_prepare_base(const float *b, long ldb, int nb, int d, int metric, Workspace &ws,
                    int slot_pack, int slot_norm, int slot_res, TcOperands *op, float *bn32,
                    SetStats *bs, int split, cudaStream_t st, int f16 = 0);

// strided view of the packed base (every stride-th row, nrows rows)
int tc_base_view(const TcOperands &full, int stride, int nrows, TcOperands *out);

// Base rows [row0, row0 + n) uploaded part by part: the bf16 buffers of the
// whole base are allocated first (tc_alloc_base, plain packing), each part is
// packed when it has arrived (tc_prepare_base_range, its statistics folded
// into bs), and a pass over one part reads a slice (tc_base_slice).
int tc_alloc_base(int nb, int d, int metric, Workspace &ws, int slot_pack, int slot_norm,
                  int slot_res, TcOperands *op, float **res);
int tc_prepare_base_range(const float *b, long ldb, long row0, int n, int d, int metric,
                          const TcOperands &op, float *bn32, float *res, SetStats *bs,
                          cudaStream_t st);
int tc_base_slice(const TcOperands &full, long row0, int nrows, TcOperands *out);

int tc_scan(const TcOperands &op, int nq, int nb, const ScanSel &sel, cudaStream_t st);

}  // namespace yg
