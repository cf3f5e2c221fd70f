// tcgen05 BF16 distance tiles with the fused selection (see tc_scan.cuh and
// tc_kernel.cuh): operand packing, the choice of kernel variant, and the
// resident-query-tile single-CTA instantiation.
#include <stdlib.h>

#include "tc_kernel.cuh"

namespace yg {

bool tc_supported(int d) { return d >= 1; }

int tc_prepare_queries(const float *q, long ldq, int nq, int d, int metric, Workspace &ws,
                       int slot_pack, int slot_norm, TcOperands *op, double *qn64,
                       unsigned char *qflag, float *qres, int split, float *lonorm,
                       cudaStream_t st, int f16) {
  if (split && f16) {
    set_error(E_ARG, "tc_prepare_queries: the split packing is bf16 only");
    return E_ARG;
  }
  const int Kp1 = ((d + 63) / 64) * 64, Kp = split ? 3 * Kp1 : Kp1;
  void *pack, *norm = nullptr;
  YG_CHECK(ws.get(slot_pack, (size_t)nq * Kp * 2, &pack));
  if (metric == METRIC_L2) YG_CHECK(ws.get(slot_norm, (size_t)nq * 32, &norm));
  const float scale = metric == METRIC_L2 ? -2.f : 1.f;
  const int nmode = metric == METRIC_L2 ? 2 : 0;
  if (split)
    YG_CHECK(prep_rows_split(q, ldq, nq, d, scale, 0, qn64, nullptr, qflag, lonorm, qres,
                             (__nv_bfloat16 *)pack, Kp1, (__nv_bfloat16 *)norm, nmode, nullptr,
                             st));
  else
    YG_CHECK(prep_rows(q, ldq, nq, d, scale, qn64, nullptr, qflag, qres, (__nv_bfloat16 *)pack,
                       Kp, (__nv_bfloat16 *)norm, nmode, nullptr, st, 8, f16));
  op->d = d;
  op->Kp = Kp;
  op->metric = metric;
  op->split = split;
  op->f16 = f16;
  op->q = (const __nv_bfloat16 *)pack;
  op->qn = (const __nv_bfloat16 *)norm;
  return OK;
}

int tc_prepare_base(const float *b, long ldb, int nb, int d, int metric, Workspace &ws,
                    int slot_pack, int slot_norm, int slot_res, TcOperands *op, float *bn32,
                    SetStats *bs, int split, cudaStream_t st, int f16) {
  if (split && f16) {
    set_error(E_ARG, "tc_prepare_base: the split packing is bf16 only");
    return E_ARG;
  }
  const int Kp1 = ((d + 63) / 64) * 64, Kp = split ? 3 * Kp1 : Kp1;
  void *pack, *norm = nullptr, *res;
  YG_CHECK(ws.get(slot_pack, (size_t)nb * Kp * 2, &pack));
  if (metric == METRIC_L2) YG_CHECK(ws.get(slot_norm, (size_t)nb * 32, &norm));
  YG_CHECK(ws.get(slot_res, (size_t)nb * 4, &res));
  const int nmode = metric == METRIC_L2 ? 1 : 0;
  if (split)
    YG_CHECK(prep_rows_split(b, ldb, nb, d, 1.f, 1, nullptr, bn32, nullptr, nullptr, (float *)res,
                             (__nv_bfloat16 *)pack, Kp1, (__nv_bfloat16 *)norm, nmode, bs, st));
  else
    YG_CHECK(prep_rows(b, ldb, nb, d, 1.f, nullptr, bn32, nullptr, (float *)res,
                       (__nv_bfloat16 *)pack, Kp, (__nv_bfloat16 *)norm, nmode, bs, st, 8, f16));
  op->d = d;
  op->Kp = Kp;
  op->metric = metric;
  op->split = split;
  op->f16 = f16;
  op->b = (const __nv_bfloat16 *)pack;
  op->bn = (const __nv_bfloat16 *)norm;
  op->b_rows = nb;
  op->b_step = 1;
  return OK;
}

int tc_prepare_base_range(const float *b, long ldb, long row0, int n, int d, int metric,
                          const TcOperands &op, float *bn32, float *res, SetStats *bs,
                          cudaStream_t st) {
  if (n <= 0) return OK;
  const int nmode = metric == METRIC_L2 ? 1 : 0;
  __nv_bfloat16 *pack = const_cast<__nv_bfloat16 *>(op.b) + row0 * op.Kp;
  __nv_bfloat16 *norm = op.bn ? const_cast<__nv_bfloat16 *>(op.bn) + row0 * 16 : nullptr;
  return prep_rows(b + row0 * ldb, ldb, n, d, 1.f, nullptr, bn32 + row0, nullptr, res + row0,
                   pack, op.Kp, norm, nmode, bs, st, 8, op.f16);
}

int tc_alloc_base(int nb, int d, int metric, Workspace &ws, int slot_pack, int slot_norm,
                  int slot_res, TcOperands *op, float **res) {
  const int Kp = ((d + 63) / 64) * 64;
  void *pack, *norm = nullptr, *r;
  YG_CHECK(ws.get(slot_pack, (size_t)nb * Kp * 2, &pack));
  if (metric == METRIC_L2) YG_CHECK(ws.get(slot_norm, (size_t)nb * 32, &norm));
  YG_CHECK(ws.get(slot_res, (size_t)nb * 4, &r));
  op->d = d;
  op->Kp = Kp;
  op->metric = metric;
  op->split = 0;
  op->b = (const __nv_bfloat16 *)pack;
  op->bn = (const __nv_bfloat16 *)norm;
  op->b_rows = nb;
  op->b_step = 1;
  *res = (float *)r;
  return OK;
}

int tc_base_slice(const TcOperands &full, long row0, int nrows, TcOperands *out) {
  *out = full;
  out->b = full.b + row0 * full.b_step * full.Kp;
  if (full.bn) out->bn = full.bn + row0 * full.b_step * 16;
  out->b_rows = nrows;
  return OK;
}

int tc_base_view(const TcOperands &full, int stride, int nrows, TcOperands *out) {
  *out = full;
  out->b_step = full.b_step * stride;
  out->b_rows = nrows;
  return OK;
}

int tc_dispatch_r1(const TcOperands &op, int nq, int nb, const ScanSel &sel, cudaStream_t st) {
  return tck::dispatch_metric<false, false>(op, nq, nb, sel, st);
}

int tc_scan(const TcOperands &op, int nq, int nb, const ScanSel &sel_in, cudaStream_t st) {
  if (nq <= 0 || nb <= 0) return OK;
  ScanSel sel = sel_in;
  sel.f16 = op.f16;  // the MMA's operand format
  sel.wait_ns = wait_limit_ns();
  sel.withhold = test_withhold_loads() ? 1 : 0;
  if (sel.units) {
    // grouped pass: the streamed-query persistent form walks the unit table;
    // ids of list passes would not be relative to their pair
    if (sel.mode == SCAN_TOPC) {
      set_error(E_UNSUPPORTED, "tc_scan: grouped pass with id lists");
      return E_UNSUPPORTED;
    }
    // the query tile stays resident when it fits beside a ring of 3 stages
    const bool res = op.Kp <= 256 || (op.Kp <= 384 && tck::make_layout(op.Kp / 64, 3, sel.mode,
                                                                       sel.mode == SCAN_THRESH ? 1 : sel.C,
                                                                       false, false)
                                                          .total <= 227 * 1024);
    return res ? tc_dispatch_r1(op, nq, nb, sel, st) : tc_dispatch_s1(op, nq, nb, sel, st);
  }
  // CTA pairs (one 256-row MMA over two SMs) halve the per-SM base traffic
  // but add a cross-SM handoff to every accumulator; measured on the 1M x 10k
  // k-NN pass they are slower (3.98 ms vs 2.87 ms), so single CTAs are the
  // default and YAEL_GPU_TC_PAIR=1 selects pairs
  static const bool pair_env = [] {
    const char *e = getenv("YAEL_GPU_TC_PAIR");
    return e && e[0] == '1';
  }();
  const bool pair = pair_env && nq > TC_TILE_M;
  // the query tile stays resident in shared memory when a ring of at least
  // three stages still fits beside it (always for K <= 256; for the 3xBF16
  // split of d <= 128, K = 384, with short lists); else it is streamed with
  // every K block
  // A unit of at most two base tiles reuses a resident tile at most twice: then
  // the streamed form, whose persistent grid also saves a CTA start-up
  // (barriers, TMEM allocation, first loads) per query tile, is faster.
  const bool few_tiles = !pair && sel.tiles_per_chunk <= 2;
  bool resident = op.Kp <= 256 && !few_tiles;
  if (!resident && !few_tiles && op.Kp <= 384) {
    const int C = sel.mode == SCAN_THRESH ? 1 : sel.C;
    resident = tck::make_layout(op.Kp / 64, 3, sel.mode, C, false, false).total <= 227 * 1024;
  }
  if (!resident)  // query tile too large to stay resident: streamed per K block
    return pair ? tc_dispatch_s2(op, nq, nb, sel, st) : tc_dispatch_s1(op, nq, nb, sel, st);
  return pair ? tc_dispatch_r2(op, nq, nb, sel, st) : tc_dispatch_r1(op, nq, nb, sel, st);
}

}  // namespace yg
