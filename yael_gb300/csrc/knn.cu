// Exact k-NN: the device pipeline (prepare -> fused distance pass with
// selection -> re-rank + certificate -> exhaustive fallback) and the nn.h
// drop-in entry points (yael/nn.h:41-83).
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <memory>

#include "alt.cuh"
#include "autotune.cuh"
#include "knn.cuh"
#include "tc_scan.cuh"
#include "../../include/yael_gpu.h"

namespace yg {

namespace {

struct Small {
  SetStats bs;   // base statistics of the plain (bf16 / fp32) packing
  SetStats bs3;  // base statistics of the split 3xBF16 packing
  int fail_cnt;
  int tc_err;    // set by a tensor-core pass whose bounded wait expired
  unsigned long long n_cand;
};

static_assert(sizeof(Small) <= kPinnedStatusBytes, "status block larger than its pinned copy");

__global__ void small_init_kernel(Small *s) {
  memset(s, 0, sizeof(Small));
  s->bs.all_exact = 1;
  s->bs3.all_exact = 1;
}

// the device status block, read through the context's pinned buffer
int read_small(Ctx *ctx, const Small *dsmall, cudaStream_t st, Small *out) {
  void *pin;
  YG_CHECK(ctx_pinned_status(ctx, &pin));
  YG_CUDA(cudaMemcpyAsync(pin, dsmall, sizeof(Small), cudaMemcpyDeviceToHost, st));
  YG_CUDA(cudaStreamSynchronize(st));
  memcpy(out, pin, sizeof(Small));
  return OK;
}

// packed base operands of the tensor-core passes (the split one is built on
// first use by the second-chance pass)
struct BaseOps {
  TcOperands plain, split;
  bool has_plain = false, has_split = false;
  float *bn32 = nullptr, *res = nullptr;  // plain packing: per-row norms and residuals
};

template <typename T>
int ws_get(Workspace &ws, int slot, size_t count, T **p) {
  void *v = nullptr;
  YG_CHECK(ws.get(slot, count * sizeof(T), &v));
  *p = reinterpret_cast<T *>(v);
  return OK;
}

int pow2_at_least(int x) {
  int p = 1;
  while (p < x) p <<= 1;
  return p;
}

__global__ void gather_rows_kernel(const float *src, long ld, const int *map, int n, int d,
                                   float *dst) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long)n * d) return;
  const long r = i / d;
  dst[i] = src[(long)map[r] * ld + (i - r * d)];
}

__global__ void scatter_rows_kernel(const int *sidx, const float *sdis, const int *map, int n,
                                    int k, int *didx, float *ddis) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long)n * k) return;
  const long r = i / k;
  const long o = (long)map[r] * k + (i - r * k);
  didx[o] = sidx[i];
  ddis[o] = sdis[i];
}

// k-th bounds of the compacted queries: the smaller of the bound the pass was
// given (band passes) and the one its re-rank found
__global__ void gather_kth_kernel(const float *in_kth, const float *out_kth, const int *map, int n,
                                  float *dst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float o = out_kth[map[i]];
  dst[i] = in_kth ? fminf(in_kth[map[i]], o) : o;
}

// per-thread list length of a TOPC pass: k when the distances are exact, else
// an oversampled list whose extra entries give the certificate its margin.
// k = 1 (k-means assignment) does not depend on exactness: lists of eight.
// Measured on the large k-means configuration (10M points, 65,536 crowded
// centroids, fp16 operands): lists of two reject 35-61% of the points (their
// second entry sits inside the error band), lists of eight 0.2-16%, and the
// band pass then costs a few ms instead of ~100; the longer lists slow the
// distance pass by 1.35x, a net 1.5x per iteration (369 -> 243 ms).
// candidate slots per THRESH region of a pass with prior thresholds: the
// nearest centroid and the few others within the error band of the bound,
// as many as the short re-rank's 32 slots hold (two regions per chunk)
int prior_cap(int nchunk) { return imax(8, 32 / (2 * nchunk)); }

int list_length(int k, int exact, int nb) {
  (void)nb;
  if (k == 1) return 8;
  if (exact) return k;
  return k <= 4 ? 8 : 2 * k;
}

__global__ void fill_f32(float *p, long n, float v) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}

// CUDA events around a pass, on the launching stream; elapsed times are read
// after the stream synchronizes at the end of the batch (no extra host sync)
struct PassTimer {
  cudaEvent_t a = nullptr, b = nullptr;
  float *dst;
  float last = 0.f;  // the elapsed time of this pass, after collect()
  PassTimer(bool enable, cudaStream_t st, float *out, bool start_now = true)
      : dst(enable ? out : nullptr) {
    if (dst) {
      cudaEventCreate(&a);
      cudaEventCreate(&b);
      if (start_now) cudaEventRecord(a, st);
    }
  }
  void start(cudaStream_t st) {
    if (dst) cudaEventRecord(a, st);
  }
  void stop(cudaStream_t st) {
    if (dst) cudaEventRecord(b, st);
  }
  void collect() {  // call after the stream has been synchronized
    if (!dst) return;
    float ms = 0;
    if (cudaEventElapsedTime(&ms, a, b) == cudaSuccess) {
      *dst += ms;
      last = ms;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    dst = nullptr;
  }
  ~PassTimer() { collect(); }
};

// distance pass on whichever producer the precision selects
int scan(const KnnJob &job, const float *q, int nq, const float *b, long ldb, int nb,
         const float *bn, long bn_stride, const TcOperands *tc, const ScanSel &sel,
         cudaStream_t st) {
  if (job.prec != PREC_FP32) return tc_scan(*tc, nq, nb, sel, st);
  return simt_scan(q, job.ldq, nq, b, ldb, nb, job.d, bn, bn_stride, job.metric, sel, st);
}

// Candidate layout of a band pass over nq queries: chunks of the base and the
// per-region capacity.  A band holds every base row whose exact distance can
// still be <= the query's k-th; ctot bounds its size (more fails the query).
struct BandLayout {
  int nchunk, tiles_per_chunk, cap, halves;
  size_t bytes_per_query() const {
    return (size_t)nchunk * halves * cap * 8 + (size_t)nchunk * halves * 4 + 64;
  }
};

BandLayout band_layout(int nq, int nb, int k, int tile_m, int tile_n, int halves, int num_sms) {
  const int nqt = (int)ceil_div(nq, tile_m), ntb = (int)ceil_div(nb, tile_n);
  BandLayout L;
  L.halves = halves;
  L.nchunk = imin(choose_chunks(nqt, ntb, num_sms, 1, 4), 1024);
  L.tiles_per_chunk = (int)ceil_div(ntb, L.nchunk);
  L.nchunk = (int)ceil_div(ntb, L.tiles_per_chunk);
  const int ctot = imin(kMaxCandidates / 2, imax(512, 4 * k));
  L.cap = pow2_at_least(imax(8, 2 * ctot / (halves * L.nchunk)));
  return L;
}

int knn_batches(KnnJob &job, Ctx *ctx, cudaStream_t st, Small *dsmall, BaseOps *bops,
                int bexact);

// Chunk layout of a main pass over a base that arrives part by part: part i
// gets nch[i] chunks of tpc[i] tiles, its lists / regions start at chunk
// first[i]; the total is returned.
int part_chunks(const BaseUpload &up, int kind, int prec, int C, int nqt, int tile_n, int slots,
                int cmax, int *nch, int *tpc, int *first, int *ticket) {
  int tot = 0;
  for (int i = 0; i < up.nparts; i++) {
    const int ntb = (int)ceil_div(up.row0[i + 1] - up.row0[i], tile_n);
    // each part shape is tuned on its own pass time (the re-rank cost does
    // not depend on the chunk count)
    const int c = tune_chunks(TuneKey{kind, prec, nqt, ntb, C},
                              imin(cmax, choose_chunks(nqt, ntb, slots, 1, 4)), cmax, slots,
                              &ticket[i]);
    tpc[i] = (int)ceil_div(ntb, c);
    nch[i] = (int)ceil_div(ntb, tpc[i]);
    first[i] = tot;
    tot += nch[i];
  }
  return tot;
}

// the main pass over every part of an uploading base: each part is packed
// once it has landed, then scanned into its own lists / regions with ids
// offset by its first row
int scan_parts(const KnnJob &job, BaseUpload &up, const BaseOps &bops, Small *dsmall,
               const TcOperands &tcq, int nq, const ScanSel &sel, const int *nch,
               const int *tpc, const int *first, std::unique_ptr<PassTimer> *ptm,
               cudaStream_t st) {
  for (int i = 0; i < up.nparts; i++) {
    const long r0 = up.row0[i];
    const int n = (int)(up.row0[i + 1] - r0);
    if (!up.packed[i]) {
      YG_CUDA(cudaStreamWaitEvent(st, up.ready[i], 0));
      YG_CHECK(tc_prepare_base_range(job.b, job.ldb, r0, n, job.d, job.metric, bops.plain,
                                     bops.bn32, bops.res, &dsmall->bs, st));
      up.packed[i] = true;
    }
    ScanSel si = sel;
    si.nchunk = nch[i];
    si.tiles_per_chunk = tpc[i];
    si.id_off = (int)r0;
    if (sel.mode == SCAN_THRESH) {
      const long reg = (long)first[i] * sel.halves;
      si.cnt = sel.cnt + reg * nq;
      si.candv = sel.candv + reg * nq * sel.cap;
      si.candi = sel.candi + reg * nq * sel.cap;
    } else {
      si.topv = sel.topv + (long)first[i] * nq * sel.C;
      si.topi = sel.topi + (long)first[i] * nq * sel.C;
    }
    TcOperands tp;
    YG_CHECK(tc_base_slice(tcq, r0, n, &tp));
    if (ptm[i]) ptm[i]->start(st);
    YG_CHECK(tc_scan(tp, nq, n, si, st));
    if (ptm[i]) ptm[i]->stop(st);
  }
  return OK;
}

// one batch of queries (all buffers sized for nq of this batch)
int knn_batch(KnnJob &job, Ctx *ctx, cudaStream_t st, Small *dsmall, BaseOps *bops,
              int bstats_exact) {
  Workspace &ws = ctx->ws;
  const int nq = job.nq, nb = job.nb, d = job.d, k = job.k;
  const bool bf16 = job.prec != PREC_FP32;  // a tensor-core pass (bf16 or split)
  const bool split = job.prec == PREC_BF16X3;
  double *qn64;
  unsigned char *qflag, *qexact;
  float *qres = nullptr, *eps, *bn32 = nullptr;
  YG_CHECK(ws_get(ws, WS_QN64, nq, &qn64));
  YG_CHECK(ws_get(ws, WS_QFLAG, nq, &qflag));
  YG_CHECK(ws_get(ws, WS_QEXACT, nq, &qexact));
  YG_CHECK(ws_get(ws, WS_EPS, nq, &eps));
  YG_CHECK(ws_get(ws, WS_QRES, nq, &qres));
  YG_CHECK(ws_get(ws, WS_BN32, nb, &bn32));  // written by knn_device

  TcOperands tcq;
  float *qlo = nullptr;
  std::unique_ptr<NvtxRange> nv(new NvtxRange("knn.pack_queries"));
  if (bf16) {
    tcq = split ? bops->split : bops->plain;
    if (split) YG_CHECK(ws_get(ws, WS_QLO, nq, &qlo));
    YG_CHECK(tc_prepare_queries(job.q, job.ldq, nq, d, job.metric, ws, WS_QPACK, WS_QNORMP,
                                &tcq, qn64, qflag, qres, split ? 1 : 0, qlo, st,
                                job.prec == PREC_FP16));
  } else {
    YG_CHECK(prep_rows(job.q, job.ldq, nq, d, 1.f, qn64, nullptr, qflag, qres, nullptr, 0,
                       nullptr, 0, nullptr, st));
  }
  if (split)
    YG_CHECK(compute_eps_split(nq, d, job.metric, qn64, qlo, qres, qflag, &dsmall->bs3, eps,
                               qexact, st));
  else
    YG_CHECK(compute_eps(nq, d, job.prec, job.metric, qn64, qres, qflag, &dsmall->bs, eps,
                         qexact, st));

  nv.reset(new NvtxRange(job.band_kth ? "knn.band_pass" : "knn.distance_pass"));
  int *fail_list;
  YG_CHECK(ws_get(ws, WS_FAIL, nq, &fail_list));
  YG_CUDA(cudaMemsetAsync(&dsmall->fail_cnt, 0, sizeof(int), st));

  RerankArgs ra;
  ra.nq = nq; ra.nb = nb; ra.d = d; ra.k = k; ra.metric = job.metric;
  ra.q = job.q; ra.ldq = job.ldq; ra.b = job.b; ra.ldb = job.ldb;
  ra.qn64 = qn64; ra.eps = eps; ra.qexact = qexact; ra.bstats = &dsmall->bs;
  ra.out_idx = job.out_idx; ra.out_dis = job.out_dis;
  ra.fail_list = fail_list; ra.fail_cnt = &dsmall->fail_cnt; ra.n_cand = &dsmall->n_cand;
  float *kth;
  YG_CHECK(ws_get(ws, WS_KTH, nq, &kth));
  ra.kth_out = kth;
  const bool band = job.band_kth != nullptr;
  const bool prior = !band && job.prior_kth != nullptr;

  const bool timed = job.timing || trace_enabled();
  const int tile_n = bf16 ? TC_TILE_N : SIMT_TILE_N;
  const int tile_m = bf16 ? TC_TILE_M : 128;
  const int nqt = (int)ceil_div(nq, tile_m);
  const int ntb = (int)ceil_div(nb, tile_n);
  const int ctas_per_sm = 1;
  // oversampling for inexact distances: the certificate needs a margin between
  // the k-th exact value and the first excluded candidate
  const int c_needed = list_length(k, bstats_exact, nb);

  std::unique_ptr<PassTimer> tm_scan, tm_sample;
  int scan_ticket = -1, sample_ticket = -1;  // autotuner trials (autotune.cuh)
  ScanSel sel;
  BaseUpload *up = (job.upload && !band && bf16 && !split) ? job.upload : nullptr;
  int pnch[BaseUpload::kMaxParts], ptpc[BaseUpload::kMaxParts], pfirst[BaseUpload::kMaxParts];
  int pticket[BaseUpload::kMaxParts];
  float part_ms[BaseUpload::kMaxParts] = {};
  std::unique_ptr<PassTimer> ptm[BaseUpload::kMaxParts];
  if (up && !band && !prior && c_needed <= 16) {
    // ---- TOPC, base arriving part by part
    sel.mode = SCAN_TOPC;
    sel.C = pow2_at_least(c_needed);
    sel.nchunk = part_chunks(*up, 0, job.prec, sel.C, nqt, tile_n, ctx->num_sms * ctas_per_sm,
                             imin(1024, kMaxCandidates / sel.C) / up->nparts, pnch, ptpc, pfirst,
                             pticket);
    YG_CHECK(ws_get(ws, WS_TOPV, (size_t)sel.nchunk * nq * sel.C, &sel.topv));
    YG_CHECK(ws_get(ws, WS_TOPI, (size_t)sel.nchunk * nq * sel.C, &sel.topi));
    for (int i = 0; i < up->nparts; i++)
      if (pticket[i] >= 0) ptm[i].reset(new PassTimer(true, st, &part_ms[i], false));
    tm_scan.reset(new PassTimer(timed, st, &job.ms_scan));
    YG_CHECK(scan_parts(job, *up, *bops, dsmall, tcq, nq, sel, pnch, ptpc, pfirst, ptm, st));
    tm_scan->stop(st);
    job.scan_launches += up->nparts;
  } else if (!band && !prior && c_needed <= 16) {
    // ---- TOPC over the full base (register lists)
    sel.mode = SCAN_TOPC;
    sel.C = pow2_at_least(c_needed);
    const int nchunk = tune_chunks(TuneKey{0, job.prec, nqt, ntb, sel.C},
                                   choose_chunks(nqt, ntb, ctx->num_sms, ctas_per_sm, 4),
                                   imin(1024, kMaxCandidates / sel.C),
                                   ctx->num_sms * ctas_per_sm, &scan_ticket);
    sel.tiles_per_chunk = (int)ceil_div(ntb, nchunk);
    sel.nchunk = (int)ceil_div(ntb, sel.tiles_per_chunk);
    YG_CHECK(ws_get(ws, WS_TOPV, (size_t)sel.nchunk * nq * sel.C, &sel.topv));
    YG_CHECK(ws_get(ws, WS_TOPI, (size_t)sel.nchunk * nq * sel.C, &sel.topi));
    tm_scan.reset(new PassTimer(timed || scan_ticket >= 0, st, &job.ms_scan));
    YG_CHECK(scan(job, job.q, nq, job.b, job.ldb, nb, bn32, 1, &tcq, sel, st));
    tm_scan->stop(st);
    job.scan_launches++;
  } else {
    // ---- THRESH: per-query thresholds from a strided sample of the base.
    // The c-th smallest of a 1/stride sample lies below ~c*stride base values;
    // with stride = k/3 the chance that fewer than k fall below it is the
    // chance that a Poisson(3) exceeds c-1 (c = 12: ~1.7e-4 per query; such a
    // query fails its certificate and the band pass settles it).  The sample
    // pass keeps 16 values per row; the c-th of them is the threshold.
    sel.mode = SCAN_THRESH;
    sel.halves = 2;
    float *thr;
    YG_CHECK(ws_get(ws, WS_THR, nq, &thr));
    const int c = 12;
    int stride = k / 3;
    if (stride < 1) stride = 1;
    const int ns = nb / stride;
    if (up) {
      sel.nchunk = part_chunks(*up, 1, job.prec, 0, nqt, tile_n, ctx->num_sms * ctas_per_sm,
                               1024 / up->nparts, pnch, ptpc, pfirst, pticket);
      for (int i = 0; i < up->nparts; i++)
        if (pticket[i] >= 0) ptm[i].reset(new PassTimer(true, st, &part_ms[i], false));
    } else {
      sel.nchunk = band    ? 1
                   : prior ? choose_chunks(nqt, ntb, ctx->num_sms, ctas_per_sm, 4)
                           : tune_chunks(TuneKey{1, job.prec, nqt, ntb, 0},
                                         choose_chunks(nqt, ntb, ctx->num_sms, ctas_per_sm, 4),
                                         1024, ctx->num_sms * ctas_per_sm, &scan_ticket);
      sel.tiles_per_chunk = (int)ceil_div(ntb, sel.nchunk);
      sel.nchunk = (int)ceil_div(ntb, sel.tiles_per_chunk);
    }
    const int nreg = sel.nregion();
    // the threshold sample: every stride-th row of the base, or, while the base
    // is still arriving, every stride0-th row of part 0 (same sample size, so
    // the same expected rank if the rows are in no particular order; any
    // other order only costs candidates or band passes, never exactness)
    int sstride = stride, sns = ns;
    if (up) {
      const long n0 = up->row0[1] - up->row0[0];
      sstride = (int)std::max<long>(1, (long)((double)stride * n0 / nb));
      sns = (int)(n0 / sstride);
    }
    if (band) {
      // thresholds from the k-th exact distance an earlier pass found
      const BandLayout L = band_layout(nq, nb, k, tile_m, tile_n, sel.halves, ctx->num_sms);
      sel.nchunk = L.nchunk;
      sel.tiles_per_chunk = L.tiles_per_chunk;
      sel.cap = L.cap;
      YG_CHECK(band_thresholds(nq, job.metric, job.band_kth, qn64, eps, thr, st));
    } else if (prior) {
      // every row whose exact distance can be <= the known bound
      sel.cap = prior_cap(sel.nchunk);
      YG_CHECK(band_thresholds(nq, job.metric, job.prior_kth, qn64, eps, thr, st));
    } else if (nb <= kMaxCandidates || sns < 4 * c) {
      // every base row is a candidate; a region holds at most its share of the chunk
      sel.cap = pow2_at_least(imax(1, sel.tiles_per_chunk * tile_n / sel.halves));
      fill_f32<<<(unsigned)ceil_div(nq, 256), 256, 0, st>>>(thr, nq, INFINITY);
      YG_LAUNCH_CHECK();
    } else {
      ra.m_expect = c * stride;
      const double er = (double)c * stride / nreg;  // expected hits per region
      sel.cap = pow2_at_least((int)(2.0 * er + 6.0 * sqrt(er) + 16.0));
      ScanSel ss;
      ss.mode = SCAN_TOPV;  // only the c-th value is needed
      ss.C = 16;
      const int nts = (int)ceil_div(sns, tile_n);
      const int nch = tune_chunks(TuneKey{2, job.prec, nqt, nts, ss.C},
                                  choose_chunks(nqt, nts, ctx->num_sms, ctas_per_sm, 2), 64,
                                  ctx->num_sms * ctas_per_sm, &sample_ticket);
      ss.tiles_per_chunk = (int)ceil_div(nts, nch);
      ss.nchunk = (int)ceil_div(nts, ss.tiles_per_chunk);
      YG_CHECK(ws_get(ws, WS_STOPV, (size_t)ss.nchunk * nq * ss.C, &ss.topv));
      YG_CHECK(ws_get(ws, WS_STOPI, (size_t)ss.nchunk * nq * ss.C, &ss.topi));
      tm_sample.reset(new PassTimer(timed || sample_ticket >= 0, st, &job.ms_sample));
      if (bf16) {
        TcOperands tcs = tcq;
        YG_CHECK(tc_base_view(tcq, sstride, sns, &tcs));
        YG_CHECK(tc_scan(tcs, nq, sns, ss, st));
      } else {
        YG_CHECK(simt_scan(job.q, job.ldq, nq, job.b, job.ldb * stride, ns, d, bn32, stride,
                           job.metric, ss, st));
      }
      tm_sample->stop(st);
      YG_CHECK(thresh_from_sample(nq, ss.nchunk, ss.C, c, ss.topv, eps, thr, st));
    }
    sel.thr = thr;
    const int nr = sel.nregion();
    YG_CHECK(ws_get(ws, WS_CNT, (size_t)nr * nq, &sel.cnt));
    YG_CHECK(ws_get(ws, WS_TOPV, (size_t)nr * nq * sel.cap, &sel.candv));
    YG_CHECK(ws_get(ws, WS_TOPI, (size_t)nr * nq * sel.cap, &sel.candi));
    tm_scan.reset(new PassTimer(timed || scan_ticket >= 0, st, &job.ms_scan));
    if (up) {
      YG_CHECK(scan_parts(job, *up, *bops, dsmall, tcq, nq, sel, pnch, ptpc, pfirst, ptm, st));
      job.scan_launches += up->nparts;
    } else {
      YG_CHECK(scan(job, job.q, nq, job.b, job.ldb, nb, bn32, 1, &tcq, sel, st));
      job.scan_launches++;
    }
    tm_scan->stop(st);
  }
  if (up) {
    // the error bounds over the whole base (the thresholds used part 0's)
    YG_CHECK(compute_eps(nq, d, job.prec, job.metric, qn64, qres, qflag, &dsmall->bs, eps,
                         qexact, st));
  }
  ra.sel = sel;
  nv.reset(new NvtxRange("knn.rerank"));
  PassTimer tr(timed || scan_ticket >= 0, st, &job.ms_rerank);
  YG_CHECK(rerank(ra, st));
  tr.stop(st);

  // ---- deferred check: the status goes to the pinned buffer, the caller
  // synchronises later and calls knn_resolve
  if (job.defer && job.level == 0 && !timed && scan_ticket < 0 && sample_ticket < 0 && !up) {
    void *pin;
    YG_CHECK(ctx_pinned_status(ctx, &pin));
    YG_CUDA(cudaMemcpyAsync(pin, dsmall, sizeof(Small), cudaMemcpyDeviceToHost, st));
    job.pending = 1;
    job.fail_dev = fail_list;
    return OK;
  }

  // ---- later chances for the queries the certificate rejected
  Small hs;
  YG_CHECK(read_small(ctx, dsmall, st, &hs));
  tr.collect();
  if (tm_scan) {
    tm_scan->collect();
    // a chunk count also sets the candidate lists the re-rank reads
    tune_report(scan_ticket, tm_scan->last + tr.last);
  }
  if (tm_sample) {
    tm_sample->collect();
    tune_report(sample_ticket, tm_sample->last);
  }
  if (up) {
    for (int i = 0; i < up->nparts; i++) {
      if (!ptm[i]) continue;
      ptm[i]->collect();
      tune_report(pticket[i], ptm[i]->last);
    }
  }
  job.n_cand = (long long)hs.n_cand;
  job.exact_class = hs.bs.all_exact;
  if (hs.tc_err) {
    set_error(E_TIMEOUT, "tensor-core pass gave up waiting (bounded wait expired)");
    return E_TIMEOUT;
  }
  const int nf = hs.fail_cnt;
  if (trace_enabled())
    fprintf(stderr,
            "[yael_gpu] knn level=%d prec=%d pass=%s nq=%d nb=%d d=%d k=%d chunks=%d "
            "scan=%.3fms sample=%.3fms rerank=%.3fms rejected=%d\n",
            job.level, job.prec,
            band ? "band" : prior ? "prior" : (sel.mode == SCAN_TOPC ? "topc" : "thresh"), nq,
            nb, d, k, sel.nchunk, job.ms_scan, job.ms_sample, job.ms_rerank, nf);
  if (nf == 0) return OK;
  // A regular pass's rejections go to a band pass at the same precision: its
  // thresholds come from the k-th exact distance the re-rank found, so it
  // collects every row that can still be in the top k.  A BF16 / FP16 band pass's
  // rejections (bands too wide for its candidate buffers) go to a band pass on
  // the 3xBF16 split operands, whose error bound and so whose band is ~2^-8 of
  // the BF16 one; everything else to the exhaustive FP64 path.
  const bool to_band = !band && job.w == nullptr;
  const bool to_split =
      band && (job.prec == PREC_BF16 || job.prec == PREC_FP16) && job.w == nullptr;
  nv.reset(new NvtxRange("knn.later_passes"));
  PassTimer t2(timed, st, &job.ms_second);
  if ((to_band || to_split) && job.level < 4) {
    const int base = WS_SC0 + job.level * WS_SC_PER_LEVEL;
    int *map, *cidx;
    float *cq, *cdis, *ckth = nullptr;
    YG_CHECK(ws_get(ws, base + 0, nf, &map));
    YG_CHECK(ws_get(ws, base + 1, (size_t)nf * d, &cq));
    YG_CHECK(ws_get(ws, base + 2, (size_t)nf * k, &cidx));
    YG_CHECK(ws_get(ws, base + 3, (size_t)nf * k, &cdis));
    YG_CUDA(cudaMemcpyAsync(map, fail_list, sizeof(int) * nf, cudaMemcpyDeviceToDevice, st));
    gather_rows_kernel<<<(unsigned)ceil_div((long)nf * d, 256), 256, 0, st>>>(job.q, job.ldq, map,
                                                                            nf, d, cq);
    YG_LAUNCH_CHECK();
    YG_CHECK(ws_get(ws, base + 4, nf, &ckth));
    gather_kth_kernel<<<(unsigned)ceil_div(nf, 256), 256, 0, st>>>(
        job.band_kth ? job.band_kth : job.prior_kth, kth, map, nf, ckth);
    YG_LAUNCH_CHECK();
    if (to_split && !bops->has_split) {
      float *bn32s;
      YG_CHECK(ws_get(ws, WS_BN32, nb, &bn32s));
      YG_CHECK(tc_prepare_base(job.b, job.ldb, nb, d, job.metric, ws, WS_BPACK3, WS_BNORMP3,
                               WS_BRES3, &bops->split, bn32s, &dsmall->bs3, 1, st));
      bops->split.err = bops->plain.err;
      bops->has_split = true;
    }
    KnnJob sub = job;
    sub.prec = to_split ? PREC_BF16X3 : job.prec;
    sub.band_kth = ckth;
    sub.prior_kth = nullptr;
    sub.level = job.level + 1;
    sub.nq = nf;
    sub.q = cq;
    sub.ldq = d;
    sub.out_idx = cidx;
    sub.out_dis = cdis;
    sub.timing = 0;
    YG_CHECK(knn_batches(sub, ctx, st, dsmall, bops, bstats_exact));
    scatter_rows_kernel<<<(unsigned)ceil_div((long)nf * k, 256), 256, 0, st>>>(cidx, cdis, map, nf,
                                                                             k, job.out_idx,
                                                                             job.out_dis);
    YG_LAUNCH_CHECK();
    if (to_band) job.n_band += nf;
    else job.n_second += nf;
    job.n_band += sub.n_band;
    job.n_second += sub.n_second;
    job.n_fallback += sub.n_fallback;
  } else {
    size_t per = exhaustive_bytes_per_query(nb);
    size_t want = per * (size_t)nf;
    const size_t cap_bytes = (size_t)1 << 30;
    if (want > cap_bytes) want = cap_bytes > per ? cap_bytes : per;
    void *scratch;
    YG_CHECK(ws.get(WS_EXH, want, &scratch));
    YG_CHECK(exhaustive(nf, fail_list, nb, d, k, job.metric, job.q, job.ldq, job.b, job.ldb,
                        nullptr, job.out_idx, job.out_dis, scratch, want, st));
    job.n_fallback += nf;
  }
  t2.stop(st);
  YG_CUDA(cudaStreamSynchronize(st));
  t2.collect();
  return OK;
}

// the queries of job in batches whose candidate buffers stay <= 2 GiB
int knn_batches(KnnJob &job, Ctx *ctx, cudaStream_t st, Small *dsmall, BaseOps *bops,
                int bexact) {
  const int nq = job.nq, nb = job.nb, k = job.k;
  const bool bf16 = job.prec != PREC_FP32;
  const int tile_n = bf16 ? TC_TILE_N : SIMT_TILE_N, tile_m = bf16 ? TC_TILE_M : 128;
  const size_t budget = (size_t)2 << 30;
  int qbatch;
  if (job.band_kth) {
    qbatch = nq;
    while (qbatch > 256 &&
           band_layout(qbatch, nb, k, tile_m, tile_n, 2, ctx->num_sms)
                       .bytes_per_query() *
                   (size_t)qbatch > budget)
      qbatch = (qbatch + 1) / 2;
  } else if (job.prior_kth) {
    const int nqt = (int)ceil_div(nq, tile_m), ntb = (int)ceil_div(nb, tile_n);
    const int nch = choose_chunks(nqt, ntb, ctx->num_sms, 1, 4);
    const size_t per_query = (size_t)nch * 2 * (prior_cap(nch) * 8 + 4) + 64;
    qbatch = (int)std::min<size_t>((size_t)nq, std::max<size_t>(256, budget / per_query));
  } else {
    const int cn = list_length(k, bexact, nb);
    const int nqt = (int)ceil_div(nq, tile_m), ntb = (int)ceil_div(nb, tile_n);
    const int C = pow2_at_least(cn);
    size_t per_query;
    if (cn <= 16) {
      // the autotuner may try up to 3x the heuristic's chunk count
      const int nch = imin(imin(1024, kMaxCandidates / C),
                           3 * choose_chunks(nqt, ntb, ctx->num_sms, 1, 4) + 2);
      per_query = (size_t)nch * C * 8 + 64;
    } else {
      per_query = (size_t)2 * kMaxCandidates * 8 + 64;
    }
    qbatch = (int)std::min<size_t>((size_t)nq, std::max<size_t>(256, budget / per_query));
  }
  long long ncand = 0;
  for (int q0 = 0; q0 < nq; q0 += qbatch) {
    KnnJob sub = job;
    sub.nq = imin(qbatch, nq - q0);
    sub.q = job.q + (long)q0 * job.ldq;
    sub.out_idx = job.out_idx + (long)q0 * k;
    sub.out_dis = job.out_dis + (long)q0 * k;
    if (job.band_kth) sub.band_kth = job.band_kth + q0;
    if (job.prior_kth) sub.prior_kth = job.prior_kth + q0;
    sub.n_fallback = sub.n_band = sub.n_second = 0;
    sub.ms_scan = sub.ms_sample = sub.ms_rerank = sub.ms_second = 0;
    sub.scan_launches = 0;
    sub.defer = job.defer && qbatch >= nq;  // a single batch only
    YG_CHECK(knn_batch(sub, ctx, st, dsmall, bops, bexact));
    if (sub.pending) {
      job.pending = 1;
      job.fail_dev = sub.fail_dev;
    }
    job.n_fallback += sub.n_fallback;
    job.n_band += sub.n_band;
    job.n_second += sub.n_second;
    ncand = sub.n_cand;  // the device counter is cumulative
    job.ms_scan += sub.ms_scan;
    job.ms_sample += sub.ms_sample;
    job.ms_rerank += sub.ms_rerank;
    job.ms_second += sub.ms_second;
    job.scan_launches += sub.scan_launches;
    job.exact_class = sub.exact_class;
  }
  job.n_cand = ncand;
  return OK;
}

}  // namespace

int knn_device(KnnJob &job, Ctx *ctx, cudaStream_t st) {
  const int nq = job.nq, nb = job.nb, d = job.d, k = job.k;
  job.n_fallback = 0;
  job.n_band = 0;
  job.n_second = 0;
  job.n_cand = 0;
  job.exact_class = 0;
  job.ms_scan = job.ms_sample = job.ms_rerank = job.ms_second = 0;
  job.band_kth = nullptr;
  job.level = 0;
  job.scan_launches = 0;
  if (nq < 0 || nb < 1 || d < 1 || k < 1) {
    set_error(E_ARG, "knn: invalid sizes nq=%d nb=%d d=%d k=%d", nq, nb, d, k);
    return E_ARG;
  }
  if (k > nb) {
    set_error(E_ARG, "knn: k=%d > nb=%d (yael asserts k <= nb)", k, nb);
    return E_ARG;
  }
  if (k > kMaxK) {
    set_error(E_UNSUPPORTED, "knn: k=%d above the supported maximum %d", k, kMaxK);
    return E_UNSUPPORTED;
  }
  const bool alt = job.metric > METRIC_ALT0 && job.metric <= METRIC_ALT0 + 6 &&
                   job.metric != METRIC_ALT0 + 2;
  if (job.metric != METRIC_L2 && job.metric != METRIC_DOT && !alt) {
    set_error(E_UNSUPPORTED, "knn: distance_type %d not supported on the GPU", job.metric);
    return E_UNSUPPORTED;
  }
  if (nq == 0) return OK;
  Workspace &ws = ctx->ws;

  Small *dsmall;
  YG_CHECK(ws_get(ws, WS_SMALL, 1, &dsmall));
  small_init_kernel<<<1, 1, 0, st>>>(dsmall);
  YG_LAUNCH_CHECK();

  if (job.w || alt) {
    // weighted distances reorder per base row, and the per-coordinate types
    // (L1, chi2, ...) have no GEMM form: the exhaustive path, which computes
    // every distance in the reference's arithmetic and keeps the k smallest
    size_t per = exhaustive_bytes_per_query(nb);
    size_t want = per * (size_t)nq;
    const size_t cap_bytes = (size_t)1 << 30;
    if (want > cap_bytes) want = cap_bytes > per ? cap_bytes : per;
    void *scratch;
    YG_CHECK(ws.get(WS_EXH, want, &scratch));
    YG_CHECK(exhaustive(nq, nullptr, nb, d, k, job.metric, job.q, job.ldq, job.b, job.ldb,
                        job.w, job.out_idx, job.out_dis, scratch, want, st));
    job.n_fallback = nq;
    return OK;
  }

  // base preparation (once for all query batches)
  NvtxRange nv_base("knn.pack_base");
  float *bn32, *bres = nullptr;
  YG_CHECK(ws_get(ws, WS_BN32, nb, &bn32));
  BaseOps bops;
  if (job.prec == PREC_BF16 && job.upload) {
    // the base arrives part by part: buffers for all of it, part 0 packed now
    BaseUpload &up = *job.upload;
    YG_CHECK(tc_alloc_base(nb, d, job.metric, ws, WS_BPACK, WS_BNORMP, WS_BRES, &bops.plain,
                           &bops.res));
    bops.bn32 = bn32;
    YG_CUDA(cudaStreamWaitEvent(st, up.ready[0], 0));
    YG_CHECK(tc_prepare_base_range(job.b, job.ldb, up.row0[0], (int)(up.row0[1] - up.row0[0]),
                                   d, job.metric, bops.plain, bn32, bops.res, &dsmall->bs, st));
    up.packed[0] = true;
    bops.has_plain = true;
  } else if (job.prec == PREC_BF16 || job.prec == PREC_FP16) {
    YG_CHECK(tc_prepare_base(job.b, job.ldb, nb, d, job.metric, ws, WS_BPACK, WS_BNORMP,
                             WS_BRES, &bops.plain, bn32, &dsmall->bs, 0, st,
                             job.prec == PREC_FP16));
    bops.has_plain = true;
  } else if (job.prec == PREC_BF16X3) {
    // the plain statistics (max norm) are needed too: dot-product bounds read them
    YG_CHECK(tc_prepare_base(job.b, job.ldb, nb, d, job.metric, ws, WS_BPACK3, WS_BNORMP3,
                             WS_BRES3, &bops.split, bn32, &dsmall->bs3, 1, st));
    YG_CHECK(prep_rows(job.b, job.ldb, nb, d, 1.f, nullptr, nullptr, nullptr, nullptr, nullptr,
                       0, nullptr, 0, &dsmall->bs, st));
    bops.has_split = true;
  } else {
    YG_CHECK(prep_rows(job.b, job.ldb, nb, d, 1.f, nullptr, bn32, nullptr, bres, nullptr, 0,
                       nullptr, 0, &dsmall->bs, st));
  }
  // the list length of k > 1 depends on whether the base is exact class (k = 1
  // does not: no host round trip then); every later read of the small state
  // also checks the tensor-core passes' error flag
  int bexact = 0;
  if (k > 1) {
    Small hs;
    YG_CHECK(read_small(ctx, dsmall, st, &hs));
    bexact = hs.bs.all_exact;
  }
  bops.plain.err = bops.split.err = &dsmall->tc_err;
  YG_CHECK(knn_batches(job, ctx, st, dsmall, &bops, bexact));
  return OK;
}

int knn_resolve(KnnJob &job, Ctx *ctx, cudaStream_t st) {
  if (!job.pending) return OK;
  job.pending = 0;
  void *pin;
  YG_CHECK(ctx_pinned_status(ctx, &pin));
  Small hs;
  memcpy(&hs, pin, sizeof(Small));
  job.n_cand = (long long)hs.n_cand;
  job.exact_class = hs.bs.all_exact;
  if (hs.tc_err) {
    set_error(E_TIMEOUT, "tensor-core pass gave up waiting (bounded wait expired)");
    return E_TIMEOUT;
  }
  const int nf = hs.fail_cnt, d = job.d, k = job.k;
  if (nf == 0) return OK;
  Workspace &ws = ctx->ws;
  int *map, *cidx;
  float *cq, *cdis;
  YG_CHECK(ws_get(ws, WS_DEF0 + 0, nf, &map));
  YG_CHECK(ws_get(ws, WS_DEF0 + 1, (size_t)nf * d, &cq));
  YG_CHECK(ws_get(ws, WS_DEF0 + 2, (size_t)nf * k, &cidx));
  YG_CHECK(ws_get(ws, WS_DEF0 + 3, (size_t)nf * k, &cdis));
  // the list is copied first: the pipeline below reuses its workspace slot
  YG_CUDA(cudaMemcpyAsync(map, job.fail_dev, sizeof(int) * nf, cudaMemcpyDeviceToDevice, st));
  gather_rows_kernel<<<(unsigned)ceil_div((long)nf * d, 256), 256, 0, st>>>(job.q, job.ldq, map, nf,
                                                                          d, cq);
  YG_LAUNCH_CHECK();
  KnnJob sub;
  sub.nq = nf; sub.nb = job.nb; sub.d = d; sub.k = k; sub.metric = job.metric;
  sub.prec = job.prec;
  sub.q = cq; sub.ldq = d; sub.b = job.b; sub.ldb = job.ldb; sub.w = job.w;
  sub.out_idx = cidx; sub.out_dis = cdis;
  YG_CHECK(knn_device(sub, ctx, st));
  scatter_rows_kernel<<<(unsigned)ceil_div((long)nf * k, 256), 256, 0, st>>>(cidx, cdis, map, nf, k,
                                                                           job.out_idx, job.out_dis);
  YG_LAUNCH_CHECK();
  YG_CUDA(cudaStreamSynchronize(st));
  job.n_band += nf + sub.n_band;
  job.n_second += sub.n_second;
  job.n_fallback += sub.n_fallback;
  return OK;
}

// host-memory entry: copies in, runs, copies out
int knn_host(int metric, int nq, int nb, int d, int k, const float *b,
                    const float *q, const float *w, int *assign, float *dis, int prec,
                    yael_gpu_knn_opts *opts) {
  Ctx *ctx;
  YG_CHECK(ctx_get(&ctx));
  cudaStream_t st = ctx->stream;
  KnnJob job;
  job.nq = nq; job.nb = nb; job.d = d; job.k = k; job.metric = metric; job.prec = prec;
  job.ldq = d; job.ldb = d;
  job.timing = opts ? opts->timing : 0;
  if (opts && opts->device_ptrs) {
    if (opts->stream) st = (cudaStream_t)opts->stream;
    job.q = q; job.b = b; job.w = w; job.out_idx = assign; job.out_dis = dis;
    YG_CHECK(knn_device(job, ctx, st));
    YG_CUDA(cudaStreamSynchronize(st));
  } else {
    if (nq == 0) return OK;
    Workspace &ws = ctx->ws;
    float *db, *dq, *dw = nullptr, *ddis;
    int *didx;
    YG_CHECK(ws_get(ws, WS_H_B, (size_t)nb * d, &db));
    YG_CHECK(ws_get(ws, WS_H_Q, (size_t)nq * d, &dq));
    YG_CHECK(ws_get(ws, WS_H_IDX, (size_t)nq * k, &didx));
    YG_CHECK(ws_get(ws, WS_H_DIS, (size_t)nq * k, &ddis));
    // A large base goes up in parts on a second stream while the passes over
    // the parts already there run (host -> device copies are ~25x slower than
    // the packing of what they carry).  The guard drains the copies and frees
    // the events on every exit path.
    const bool stream_up =
        w == nullptr && prec == PREC_BF16 && metric < METRIC_ALT0 && nb >= (1 << 18);
    BaseUpload up;
    struct UploadGuard {
      BaseUpload *u;
      cudaStream_t cs;
      ~UploadGuard() {
        if (cs) cudaStreamSynchronize(cs);
        for (int i = 0; i < u->nparts; i++)
          if (u->ready[i]) cudaEventDestroy(u->ready[i]);
      }
    } guard{&up, nullptr};
    cudaEvent_t tl[3] = {nullptr, nullptr, nullptr};  // trace timeline (streamed upload)
    if (stream_up) {
      if (!ctx->copy_stream)
        YG_CUDA(cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
      cudaStream_t cs = ctx->copy_stream;
      guard.cs = cs;
      if (trace_enabled()) {
        YG_CUDA(cudaEventCreate(&tl[0]));
        YG_CUDA(cudaEventRecord(tl[0], st));
      }
      // the queries first: a copy issued after the base parts would wait for them
      YG_CUDA(cudaMemcpyAsync(dq, q, sizeof(float) * nq * (size_t)d, cudaMemcpyHostToDevice, st));
      cudaEvent_t qdone;
      YG_CUDA(cudaEventCreateWithFlags(&qdone, cudaEventDisableTiming));
      YG_CUDA(cudaEventRecord(qdone, st));
      YG_CUDA(cudaStreamWaitEvent(cs, qdone, 0));
      YG_CUDA(cudaEventDestroy(qdone));
      // parts of 1/8, 1/4, 1/4, 1/4, 1/8 of the base (whole 256-row tiles): a
      // small first part starts the passes early, a small last one leaves
      // little to do after the final copy
      const int parts = 5;
      const double frac[parts + 1] = {0.0, 0.125, 0.375, 0.625, 0.875, 1.0};
      up.nparts = parts;
      for (int i = 0; i <= parts; i++)
        up.row0[i] = std::min<long>((long)nb, (long)(frac[i] * nb / 256) * 256);
      up.row0[parts] = nb;
      for (int i = 0; i < parts; i++) {
        YG_CUDA(cudaEventCreateWithFlags(&up.ready[i],
                                         tl[0] ? cudaEventDefault : cudaEventDisableTiming));
        const long r0 = up.row0[i], n = up.row0[i + 1] - r0;
        YG_CUDA(cudaMemcpyAsync(db + r0 * d, b + r0 * d, sizeof(float) * n * (size_t)d,
                                cudaMemcpyHostToDevice, cs));
        YG_CUDA(cudaEventRecord(up.ready[i], cs));
      }
      job.upload = &up;
    } else {
      YG_CUDA(cudaMemcpyAsync(db, b, sizeof(float) * nb * (size_t)d, cudaMemcpyHostToDevice, st));
      YG_CUDA(cudaMemcpyAsync(dq, q, sizeof(float) * nq * (size_t)d, cudaMemcpyHostToDevice, st));
    }
    if (w) {
      YG_CHECK(ws_get(ws, WS_H_W, (size_t)nb, &dw));
      YG_CUDA(cudaMemcpyAsync(dw, w, sizeof(float) * nb, cudaMemcpyHostToDevice, st));
    }
    job.q = dq; job.b = db; job.w = dw; job.out_idx = didx; job.out_dis = ddis;
    YG_CHECK(knn_device(job, ctx, st));
    if (tl[0]) {
      YG_CUDA(cudaEventCreate(&tl[1]));
      YG_CUDA(cudaEventRecord(tl[1], st));
    }
    YG_CUDA(cudaMemcpyAsync(assign, didx, sizeof(int) * nq * (size_t)k, cudaMemcpyDeviceToHost, st));
    YG_CUDA(cudaMemcpyAsync(dis, ddis, sizeof(float) * nq * (size_t)k, cudaMemcpyDeviceToHost, st));
    if (tl[0]) {
      YG_CUDA(cudaEventCreate(&tl[2]));
      YG_CUDA(cudaEventRecord(tl[2], st));
    }
    YG_CUDA(cudaStreamSynchronize(st));
    if (tl[0]) {
      // trace: the host call's timeline (base parts landed, passes done, results back)
      float t;
      fprintf(stderr, "[yael_gpu] knn host call timeline (ms):");
      for (int i = 0; i < up.nparts; i++) {
        cudaEventElapsedTime(&t, tl[0], up.ready[i]);
        fprintf(stderr, " part%d %.3f", i, t);
      }
      cudaEventElapsedTime(&t, tl[0], tl[1]);
      fprintf(stderr, " | passes %.3f", t);
      cudaEventElapsedTime(&t, tl[0], tl[2]);
      fprintf(stderr, " | results %.3f\n", t);
      for (auto &e : tl) {
        cudaEventDestroy(e);
        e = nullptr;
      }
    }
  }
  if (opts) {
    opts->n_fallback = job.n_fallback;
    opts->n_candidates = (int)(job.n_cand > 0x7fffffff ? 0x7fffffff : job.n_cand);
    opts->exact_class = job.exact_class;
    opts->ms_scan = job.ms_scan;
    opts->ms_sample = job.ms_sample;
    opts->ms_rerank = job.ms_rerank;
    opts->scan_launches = job.scan_launches;
    opts->n_second = job.n_second;
    opts->n_band = job.n_band;
    opts->ms_second = job.ms_second;
  }
  return OK;
}

static int metric_of(int distance_type) {
  if (distance_type == 2 || distance_type == 12) return METRIC_L2;
  if (distance_type == 16) return METRIC_DOT;
  // L1, the chi2 forms, histogram intersection, float dot (yael/nn.c:311-350)
  if (distance_type == 1 || (distance_type >= 3 && distance_type <= 6))
    return METRIC_ALT0 + distance_type;
  return -1;
}

}  // namespace yg

using namespace yg;

extern "C" {

int yael_gpu_knn_ex(int nq, int nb, int d, int k, const float *b, const float *q,
                    int *assign, float *dis, yael_gpu_knn_opts *opts) {
  int prec = default_precision();
  int metric = METRIC_L2;
  if (opts) {
    if (explicit_precision(opts->precision))
      prec = opts->precision;
    if (opts->metric) metric = metric_of(opts->metric);
  }
  if (metric < 0) {
    set_error(E_UNSUPPORTED, "distance_type %d not supported", opts ? opts->metric : 0);
    return E_UNSUPPORTED;
  }
  WaitLimitScope wls(opts ? opts->wait_limit_us : 0);
  return knn_host(metric, nq, nb, d, k, b, q, nullptr, assign, dis, prec, opts);
}

void knn_full(int distance_type, int nq, int nb, int d, int k, const float *b,
              const float *q, const float *b_weights, int *assign, float *dis) {
  const int metric = metric_of(distance_type);
  if (metric < 0) {
    set_error(E_UNSUPPORTED,
              "distance_type %d has no GPU implementation (supported: 1-6, 12, 16)",
              distance_type);
    fatal_last("knn_full");
  }
  if (knn_host(metric, nq, nb, d, k, b, q, b_weights, assign, dis, default_precision(),
               nullptr) != OK)
    fatal_last("knn_full");
}

void knn_full_thread(int distance_type, int nq, int nb, int d, int k, const float *b,
                     const float *q, const float *b_weights, int *assign, float *dis,
                     int n_thread) {
  (void)n_thread;
  knn_full(distance_type, nq, nb, d, k, b, q, b_weights, assign, dis);
}

double nn(int n, int nb, int d, const float *b, const float *v, int *assign) {
  float *dis = (float *)malloc(sizeof(float) * (size_t)(n > 0 ? n : 1));
  knn_full(2, n, nb, d, 1, b, v, nullptr, assign, dis);
  double s = 0;  // fvec_sum order (yael/vector.c:2066-2073)
  for (long i = 0; i < n; i++) s += dis[i];
  free(dis);
  return s;
}

double nn_thread(int n, int nb, int d, const float *b, const float *v, int *assign,
                 int n_thread) {
  (void)n_thread;
  return nn(n, nb, d, b, v, assign);
}

float *knn(int n, int nb, int d, int k, const float *b, const float *v, int *assign) {
  float *dis = (float *)malloc(sizeof(float) * (size_t)n * k + 4);
  knn_full(2, n, nb, d, k, b, v, nullptr, assign, dis);
  return dis;
}

float *knn_thread(int nq, int nb, int d, int k, const float *b, const float *v,
                  int *assign, int n_thread) {
  (void)n_thread;
  return knn(nq, nb, d, k, b, v, assign);
}

}  // extern "C"
