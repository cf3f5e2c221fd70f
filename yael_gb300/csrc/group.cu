// Grouped exact k-NN over many independent (queries, base) pairs of uneven
// sizes: one persistent launch per pass over all the pairs instead of a
// pipeline per pair (yael_gpu_knn_batch with device arrays, the BF16 pass and
// k >= 9, i.e. the threshold form of the selection).
//
// Layout (per wave of pairs, bounded in memory):
//   * the pairs' queries are packed one after the other (rows qoff_p ...);
//   * their bases likewise, each padded to a multiple of P = 256 * stride rows
//     (stride: the threshold sample's), so that the pair's tiles start at a
//     tile boundary both in the base and in its every-stride-th-row view;
//   * unit tables list (query tile of a pair, range of that pair's base tiles).
// Passes (as in the single-pair pipeline, knn.cu): operand packing and error
// bounds per pair; the threshold sample pass (TOPV 16 over every stride-th base
// row, one chunk per pair); thresholds; the main THRESH pass (chunks of up to
// kGroupTiles tiles, candidate regions laid out per pair); the re-rank of
// every query against its own pair.  Queries whose certificate fails are run
// again through the single-pair pipeline (band passes, FP64 fallback), which
// makes the results exactly those of a loop of knn_full calls.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "knn.cuh"
#include "select.cuh"
#include "tc_scan.cuh"

namespace yg {
namespace {

constexpr int kGroupTiles = 128;       // base tiles per main-pass unit
constexpr int kSampleC = 12;           // threshold rank in the sample (knn.cu)

// workspace slots of the grouped pipeline (disjoint from the per-call ones)
enum GroupSlot : int {
  GS_BPACK = 140, GS_BNORM, GS_QPACK, GS_QNORM, GS_QN64, GS_QFLAG, GS_QRES, GS_EPS, GS_QEXACT,
  GS_STATS, GS_PAIRS, GS_QPAIR, GS_SUNITS, GS_MUNITS, GS_STOPV, GS_THR, GS_CNT, GS_CANDV,
  GS_CANDI, GS_FAIL, GS_KTH, GS_STATUS, GS_FQ, GS_FIDX, GS_FDIS, GS_INF, GS_FROWS, GS_STOPI,
};

struct GroupStatus {
  int fail_cnt;
  int tc_err;
  unsigned long long n_cand;
};

template <typename T>
int gs_get(Workspace &ws, int slot, size_t count, T **p) {
  void *v = nullptr;
  YG_CHECK(ws.get(slot, (count ? count : 1) * sizeof(T), &v));
  *p = reinterpret_cast<T *>(v);
  return OK;
}

__global__ void stats_init_kernel(SetStats *s, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    s[i].max_norm_bits = 0u;
    s[i].max_resid_bits = 0u;
    s[i].all_exact = 1;
    s[i].n_nan = 0;
    s[i].max_lo_bits = 0u;
  }
}

__global__ void qpair_kernel(int *qpair, int p, int q0, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) qpair[q0 + i] = p;
}

// thresholds of the queries of pairs without a sample (every row a candidate)
__global__ void thr_inf_kernel(const int *qpair, const GroupPair *gp, const unsigned char *inf,
                               int nq, float *thr) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < nq && inf[qpair[q]]) thr[q] = INFINITY;
}

__global__ void gather_rows_k(const float *src, int d, const int *rows, int n, float *dst) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long)n * d) return;
  const long r = i / d;
  dst[i] = src[(long)rows[r] * d + (i - r * d)];
}

__global__ void scatter_rows_k(const int *idx, const float *dis, const int *rows, int n, int k,
                               int *oidx, float *odis) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long)n * k) return;
  const long r = i / k;
  const long o = (long)rows[r] * k + (i - r * k);
  oidx[o] = idx[i];
  odis[o] = dis[i];
}

long round_up(long x, long m) { return (x + m - 1) / m * m; }

int pow2_ge(int x) {
  int p = 1;
  while (p < x) p <<= 1;
  return p;
}

// candidate layout of one pair's main pass: regions per query and slots per
// region (every row a candidate when the pair has no threshold sample)
void pair_layout(int nb, int stride, bool inf, int *nreg, int *cap, int *tpc) {
  const int ntb = (int)ceil_div(nb, TC_TILE_N);
  const int nch = (int)ceil_div(ntb, kGroupTiles);
  *tpc = (int)ceil_div(ntb, nch);
  *nreg = 2 * nch;
  if (inf) {
    *cap = pow2_ge(std::max(1, *tpc * TC_TILE_N / 2));
  } else {
    const double er = (double)kSampleC * stride / *nreg;
    *cap = pow2_ge((int)(2.0 * er + 6.0 * sqrt(er) + 16.0));
  }
}

bool pair_inf(int nb, int stride) { return nb <= kMaxCandidates || nb / stride < 4 * kSampleC; }

struct Wave {
  std::vector<int> pairs;  // indices into the caller's pair array
};

// One wave: every pair of w through the grouped passes; results in the pairs'
// output arrays, counters added to *gc.
int run_wave(const yael_gpu_knn_pair *pairs, const Wave &w, int d, int k, int metric, Ctx *ctx,
             cudaStream_t st, GroupCounters *gc) {
  Workspace &ws = ctx->ws;
  const int np = (int)w.pairs.size();
  const int Kp = ((d + 63) / 64) * 64;
  const bool L2 = metric == METRIC_L2;
  const int stride = std::max(1, k / 3);
  const long P = (long)TC_TILE_N * stride;
  // ---- layout
  std::vector<GroupPair> hp(np);
  std::vector<unsigned char> hinf(np);
  long nqt_all = 0, brows = 0;
  int nq_all = 0;
  for (int i = 0; i < np; i++) {
    const yael_gpu_knn_pair &x = pairs[w.pairs[i]];
    GroupPair &g = hp[i];
    g.qoff = nq_all;
    g.nq = x.nq;
    g.boff = (int)brows;
    g.nb = x.nb;
    g.q = x.q;
    g.b = x.b;
    g.out_idx = x.assign;
    g.out_dis = x.dis;
    nq_all += x.nq;
    brows += round_up(x.nb, P);
    nqt_all += ceil_div(x.nq, TC_TILE_M);
    hinf[i] = pair_inf(x.nb, stride) ? 1 : 0;
  }
  if (nq_all == 0) return OK;
  if (brows > 0x7fffffffL) {
    set_error(E_UNSUPPORTED, "knn_batch: %ld padded base rows in one group", brows);
    return E_UNSUPPORTED;
  }
  // ---- buffers
  __nv_bfloat16 *bpack, *bnorm = nullptr, *qpack, *qnorm = nullptr;
  double *qn64;
  unsigned char *qflag, *qexact, *dinf;
  float *qres, *eps, *thr, *kth;
  SetStats *stats;
  GroupPair *dpairs;
  int *qpair, *fail;
  GroupStatus *status;
  YG_CHECK(gs_get(ws, GS_BPACK, (size_t)brows * Kp, &bpack));
  if (L2) YG_CHECK(gs_get(ws, GS_BNORM, (size_t)brows * 16, &bnorm));
  YG_CHECK(gs_get(ws, GS_QPACK, (size_t)nq_all * Kp, &qpack));
  if (L2) YG_CHECK(gs_get(ws, GS_QNORM, (size_t)nq_all * 16, &qnorm));
  YG_CHECK(gs_get(ws, GS_QN64, nq_all, &qn64));
  YG_CHECK(gs_get(ws, GS_QFLAG, nq_all, &qflag));
  YG_CHECK(gs_get(ws, GS_QRES, nq_all, &qres));
  YG_CHECK(gs_get(ws, GS_EPS, nq_all, &eps));
  YG_CHECK(gs_get(ws, GS_QEXACT, nq_all, &qexact));
  YG_CHECK(gs_get(ws, GS_THR, nq_all, &thr));
  YG_CHECK(gs_get(ws, GS_KTH, nq_all, &kth));
  YG_CHECK(gs_get(ws, GS_FAIL, nq_all, &fail));
  YG_CHECK(gs_get(ws, GS_QPAIR, nq_all, &qpair));
  YG_CHECK(gs_get(ws, GS_STATS, np, &stats));
  YG_CHECK(gs_get(ws, GS_INF, np, &dinf));
  YG_CHECK(gs_get(ws, GS_STATUS, 1, &status));
  for (int i = 0; i < np; i++) hp[i].bs = stats + i;

  // trace: events between the passes (YAEL_GPU_TRACE)
  const bool tr = trace_enabled();
  cudaEvent_t ev[5] = {};
  if (tr)
    for (auto &e : ev) cudaEventCreate(&e);
  if (tr) cudaEventRecord(ev[0], st);

  // ---- packing: every pair's base and queries into the concatenated buffers
  stats_init_kernel<<<(unsigned)ceil_div(np, 128), 128, 0, st>>>(stats, np);
  YG_LAUNCH_CHECK();
  YG_CUDA(cudaMemsetAsync(status, 0, sizeof(GroupStatus), st));
  const float qscale = L2 ? -2.f : 1.f;
  for (int i = 0; i < np; i++) {
    const GroupPair &g = hp[i];
    YG_CHECK(prep_rows(g.b, d, g.nb, d, 1.f, nullptr, nullptr, nullptr, nullptr,
                       bpack + (size_t)g.boff * Kp, Kp, L2 ? bnorm + (size_t)g.boff * 16 : nullptr,
                       L2 ? 1 : 0, stats + i, st));
    if (g.nq == 0) continue;
    const float *q = pairs[w.pairs[i]].q;
    YG_CHECK(prep_rows(q, d, g.nq, d, qscale, qn64 + g.qoff, nullptr, qflag + g.qoff,
                       qres + g.qoff, qpack + (size_t)g.qoff * Kp, Kp,
                       L2 ? qnorm + (size_t)g.qoff * 16 : nullptr, L2 ? 2 : 0, nullptr, st));
    qpair_kernel<<<(unsigned)ceil_div(g.nq, 256), 256, 0, st>>>(qpair, i, g.qoff, g.nq);
    YG_LAUNCH_CHECK();
  }

  // ---- main-pass layout: chunks, regions and capacities per pair
  std::vector<GroupUnit> mu, su;
  long cnt_tot = 0, cand_tot = 0;
  int max_cand = 4 * kSampleC * stride + 64;
  for (int i = 0; i < np; i++) {
    GroupPair &g = hp[i];
    const int ntb = (int)ceil_div(g.nb, TC_TILE_N);
    int tpc;
    pair_layout(g.nb, stride, hinf[i], &g.nreg, &g.cap, &tpc);
    const int nch = g.nreg / 2;
    if (hinf[i]) max_cand = std::max(max_cand, g.nb);
    g.cnt_off = cnt_tot;
    g.cand_off = cand_tot;
    cnt_tot += (long)g.nreg * g.nq;
    cand_tot += (long)g.nreg * g.nq * g.cap;
    const int tb0 = g.boff / TC_TILE_N;
    const int nqt = (int)ceil_div(g.nq, TC_TILE_M);
    // query tiles innermost: CTAs that run together read the same base chunk
    // (from L2 rather than DRAM, as in the single-pair grid)
    for (int c = 0; c < nch; c++)
      for (int qt = 0; qt < nqt; qt++) {
        GroupUnit u;
        u.q0 = g.qoff + qt * TC_TILE_M;
        u.qend = g.qoff + g.nq;
        u.t_begin = tb0 + c * tpc;
        u.t_end = tb0 + std::min(ntb, (c + 1) * tpc);
        u.bend = g.boff + g.nb;
        u.pair = i;
        u.chunk = c;
        u.pad_ = 0;
        mu.push_back(u);
      }
    if (!hinf[i]) {  // the sample view: every stride-th row, tiles of 256 sampled rows
      const int ns = g.nb / stride;
      const int sb0 = g.boff / stride;  // a multiple of 256 (boff is a multiple of P)
      for (int qt = 0; qt < nqt; qt++) {
        GroupUnit u;
        u.q0 = g.qoff + qt * TC_TILE_M;
        u.qend = g.qoff + g.nq;
        u.t_begin = sb0 / TC_TILE_N;
        u.t_end = u.t_begin + (int)ceil_div(ns, TC_TILE_N);
        u.bend = sb0 + ns;
        u.pair = i;
        u.chunk = 0;
        u.pad_ = 0;
        su.push_back(u);
      }
    }
  }
  max_cand = std::min(max_cand, kMaxCandidates);
  // longest units first: the persistent CTAs take units round robin
  auto by_len = [](const GroupUnit &a, const GroupUnit &b) {
    return a.t_end - a.t_begin > b.t_end - b.t_begin;
  };
  std::stable_sort(mu.begin(), mu.end(), by_len);
  std::stable_sort(su.begin(), su.end(), by_len);
  if (mu.size() > 0x7fffffffu || su.size() > 0x7fffffffu) {
    set_error(E_UNSUPPORTED, "knn_batch: too many work units");
    return E_UNSUPPORTED;
  }

  GroupUnit *dmu, *dsu = nullptr;
  float *stopv = nullptr, *candv;
  int *cnt, *candi, *stopi = nullptr;
  YG_CHECK(gs_get(ws, GS_PAIRS, np, &dpairs));
  YG_CHECK(gs_get(ws, GS_MUNITS, mu.size(), &dmu));
  if (!su.empty()) {
    YG_CHECK(gs_get(ws, GS_SUNITS, su.size(), &dsu));
    YG_CHECK(gs_get(ws, GS_STOPV, (size_t)nq_all * 16, &stopv));
    YG_CHECK(gs_get(ws, GS_STOPI, (size_t)nq_all * 16, &stopi));
  }
  YG_CHECK(gs_get(ws, GS_CNT, cnt_tot, &cnt));
  YG_CHECK(gs_get(ws, GS_CANDV, cand_tot, &candv));
  YG_CHECK(gs_get(ws, GS_CANDI, cand_tot, &candi));
  // the host tables are copied before they go out of scope: pageable copies
  // are staged before cudaMemcpyAsync returns
  YG_CUDA(cudaMemcpyAsync(dpairs, hp.data(), sizeof(GroupPair) * np, cudaMemcpyHostToDevice, st));
  YG_CUDA(cudaMemcpyAsync(dinf, hinf.data(), np, cudaMemcpyHostToDevice, st));
  YG_CUDA(cudaMemcpyAsync(dmu, mu.data(), sizeof(GroupUnit) * mu.size(), cudaMemcpyHostToDevice,
                          st));
  if (!su.empty())
    YG_CUDA(cudaMemcpyAsync(dsu, su.data(), sizeof(GroupUnit) * su.size(),
                            cudaMemcpyHostToDevice, st));

  // ---- error bounds, per query against its own pair's statistics
  YG_CHECK(compute_eps(nq_all, d, PREC_BF16, metric, qn64, qres, qflag, nullptr, eps, qexact, st,
                       qpair, dpairs));

  TcOperands op;
  op.d = d;
  op.Kp = Kp;
  op.metric = metric;
  op.split = 0;
  op.q = qpack;
  op.qn = qnorm;
  op.b = bpack;
  op.bn = bnorm;
  op.b_rows = brows;
  op.b_step = 1;
  op.err = &status->tc_err;

  // ---- threshold sample pass and thresholds
  if (tr) cudaEventRecord(ev[1], st);
  if (!su.empty()) {
    ScanSel ss;
    ss.mode = SCAN_TOPV;
    ss.C = 16;
    ss.nchunk = 1;
    ss.topv = stopv;
    ss.topi = stopi;
    ss.units = dsu;
    ss.nunits = (int)su.size();
    ss.gpairs = dpairs;
    TcOperands ops;
    YG_CHECK(tc_base_view(op, stride, (int)(brows / stride), &ops));
    YG_CHECK(tc_scan(ops, nq_all, (int)(brows / stride), ss, st));
    YG_CHECK(thresh_from_sample(nq_all, 1, 16, kSampleC, stopv, eps, thr, st));
  }
  thr_inf_kernel<<<(unsigned)ceil_div(nq_all, 256), 256, 0, st>>>(qpair, dpairs, dinf, nq_all,
                                                                  thr);
  YG_LAUNCH_CHECK();

  // ---- main pass
  if (tr) cudaEventRecord(ev[2], st);
  ScanSel sel;
  sel.mode = SCAN_THRESH;
  sel.halves = 2;
  sel.thr = thr;
  sel.cnt = cnt;
  sel.candv = candv;
  sel.candi = candi;
  sel.units = dmu;
  sel.nunits = (int)mu.size();
  sel.gpairs = dpairs;
  YG_CHECK(tc_scan(op, nq_all, (int)brows, sel, st));

  // ---- re-rank every query against its pair
  RerankArgs ra;
  ra.nq = nq_all;
  ra.nb = 0;
  ra.d = d;
  ra.k = k;
  ra.metric = metric;
  ra.qn64 = qn64;
  ra.eps = eps;
  ra.qexact = qexact;
  ra.sel = sel;
  ra.fail_list = fail;
  ra.fail_cnt = &status->fail_cnt;
  ra.n_cand = &status->n_cand;
  ra.kth_out = kth;
  ra.m_expect = kSampleC * stride;
  ra.qpair = qpair;
  ra.gpairs = dpairs;
  ra.max_candidates = max_cand;
  if (tr) cudaEventRecord(ev[3], st);
  YG_CHECK(rerank(ra, st));
  if (tr) cudaEventRecord(ev[4], st);

  // ---- status, base statistics; queries the certificate rejected go
  // through the single-pair pipeline of their pair
  void *pin;
  YG_CHECK(ctx_pinned_status(ctx, &pin));
  YG_CUDA(cudaMemcpyAsync(pin, status, sizeof(GroupStatus), cudaMemcpyDeviceToHost, st));
  std::vector<SetStats> hs(np);
  YG_CUDA(cudaMemcpyAsync(hs.data(), stats, sizeof(SetStats) * np, cudaMemcpyDeviceToHost, st));
  YG_CUDA(cudaStreamSynchronize(st));
  GroupStatus gst;
  memcpy(&gst, pin, sizeof(gst));
  if (gst.tc_err) {
    set_error(E_TIMEOUT, "tensor-core pass gave up waiting (bounded wait expired)");
    return E_TIMEOUT;
  }
  gc->n_cand += (long long)gst.n_cand;
  for (int i = 0; i < np; i++)
    if (!hs[i].all_exact) gc->all_exact = 0;
  const int nf = gst.fail_cnt;
  if (tr) {
    float t[4];
    for (int i = 0; i < 4; i++) cudaEventElapsedTime(&t[i], ev[i], ev[i + 1]);
    fprintf(stderr,
            "[yael_gpu] grouped wave: %d pairs, %d queries, %ld base rows, %zu + %zu units: "
            "pack %.3f ms, sample %.3f ms, main %.3f ms, rerank %.3f ms, rejected %d\n",
            np, nq_all, brows, su.size(), mu.size(), t[0], t[1], t[2], t[3], nf);
    for (auto &e : ev) cudaEventDestroy(e);
  }
  if (nf == 0) return OK;
  std::vector<int> hf(nf), hqp(nf);
  YG_CUDA(cudaMemcpyAsync(hf.data(), fail, sizeof(int) * nf, cudaMemcpyDeviceToHost, st));
  YG_CUDA(cudaStreamSynchronize(st));
  std::sort(hf.begin(), hf.end());
  size_t a0 = 0;
  while (a0 < hf.size()) {
    // the failed rows of one pair (rows are concatenated pair by pair)
    int i = (int)(std::upper_bound(hp.begin(), hp.end(), hf[a0],
                                   [](int r, const GroupPair &g) { return r < g.qoff; }) -
                  hp.begin()) - 1;
    while (hp[i].nq == 0) i++;  // empty pairs share their successor's offset
    const GroupPair &g = hp[i];
    size_t a1 = a0;
    while (a1 < hf.size() && hf[a1] < g.qoff + g.nq) a1++;
    const int m = (int)(a1 - a0);
    std::vector<int> rows(m);
    for (int r = 0; r < m; r++) rows[r] = hf[a0 + r] - g.qoff;
    int *drows, *fidx;
    float *fq, *fdis;
    YG_CHECK(gs_get(ws, GS_FROWS, m, &drows));
    YG_CHECK(gs_get(ws, GS_FQ, (size_t)m * d, &fq));
    YG_CHECK(gs_get(ws, GS_FIDX, (size_t)m * k, &fidx));
    YG_CHECK(gs_get(ws, GS_FDIS, (size_t)m * k, &fdis));
    YG_CUDA(cudaMemcpyAsync(drows, rows.data(), sizeof(int) * m, cudaMemcpyHostToDevice, st));
    gather_rows_k<<<(unsigned)ceil_div((long)m * d, 256), 256, 0, st>>>(g.q, d, drows, m, fq);
    YG_LAUNCH_CHECK();
    KnnJob job;
    job.nq = m; job.nb = g.nb; job.d = d; job.k = k; job.metric = metric; job.prec = PREC_BF16;
    job.q = fq; job.ldq = d; job.b = g.b; job.ldb = d;
    job.out_idx = fidx; job.out_dis = fdis;
    YG_CHECK(knn_device(job, ctx, st));
    scatter_rows_k<<<(unsigned)ceil_div((long)m * k, 256), 256, 0, st>>>(fidx, fdis, drows, m, k,
                                                                         g.out_idx, g.out_dis);
    YG_LAUNCH_CHECK();
    YG_CUDA(cudaStreamSynchronize(st));  // rows is a host vector of this iteration
    gc->n_band += m + job.n_band;
    gc->n_second += job.n_second;
    gc->n_fallback += job.n_fallback;
    a0 = a1;
  }
  return OK;
}

}  // namespace

bool knn_grouped_eligible(int d, int k, int prec, int device_ptrs) {
  static const bool on = [] {
    const char *e = getenv("YAEL_GPU_BATCH_GROUPED");
    return !(e && e[0] == '0');
  }();
  return on && device_ptrs && prec == PREC_BF16 && k >= 9 && k <= kMaxK && tc_supported(d);
}

int knn_grouped(int npairs, const yael_gpu_knn_pair *pairs, int d, int k, int metric,
                cudaStream_t st, GroupCounters *gc) {
  Ctx *ctx;
  YG_CHECK(ctx_get(&ctx));
  const int Kp = ((d + 63) / 64) * 64;
  const int stride = std::max(1, k / 3);
  const long P = (long)TC_TILE_N * stride;
  // waves of pairs whose buffers stay within a budget (YAEL_GPU_GROUP_BYTES)
  size_t budget = (size_t)24 << 30;
  if (const char *e = getenv("YAEL_GPU_GROUP_BYTES")) {
    const double v = atof(e);
    if (v > 0) budget = (size_t)v;
  }
  std::vector<Wave> waves(1);
  size_t used = 0;
  for (int i = 0; i < npairs; i++) {
    const yael_gpu_knn_pair &x = pairs[i];
    int nreg, cap, tpc;
    pair_layout(x.nb, stride, pair_inf(x.nb, stride), &nreg, &cap, &tpc);
    const size_t bytes = (size_t)round_up(x.nb, P) * (Kp * 2 + 32) +
                         (size_t)x.nq * (Kp * 2 + 32 + 128) +
                         (size_t)x.nq * nreg * ((size_t)cap * 8 + 4);
    if (used > 0 && used + bytes > budget) {
      waves.emplace_back();
      used = 0;
    }
    waves.back().pairs.push_back(i);
    used += bytes;
  }
  for (const Wave &w : waves) YG_CHECK(run_wave(pairs, w, d, k, metric, ctx, st, gc));
  return OK;
}

}  // namespace yg
