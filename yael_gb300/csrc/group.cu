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
__global__ void thr_inf_kernel(const int *qpair, const unsigned char *inf, int nq, float *thr) {
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

// Everything a wave's passes need, on the device, plus the host copy of its
// pair table for the final checks.  Two sets of buffers alternate between
// consecutive waves, so wave i + 1 is packed while wave i's passes run.
struct WaveState {
  int np = 0, nq_all = 0, stride = 1, max_cand = 0;
  long brows = 0;
  std::vector<GroupPair> hp;
  size_t n_mu = 0, n_su = 0;
  __nv_bfloat16 *bpack = nullptr, *bnorm = nullptr, *qpack = nullptr, *qnorm = nullptr;
  double *qn64 = nullptr;
  unsigned char *qflag = nullptr, *qexact = nullptr, *dinf = nullptr;
  float *qres = nullptr, *eps = nullptr, *thr = nullptr, *kth = nullptr, *stopv = nullptr;
  float *candv = nullptr;
  int *qpair = nullptr, *fail = nullptr, *cnt = nullptr, *candi = nullptr, *stopi = nullptr;
  SetStats *stats = nullptr;
  GroupPair *dpairs = nullptr;
  GroupUnit *dmu = nullptr, *dsu = nullptr;
  GroupStatus *status = nullptr;
  cudaEvent_t ev[5] = {};  // trace: pack | sample | main | rerank
};

constexpr int kSetSlots = 32;  // slot distance between the two buffer sets

// Phase 1 (stream sp): layout, buffers of set `set`, packing, unit tables,
// error bounds.
int wave_prepare(const yael_gpu_knn_pair *pairs, const Wave &w, int d, int k, int metric,
                 Ctx *ctx, int set, cudaStream_t sp, WaveState &S) {
  Workspace &ws = ctx->ws;
  const int o = set * kSetSlots;
  const int np = (int)w.pairs.size();
  const int Kp = ((d + 63) / 64) * 64;
  const bool L2 = metric == METRIC_L2;
  const int stride = std::max(1, k / 3);
  const long P = (long)TC_TILE_N * stride;
  S.np = np;
  S.stride = stride;
  // ---- layout
  std::vector<GroupPair> &hp = S.hp;
  hp.assign(np, GroupPair());
  std::vector<unsigned char> hinf(np);
  long brows = 0;
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
    hinf[i] = pair_inf(x.nb, stride) ? 1 : 0;
  }
  S.nq_all = nq_all;
  S.brows = brows;
  if (nq_all == 0) return OK;
  if (brows > 0x7fffffffL) {
    set_error(E_UNSUPPORTED, "knn_batch: %ld padded base rows in one group", brows);
    return E_UNSUPPORTED;
  }
  // ---- buffers
  YG_CHECK(gs_get(ws, o + GS_BPACK, (size_t)brows * Kp, &S.bpack));
  if (L2) YG_CHECK(gs_get(ws, o + GS_BNORM, (size_t)brows * 16, &S.bnorm));
  YG_CHECK(gs_get(ws, o + GS_QPACK, (size_t)nq_all * Kp, &S.qpack));
  if (L2) YG_CHECK(gs_get(ws, o + GS_QNORM, (size_t)nq_all * 16, &S.qnorm));
  YG_CHECK(gs_get(ws, o + GS_QN64, nq_all, &S.qn64));
  YG_CHECK(gs_get(ws, o + GS_QFLAG, nq_all, &S.qflag));
  YG_CHECK(gs_get(ws, o + GS_QRES, nq_all, &S.qres));
  YG_CHECK(gs_get(ws, o + GS_EPS, nq_all, &S.eps));
  YG_CHECK(gs_get(ws, o + GS_QEXACT, nq_all, &S.qexact));
  YG_CHECK(gs_get(ws, o + GS_THR, nq_all, &S.thr));
  YG_CHECK(gs_get(ws, o + GS_KTH, nq_all, &S.kth));
  YG_CHECK(gs_get(ws, o + GS_FAIL, nq_all, &S.fail));
  YG_CHECK(gs_get(ws, o + GS_QPAIR, nq_all, &S.qpair));
  YG_CHECK(gs_get(ws, o + GS_STATS, np, &S.stats));
  YG_CHECK(gs_get(ws, o + GS_INF, np, &S.dinf));
  YG_CHECK(gs_get(ws, o + GS_STATUS, 1, &S.status));
  for (int i = 0; i < np; i++) hp[i].bs = S.stats + i;

  // trace: events between the passes (YAEL_GPU_TRACE)
  if (trace_enabled()) {
    for (auto &e : S.ev) cudaEventCreate(&e);
    cudaEventRecord(S.ev[0], sp);
  }

  // ---- packing: every pair's base and queries into the concatenated buffers
  stats_init_kernel<<<(unsigned)ceil_div(np, 128), 128, 0, sp>>>(S.stats, np);
  YG_LAUNCH_CHECK();
  YG_CUDA(cudaMemsetAsync(S.status, 0, sizeof(GroupStatus), sp));
  const float qscale = L2 ? -2.f : 1.f;
  for (int i = 0; i < np; i++) {
    const GroupPair &g = hp[i];
    YG_CHECK(prep_rows(g.b, d, g.nb, d, 1.f, nullptr, nullptr, nullptr, nullptr,
                       S.bpack + (size_t)g.boff * Kp, Kp,
                       L2 ? S.bnorm + (size_t)g.boff * 16 : nullptr, L2 ? 1 : 0, S.stats + i,
                       sp));
    if (g.nq == 0) continue;
    YG_CHECK(prep_rows(g.q, d, g.nq, d, qscale, S.qn64 + g.qoff, nullptr, S.qflag + g.qoff,
                       S.qres + g.qoff, S.qpack + (size_t)g.qoff * Kp, Kp,
                       L2 ? S.qnorm + (size_t)g.qoff * 16 : nullptr, L2 ? 2 : 0, nullptr, sp));
    qpair_kernel<<<(unsigned)ceil_div(g.nq, 256), 256, 0, sp>>>(S.qpair, i, g.qoff, g.nq);
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
  S.max_cand = std::min(max_cand, kMaxCandidates);
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
  S.n_mu = mu.size();
  S.n_su = su.size();
  YG_CHECK(gs_get(ws, o + GS_PAIRS, np, &S.dpairs));
  YG_CHECK(gs_get(ws, o + GS_MUNITS, mu.size(), &S.dmu));
  if (!su.empty()) {
    YG_CHECK(gs_get(ws, o + GS_SUNITS, su.size(), &S.dsu));
    YG_CHECK(gs_get(ws, o + GS_STOPV, (size_t)nq_all * 16, &S.stopv));
    YG_CHECK(gs_get(ws, o + GS_STOPI, (size_t)nq_all * 16, &S.stopi));
  }
  YG_CHECK(gs_get(ws, o + GS_CNT, cnt_tot, &S.cnt));
  YG_CHECK(gs_get(ws, o + GS_CANDV, cand_tot, &S.candv));
  YG_CHECK(gs_get(ws, o + GS_CANDI, cand_tot, &S.candi));
  // the host tables are copied before they go out of scope: pageable copies
  // are staged before cudaMemcpyAsync returns
  YG_CUDA(cudaMemcpyAsync(S.dpairs, hp.data(), sizeof(GroupPair) * np, cudaMemcpyHostToDevice,
                          sp));
  YG_CUDA(cudaMemcpyAsync(S.dinf, hinf.data(), np, cudaMemcpyHostToDevice, sp));
  YG_CUDA(cudaMemcpyAsync(S.dmu, mu.data(), sizeof(GroupUnit) * mu.size(),
                          cudaMemcpyHostToDevice, sp));
  if (!su.empty())
    YG_CUDA(cudaMemcpyAsync(S.dsu, su.data(), sizeof(GroupUnit) * su.size(),
                            cudaMemcpyHostToDevice, sp));

  // ---- error bounds, per query against its own pair's statistics
  YG_CHECK(compute_eps(nq_all, d, PREC_BF16, metric, S.qn64, S.qres, S.qflag, nullptr, S.eps,
                       S.qexact, sp, S.qpair, S.dpairs));
  return OK;
}

// Phase 2 (stream st): the sample pass, thresholds, main pass and re-rank.
// max_ctas > 0 leaves SMs free for the next wave's packing.
int wave_execute(WaveState &S, int d, int k, int metric, int max_ctas, cudaStream_t st) {
  if (S.nq_all == 0) return OK;
  const int Kp = ((d + 63) / 64) * 64;
  TcOperands op;
  op.d = d;
  op.Kp = Kp;
  op.metric = metric;
  op.split = 0;
  op.q = S.qpack;
  op.qn = S.qnorm;
  op.b = S.bpack;
  op.bn = S.bnorm;
  op.b_rows = S.brows;
  op.b_step = 1;
  op.err = &S.status->tc_err;
  if (S.ev[1]) cudaEventRecord(S.ev[1], st);
  if (S.n_su) {
    ScanSel ss;
    ss.mode = SCAN_TOPV;
    ss.C = 16;
    ss.nchunk = 1;
    ss.topv = S.stopv;
    ss.topi = S.stopi;
    ss.units = S.dsu;
    ss.nunits = (int)S.n_su;
    ss.gpairs = S.dpairs;
    ss.max_ctas = max_ctas;
    TcOperands ops;
    YG_CHECK(tc_base_view(op, S.stride, (int)(S.brows / S.stride), &ops));
    YG_CHECK(tc_scan(ops, S.nq_all, (int)(S.brows / S.stride), ss, st));
    YG_CHECK(thresh_from_sample(S.nq_all, 1, 16, kSampleC, S.stopv, S.eps, S.thr, st));
  }
  thr_inf_kernel<<<(unsigned)ceil_div(S.nq_all, 256), 256, 0, st>>>(S.qpair, S.dinf, S.nq_all,
                                                                    S.thr);
  YG_LAUNCH_CHECK();
  if (S.ev[2]) cudaEventRecord(S.ev[2], st);
  ScanSel sel;
  sel.mode = SCAN_THRESH;
  sel.halves = 2;
  sel.thr = S.thr;
  sel.cnt = S.cnt;
  sel.candv = S.candv;
  sel.candi = S.candi;
  sel.units = S.dmu;
  sel.nunits = (int)S.n_mu;
  sel.gpairs = S.dpairs;
  sel.max_ctas = max_ctas;
  YG_CHECK(tc_scan(op, S.nq_all, (int)S.brows, sel, st));
  if (S.ev[3]) cudaEventRecord(S.ev[3], st);
  RerankArgs ra;
  ra.nq = S.nq_all;
  ra.nb = 0;
  ra.d = d;
  ra.k = k;
  ra.metric = metric;
  ra.qn64 = S.qn64;
  ra.eps = S.eps;
  ra.qexact = S.qexact;
  ra.sel = sel;
  ra.fail_list = S.fail;
  ra.fail_cnt = &S.status->fail_cnt;
  ra.n_cand = &S.status->n_cand;
  ra.kth_out = S.kth;
  ra.m_expect = kSampleC * S.stride;
  ra.qpair = S.qpair;
  ra.gpairs = S.dpairs;
  ra.max_candidates = S.max_cand;
  YG_CHECK(rerank(ra, st));
  if (S.ev[4]) cudaEventRecord(S.ev[4], st);
  return OK;
}

// Phase 3 (stream st, host sync): status, base statistics; the queries the
// certificate rejected go through the single-pair pipeline of their pair.
int wave_finish(WaveState &S, int d, int k, int metric, Ctx *ctx, int set, cudaStream_t st,
                GroupCounters *gc) {
  if (S.nq_all == 0) return OK;
  Workspace &ws = ctx->ws;
  const int o = set * kSetSlots;
  const int np = S.np;
  void *pin;
  YG_CHECK(ctx_pinned_status(ctx, &pin));
  YG_CUDA(cudaMemcpyAsync(pin, S.status, sizeof(GroupStatus), cudaMemcpyDeviceToHost, st));
  std::vector<SetStats> hs(np);
  YG_CUDA(cudaMemcpyAsync(hs.data(), S.stats, sizeof(SetStats) * np, cudaMemcpyDeviceToHost, st));
  YG_CUDA(cudaStreamSynchronize(st));
  GroupStatus gst;
  memcpy(&gst, pin, sizeof(gst));
  if (S.ev[0]) {
    float t[4];
    for (int i = 0; i < 4; i++) cudaEventElapsedTime(&t[i], S.ev[i], S.ev[i + 1]);
    fprintf(stderr,
            "[yael_gpu] grouped wave: %d pairs, %d queries, %ld base rows, %zu + %zu units: "
            "pack %.3f ms (to the passes' start), sample %.3f ms, main %.3f ms, rerank %.3f ms, "
            "rejected %d\n",
            np, S.nq_all, S.brows, S.n_su, S.n_mu, t[0], t[1], t[2], t[3], gst.fail_cnt);
    for (auto &e : S.ev) {
      cudaEventDestroy(e);
      e = nullptr;
    }
  }
  if (gst.tc_err) {
    set_error(E_TIMEOUT, "tensor-core pass gave up waiting (bounded wait expired)");
    return E_TIMEOUT;
  }
  gc->n_cand += (long long)gst.n_cand;
  for (int i = 0; i < np; i++)
    if (!hs[i].all_exact) gc->all_exact = 0;
  const int nf = gst.fail_cnt;
  if (nf == 0) return OK;
  std::vector<int> hf(nf);
  YG_CUDA(cudaMemcpyAsync(hf.data(), S.fail, sizeof(int) * nf, cudaMemcpyDeviceToHost, st));
  YG_CUDA(cudaStreamSynchronize(st));
  std::sort(hf.begin(), hf.end());
  const std::vector<GroupPair> &hp = S.hp;
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
    YG_CHECK(gs_get(ws, o + GS_FROWS, m, &drows));
    YG_CHECK(gs_get(ws, o + GS_FQ, (size_t)m * d, &fq));
    YG_CHECK(gs_get(ws, o + GS_FIDX, (size_t)m * k, &fidx));
    YG_CHECK(gs_get(ws, o + GS_FDIS, (size_t)m * k, &fdis));
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
  // waves of pairs whose buffers stay within a budget (YAEL_GPU_GROUP_BYTES;
  // two waves' buffers are live at a time)
  static const bool pipeline = [] {
    const char *e = getenv("YAEL_GPU_GROUP_PIPELINE");
    return !(e && e[0] == '0');
  }();
  size_t budget = (size_t)(pipeline ? 16 : 24) << 30;
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
  // Pipeline (YAEL_GPU_GROUP_PIPELINE=0 turns it off): wave i + 1 is packed on
  // a side stream while wave i's passes run on st with a grid that leaves
  // YAEL_GPU_GROUP_PACK_SMS (default 24) SMs to the packing, whose blocks do
  // not fit beside a distance-pass CTA.  512-pair batch: 93.7 ms pipelined,
  // 97.4 ms one wave after the other (8 to 48 reserved SMs: 93.9-95.7 ms).
  int pack_sms = 24;
  if (const char *e = getenv("YAEL_GPU_GROUP_PACK_SMS")) pack_sms = std::max(0, atoi(e));
  const int pass_ctas = std::max(1, ctx->num_sms - pack_sms);
  cudaStream_t sp = nullptr;
  YG_CUDA(cudaStreamCreateWithFlags(&sp, cudaStreamNonBlocking));
  struct StreamGuard {
    cudaStream_t s;
    ~StreamGuard() { cudaStreamDestroy(s); }
  } guard{sp};
  cudaEvent_t packed[2];
  YG_CUDA(cudaEventCreateWithFlags(&packed[0], cudaEventDisableTiming));
  YG_CUDA(cudaEventCreateWithFlags(&packed[1], cudaEventDisableTiming));
  struct EventGuard {
    cudaEvent_t *e;
    ~EventGuard() { cudaEventDestroy(e[0]); cudaEventDestroy(e[1]); }
  } eguard{packed};
  const int nw = (int)waves.size();
  WaveState S[2];
  // the first wave packs alone: full-size blocks
  YG_CHECK(wave_prepare(pairs, waves[0], d, k, metric, ctx, 0, sp, S[0]));
  YG_CUDA(cudaEventRecord(packed[0], sp));
  for (int i = 0; i < nw; i++) {
    const int cur = i & 1, nxt = cur ^ 1;
    YG_CUDA(cudaStreamWaitEvent(st, packed[cur], 0));
    YG_CHECK(wave_execute(S[cur], d, k, metric, pipeline && i + 1 < nw ? pass_ctas : 0, st));
    if (pipeline && i + 1 < nw) {
      // set nxt was last used by wave i - 1, finished before this iteration
      YG_CHECK(wave_prepare(pairs, waves[i + 1], d, k, metric, ctx, nxt, sp, S[nxt]));
      YG_CUDA(cudaEventRecord(packed[nxt], sp));
    }
    YG_CHECK(wave_finish(S[cur], d, k, metric, ctx, cur, st, gc));
    if (!pipeline && i + 1 < nw) {
      YG_CHECK(wave_prepare(pairs, waves[i + 1], d, k, metric, ctx, nxt, sp, S[nxt]));
      YG_CUDA(cudaEventRecord(packed[nxt], sp));
    }
  }
  YG_CUDA(cudaStreamSynchronize(sp));
  return OK;
}

}  // namespace yg
