// k-means Lloyd loop and hierarchical k-means on the GPU: the host control
// flow of yael/kmeans.c:166-447 and yael/hkm.c:36-232 (seeds, init, empty
// cluster splits, stopping rules, outputs) around the device step of
// kmeans.cuh.  Every random draw is the reference's, from libc rand_r /
// lrand48 in the same order, so runs are reproducible against it.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include <algorithm>
#include <memory>
#include <vector>

#include "alt.cuh"
#include "kmeans.cuh"
#include "knn.cuh"
#include "km_host.h"
#include "../../include/yael_gpu.h"

namespace yg {

namespace {

template <typename T>
int ws_get(Workspace &ws, int slot, size_t count, T **p) {
  void *v = nullptr;
  YG_CHECK(ws.get(slot, count * sizeof(T) + 16, &v));
  *p = reinterpret_cast<T *>(v);
  return OK;
}

enum KmSlot : int {
  KS_V = WS_KM0, KS_C, KS_ASSIGN, KS_DIS, KS_COUNTS, KS_OFFS, KS_CURSOR, KS_PERM, KS_ACC,
  KS_SHIFT, KS_ACTIVE, KS_PINST, KS_WORK, KS_SLICES, KS_PART, KS_ROWS, KS_AMAX,
  KS_BEST_C, KS_BEST_DIS, KS_BEST_ASSIGN, KS_NODE, KS_VSORT, KS_TMP, KS_CPREV,
  KS_AKEYS, KS_AKEYS2, KS_AVALS, KS_AVALS2, KS_AOFFS, KS_ATMP, KS_ASORT,
  // the small-k tensor-core assignment
  KS_TCU = 160, KS_TCPK, KS_TCSIDE, KS_TCXN, KS_TCXRES, KS_TCCPK, KS_TCCSIDE, KS_TCSTATS,
  KS_TCERR, KS_PRIOR, KS_TCMU, KS_TCMUPART, KS_TCSLF, KS_TCNPT, KS_TCHMAX,
  KS_HSTART, KS_HPINST, KS_GCNT, KS_GTOT, KS_TCTSIDE, KS_TCCSCR, KS_TCIB, KS_SPLITROWS,
  KS_SPLITBUF,
};

// the split centroid rows put back: row r of src to row rows[r] of dst
__global__ void scatter_rows64_kernel(const float *src, const long *rows, long m, int d,
                                      float *dst) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= m * d) return;
  const long r = t / d;
  dst[rows[r] * d + (t - r * d)] = src[t];
}

int fixed_shift(long n, float maxabs) {
  int e = 0;
  if (maxabs > 0) frexp((double)maxabs, &e);
  int lg = 0;
  while ((1L << lg) < n) lg++;
  return 62 - lg - e;
}

// ---- the batched Lloyd engine --------------------------------------------

double wall_ms() {
  timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec * 1e3 + ts.tv_nsec * 1e-6;
}

// statistics of the calling thread's last kmeans / hkm call (yael_gpu_last_stats)
thread_local yael_gpu_call_stats g_last_stats = {};

struct Instance {
  long p0 = 0;
  int n = 0;
  unsigned seed = 0;  // the kmeans() seed after the seed_in -> unsigned conversion
  unsigned core = 0;  // rand_r stream of kmeans_core
  int tot_re = 0, iters = 0, ret = 0;
  double qerr = HUGE_VAL, qerr_old = HUGE_VAL;
  bool done = false;
};

struct Engine {
  Ctx *ctx;
  cudaStream_t st;
  int d, k, niter, flags, prec;
  bool verbose;
  const float *v;  // device points (all instances, contiguous)
  long ntot;
  std::vector<Instance> in;
  // device buffers
  float *C, *dis, *amax;
  float *inst_mu = nullptr, *inst_cmax = nullptr;  // per instance: mean, max |v - mean|
  std::vector<float> hcmax;
  int *assign, *counts, *shift, *pinst;
  const int *pinst_given = nullptr;  // the points' instances, when the caller has them on the device
  unsigned char *active;
  long *offs, *cursor, *perm, *rows;
  long long *acc;
  KmWork *work;
  KmSlice *slices;
  double *part;
  int nwork = 0, nsl = 0;
  std::vector<KmSlice> hsl;
  std::vector<int> hcounts;
  std::vector<double> hpart;
  long n_fallback = 0, n_second = 0, n_band = 0;
  float ms_assign = 0, ms_update = 0;
  long point_iters = 0, engine_iters = 0;  // sum of active points per iteration; iterations

  // CUDA graphs of one Lloyd iteration's device work: the update always, the
  // assignment on the grouped small-k path (the k-NN path reads its
  // certificate results on the host).  Both are captured on the second
  // iteration (the first runs eagerly and sets every kernel attribute) and
  // replayed after.
  // Their arguments never change within a run: the per-iteration state (active
  // instances, split centroids) lives in device buffers written between
  // replays.  YAEL_GPU_GRAPHS=0 runs every iteration eagerly.
  cudaGraphExec_t g_assign = nullptr, g_update = nullptr;
  bool eager_done = false;
  // The chosen form's assignment for k <= 256 (km_tc.cu): the 16-bit tensor
  // cores with an exact band re-check, and, when k * d fits shared memory, the
  // centroid sums fused into it (no second pass over the points).
  bool tc = false, tc_fuse = false;
  bool tc_live = false;  // the fused sums hold the last assignment's (reset per run)
  KmTcUnit *tc_units = nullptr;
  int tc_nunits = 0;
  KmTcPoints tcP;
  void *tc_cpk = nullptr, *tc_cside = nullptr;
  SetStats *tc_cstats = nullptr;
  int *tc_err = nullptr;
  int *ph_err = nullptr;  // pinned copy of tc_err the update graph writes
  bool assign_settled = false;  // the grouped assignment's variant is tuned
  long g_assign_n = 0, g_update_n = 0;  // kernels per replay
  bool graphs_failed = false;
  int *ph_counts = nullptr;     // pinned copies the update graph writes
  double *ph_part = nullptr;

  ~Engine() {
    if (g_assign) cudaGraphExecDestroy(g_assign);
    if (g_update) cudaGraphExecDestroy(g_update);
  }

  // L1 / chi2 k-means (one instance): per-coordinate distances searched
  // exhaustively, medians / chi2 minimisers as centroids
  bool alt_mode() const { return (flags & (YAEL_KMEANS_L1 | YAEL_KMEANS_CHI2)) != 0; }

  bool graphs_wanted() const {
    static const bool on = [] {
      const char *e = getenv("YAEL_GPU_GRAPHS");
      return !(e && e[0] == '0');
    }();
    return on && !graphs_failed && !alt_mode();
  }
  bool assign_graph_wanted() const {
    return graphs_wanted() && (tc || !(in.size() == 1 && k > kSmallK));
  }

  // captures body() on st into *exec; false (and eager mode) on any failure
  template <typename F>
  bool capture(F body, cudaGraphExec_t *exec, long *nlaunch) {
    const long l0 = launch_count();
    if (cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed) != cudaSuccess) {
      (void)cudaGetLastError();
      return false;
    }
    const int rc = body();
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(st, &g);
    // uploaded here, so that the first replay does not carry the upload
    bool ok = rc == OK && e == cudaSuccess && g != nullptr &&
              cudaGraphInstantiate(exec, g, 0) == cudaSuccess &&
              cudaGraphUpload(*exec, st) == cudaSuccess;
    if (g) cudaGraphDestroy(g);
    if (!ok) {
      (void)cudaGetLastError();
      *exec = nullptr;
    }
    *nlaunch = launch_count() - l0;
    return ok;
  }

  int setup() {
    Workspace &ws = ctx->ws;
    const int ni = (int)in.size();
    const long ncl = (long)ni * k;
    YG_CHECK(ws_get(ws, KS_C, (size_t)ncl * d, &C));
    YG_CHECK(ws_get(ws, KS_ASSIGN, (size_t)ntot, &assign));
    YG_CHECK(ws_get(ws, KS_DIS, (size_t)ntot, &dis));
    YG_CHECK(ws_get(ws, KS_COUNTS, (size_t)ncl, &counts));
    YG_CHECK(ws_get(ws, KS_OFFS, (size_t)ncl + 1, &offs));
    YG_CHECK(ws_get(ws, KS_CURSOR, (size_t)ncl, &cursor));
    YG_CHECK(ws_get(ws, KS_PERM, (size_t)ntot, &perm));
    YG_CHECK(ws_get(ws, KS_ACC, (size_t)ncl * d, &acc));
    YG_CHECK(ws_get(ws, KS_SHIFT, (size_t)ni, &shift));
    YG_CHECK(ws_get(ws, KS_ACTIVE, (size_t)ni, &active));
    YG_CHECK(ws_get(ws, KS_AMAX, (size_t)ni, &amax));
    pinst = nullptr;
    std::vector<KmWork> hw;
    hsl.clear();
    std::vector<int> hpinst;
    const bool host_pinst = ni > 1 && !pinst_given;
    if (host_pinst) hpinst.resize(ntot);
    for (int i = 0; i < ni; i++) {
      for (long o = 0; o < in[i].n; o += kAssignChunk)
        hw.push_back({i, in[i].p0 + o, (int)std::min<long>(kAssignChunk, in[i].n - o)});
      for (long o = 0; o < in[i].n; o += kSliceLen)
        hsl.push_back({in[i].p0 + o, (int)std::min<long>(kSliceLen, in[i].n - o), i});
      if (host_pinst)
        for (long p = 0; p < in[i].n; p++) hpinst[in[i].p0 + p] = i;
    }
    nwork = (int)hw.size();
    nsl = (int)hsl.size();
    YG_CHECK(ws_get(ws, KS_WORK, (size_t)nwork, &work));
    YG_CHECK(ws_get(ws, KS_SLICES, (size_t)nsl, &slices));
    YG_CHECK(ws_get(ws, KS_PART, (size_t)nsl, &part));
    YG_CUDA(cudaMemcpyAsync(work, hw.data(), sizeof(KmWork) * nwork, cudaMemcpyHostToDevice, st));
    YG_CUDA(cudaMemcpyAsync(slices, hsl.data(), sizeof(KmSlice) * nsl, cudaMemcpyHostToDevice, st));
    if (host_pinst) {
      YG_CHECK(ws_get(ws, KS_PINST, (size_t)ntot, &pinst));
      YG_CUDA(cudaMemcpyAsync(pinst, hpinst.data(), sizeof(int) * ntot, cudaMemcpyHostToDevice, st));
    } else if (ni > 1) {
      pinst = const_cast<int *>(pinst_given);
    }
    // per instance: max |v| (the fixed-point shift of the exact integer sums),
    // the mean mu and max |v - mu| (the translation of the 16-bit packing)
    {
      float *part;
      int *slf;
      long *npt;
      YG_CHECK(ws_get(ws, KS_TCMU, (size_t)ni * d, &inst_mu));
      YG_CHECK(ws_get(ws, KS_TCMUPART, (size_t)std::max(1, nsl) * d * 3, &part));
      YG_CHECK(ws_get(ws, KS_TCSLF, (size_t)ni * 2, &slf));
      YG_CHECK(ws_get(ws, KS_TCNPT, (size_t)ni, &npt));
      YG_CHECK(ws_get(ws, KS_TCHMAX, (size_t)ni, &inst_cmax));
      std::vector<int> hf((size_t)ni * 2, 0);
      std::vector<long> hn(ni);
      for (int s = nsl - 1; s >= 0; s--) {
        hf[hsl[s].inst] = s;
        hf[ni + hsl[s].inst]++;
      }
      for (int i = 0; i < ni; i++) hn[i] = in[i].n;
      YG_CUDA(cudaMemcpyAsync(slf, hf.data(), sizeof(int) * hf.size(), cudaMemcpyHostToDevice,
                              st));
      YG_CUDA(cudaMemcpyAsync(npt, hn.data(), sizeof(long) * ni, cudaMemcpyHostToDevice, st));
      YG_CHECK(km_inst_stats(slices, nsl, v, d, ni, slf, slf + ni, npt, part, inst_mu, amax,
                             inst_cmax, st));
      hcmax.resize(ni);
      YG_CUDA(cudaMemcpyAsync(hcmax.data(), inst_cmax, sizeof(float) * ni,
                              cudaMemcpyDeviceToHost, st));
      YG_CUDA(cudaStreamSynchronize(st));  // hf, hn are host buffers
    }
    std::vector<float> ha(ni);
    YG_CUDA(cudaMemcpyAsync(ha.data(), amax, sizeof(float) * ni, cudaMemcpyDeviceToHost, st));
    YG_CUDA(cudaStreamSynchronize(st));
    std::vector<int> hs(ni);
    for (int i = 0; i < ni; i++) hs[i] = fixed_shift(in[i].n, ha[i]);
    // every centroid is a mean of points (or a split of one, 1e-7 apart), so
    // |c| <= max |v| and ||c|| <= sqrt(d) max |v|: fp16 holds both operands of
    // the assignment when that norm stays below 128 (||c||^2 < 2^14)
    f16_fits = ni == 1 && ha[0] >= 0.f && ha[0] * sqrtf((float)d) < 128.f;
    YG_CUDA(cudaMemcpyAsync(shift, hs.data(), sizeof(int) * ni, cudaMemcpyHostToDevice, st));
    hcounts.resize(ncl);
    hpart.resize(nsl);
    // pinned host buffers of the context (grow-only, kept across calls)
    YG_CHECK(ctx->pinned.get(0, sizeof(int) * (size_t)ncl, reinterpret_cast<void **>(&ph_counts)));
    YG_CHECK(ctx->pinned.get(1, sizeof(double) * (size_t)std::max(1, nsl),
                             reinterpret_cast<void **>(&ph_part)));
    YG_CHECK(ctx->pinned.get(2, sizeof(int), reinterpret_cast<void **>(&ph_err)));
    *ph_err = 0;
    float hmax = 0.f;
    for (int i = 0; i < ni; i++) hmax = ha[i] > hmax ? ha[i] : (ha[i] >= 0.f ? hmax : NAN);
    const double ts0 = trace_enabled() ? wall_ms() : 0.0;
    YG_CHECK(setup_tc(hmax));
    if (trace_enabled()) {
      YG_CUDA(cudaStreamSynchronize(st));
      fprintf(stderr, "[yael_gpu] engine set-up: tensor-core packing %.3f ms\n", wall_ms() - ts0);
    }
    YG_CUDA(cudaStreamSynchronize(st));
    return OK;
  }

  // The small-k tensor-core assignment: the chosen form (a 16-bit pass) for
  // k <= 256 and aligned rows with d % 4 == 0.  Its unit table (tiles of up
  // to 128 points of one instance) and the points' 16-bit packing are built
  // once; the centroids are packed at every assignment.
  int setup_tc(float hmax) {
    tc = (prec == PREC_BF16 || prec == PREC_FP16) && !alt_mode() && km_tc_supported(d, k, v, C);
    if (!tc) return OK;
    tc_fuse = true;  // the sums come with the assignment (shared memory or global atomics)
    Workspace &ws = ctx->ws;
    const int ni = (int)in.size();
    const long ncl = (long)ni * k;
    // every instance's rows (points and centroids) are packed relative to its
    // mean: the 16-bit rounding errors then scale with the instance's spread,
    // which is what the bound on the distances needs
    {
      float hc = 0.f;
      for (int i = 0; i < ni; i++) hc = hcmax[i] > hc ? hcmax[i] : (hcmax[i] >= 0.f ? hc : NAN);
      // centroids are means of the instance's points (a split moves one by
      // 1e-7 relative), so |c - mu| stays within the points' |x - mu| plus
      // that much of max |x|
      hmax = hmax >= 0.f && hc >= 0.f ? hc + 1e-6f * hmax : NAN;
    }
    std::vector<KmTcUnit> hu;
    for (int i = 0; i < ni; i++)
      for (long o = 0; o < in[i].n; o += 128)
        hu.push_back({i, (int)std::min<long>(128, in[i].n - o), in[i].p0 + o});
    tc_nunits = (int)hu.size();
    YG_CHECK(ws_get(ws, KS_TCU, hu.size(), &tc_units));
    YG_CUDA(cudaMemcpyAsync(tc_units, hu.data(), sizeof(KmTcUnit) * hu.size(),
                            cudaMemcpyHostToDevice, st));
    // fp16 operands when every value and every centroid norm fits (see f16_fits)
    tcP.f16 = hmax >= 0.f && hmax * sqrtf((float)d) < 128.f;
    tcP.Kp = ((d + 63) / 64) * 64;
    tcP.n = ntot;
    uint16_t *pk, *side, *cpk, *cside;
    YG_CHECK(ws_get(ws, KS_TCPK, (size_t)ntot * tcP.Kp, &pk));
    YG_CHECK(ws_get(ws, KS_TCSIDE, (size_t)ntot * 16, &side));
    YG_CHECK(ws_get(ws, KS_TCXN, (size_t)ntot, &tcP.xn64));
    YG_CHECK(ws_get(ws, KS_TCXRES, (size_t)ntot, &tcP.xres));
    YG_CHECK(ws_get(ws, KS_TCCPK, (size_t)ncl * tcP.Kp, &cpk));
    YG_CHECK(ws_get(ws, KS_TCCSIDE, (size_t)ncl * 16, &cside));
    YG_CHECK(ws_get(ws, KS_TCSTATS, 1, &tc_cstats));
    YG_CHECK(ws_get(ws, KS_TCERR, 1, &tc_err));
    YG_CUDA(cudaMemsetAsync(tc_err, 0, sizeof(int), st));
    tcP.pk = pk;
    tcP.side = side;
    tc_cpk = cpk;
    tc_cside = cside;
    tcP.mu = inst_mu;
    RowShift rs;
    rs.mu = inst_mu;
    rs.row_inst = ni > 1 ? pinst : nullptr;
    rs.rows_per_inst = (int)ntot;
    YG_CHECK(prep_rows(v, d, (int)ntot, d, -2.f, tcP.xn64, nullptr, nullptr, tcP.xres,
                       (__nv_bfloat16 *)pk, tcP.Kp, (__nv_bfloat16 *)side, 2, nullptr, st, 8,
                       tcP.f16, rs));
    YG_CHECK(ws_get(ws, KS_TCTSIDE, (size_t)tc_nunits * 128, &tcP.tside));
    YG_CHECK(km_tc_tile_side(tc_units, tc_nunits, tcP.xn64, tcP.xres, tcP.tside, st));
    assign_settled = true;  // no variant tuner on this path
    return OK;
  }

  // random-point initialisation of every instance (yael/kmeans.c:401-405)
  int init_random() {
    const int ni = (int)in.size();
    std::vector<long> hrows((size_t)ni * k);
    for (int i = 0; i < ni; i++) {
      if (in[i].n < k) {  // a node too small for k clusters: one child per point
        for (int j = 0; j < k; j++) hrows[(size_t)i * k + j] = in[i].p0 + std::min(j, in[i].n - 1);
        continue;
      }
      random_init_first_k(in[i].n, k, rand_r(&in[i].seed), hrows.data() + (size_t)i * k);
      for (int j = 0; j < k; j++) hrows[(size_t)i * k + j] += in[i].p0;
    }
    YG_CHECK(ws_get(ctx->ws, KS_ROWS, hrows.size(), &rows));
    YG_CUDA(cudaMemcpyAsync(rows, hrows.data(), sizeof(long) * hrows.size(),
                            cudaMemcpyHostToDevice, st));
    YG_CHECK(km_gather(v, d, rows, (long)hrows.size(), C, st));
    return OK;
  }

  std::vector<unsigned char> hactive;  // the flags last written to the device

  int set_active() {
    std::vector<unsigned char> h(in.size());
    for (size_t i = 0; i < in.size(); i++) h[i] = !in[i].done;
    if (h == hactive) return OK;
    YG_CUDA(cudaMemcpyAsync(active, h.data(), h.size(), cudaMemcpyHostToDevice, st));
    YG_CUDA(cudaStreamSynchronize(st));  // h is a stack buffer
    hactive = h;
    return OK;
  }

  // When the 16-bit certificate rejects more than 60% of the points, the band
  // passes that settle them cost more than running the whole assignment on
  // the 3xBF16 split operands (measured on the large configuration: band
  // passes ~32 ns per rejected point on bf16 crowding, the split pass ~19 ns
  // more per point than the 16-bit one); later iterations see similar
  // centroid geometry, so the switch is kept for the rest of the run.
  bool split_assign = false;
  // The 16-bit tensor-core pass of the chosen form runs on fp16 operands when
  // the data range allows (the same tensor rate as bf16, 8x finer rounding,
  // so an 8x narrower error band and far fewer points sent to later passes)
  bool f16_fits = false;
  int prec_used = -1;  // the distance pass of the last assignment
  // per-iteration record (yael_gpu_kmeans_opts' probe fields), single instance
  const yael_gpu_kmeans_opts *probe = nullptr;
  long probe_t = 0;
  std::vector<int> probe_all;
  // The k-NN assignment defers its certificate check to the end of the
  // iteration (the update is queued right behind it); rejected points are
  // settled then and the update is run again.  Only after an iteration that
  // rejected under 1% of the points: a pass that rejects many (BF16 on close
  // centroids) does better with the in-line band passes.
  KnnJob pend;
  long last_rejected = -1;  // rejected points of the previous assignment
  // From the second iteration of a run on, the chosen form's k-NN assignment
  // starts from each point's distance to its previous centroid's new
  // position, an upper bound of its nearest distance: a THRESH pass with those
  // thresholds finds every possible winner with the cheapest selection, and no
  // sample pass.  (The plain FP32 path keeps its list pass: its CUDA-core
  // scan does not gain from the cheaper selection.)
  bool have_prev = false;

  void count_assign(const KnnJob &job) {
    last_rejected = (long)job.n_band + job.n_fallback;
    n_fallback += job.n_fallback;
    n_second += job.n_second;
    n_band += job.n_band;
    if ((job.prec == PREC_BF16 || job.prec == PREC_FP16) &&
        10L * (job.n_band + job.n_fallback) > 6L * (long)job.nq)
      split_assign = true;
  }

  int assign_step() {
    if (tc) {
      const long ncl = (long)in.size() * k;
      // the sums start from zero once per run; later assignments add the
      // points that change centroid (the sums stay those of the assignment)
      const int delta = tc_fuse && tc_live ? 1 : 0;
      if (tc_fuse && !tc_live) {
        YG_CUDA(cudaMemsetAsync(acc, 0, sizeof(long long) * ncl * d, st));
        YG_CUDA(cudaMemsetAsync(counts, 0, sizeof(int) * ncl, st));
      }
      tc_live = tc_fuse;
      prec_used = tcP.f16 ? PREC_FP16 : PREC_BF16;
      float *cscr;
      float2 *ib;
      YG_CHECK(ws_get(ctx->ws, KS_TCCSCR, (size_t)ncl * 2, &cscr));
      YG_CHECK(ws_get(ctx->ws, KS_TCIB, in.size(), &ib));
      return km_tc_assign(tc_units, tc_nunits, tcP, v, d, C, (int)in.size(), k, tc_cpk,
                          tc_cside, cscr, ib, tc_cstats, active, assign, dis,
                          tc_fuse ? acc : nullptr, tc_fuse ? counts : nullptr, shift, delta,
                          tc_err, st);
    }
    if (alt_mode()) {
      // yael/kmeans.c:242-244: knn_full with distance type 1 (L1) or 3 (chi2)
      KnnJob job;
      job.nq = in[0].n; job.nb = k; job.d = d; job.k = 1;
      job.metric = METRIC_ALT0 + ((flags & YAEL_KMEANS_L1) ? 1 : 3);
      job.prec = PREC_FP32;
      prec_used = PREC_FP32;
      job.q = v + in[0].p0 * d; job.ldq = d; job.b = C; job.ldb = d;
      job.out_idx = assign + in[0].p0; job.out_dis = dis + in[0].p0;
      return knn_device(job, ctx, st);
    }
    if (in.size() == 1 && k > kSmallK) {
      KnnJob job;
      job.nq = in[0].n; job.nb = k; job.d = d; job.k = 1; job.metric = METRIC_L2;
      job.prec = prec == PREC_BF16 ? (split_assign ? PREC_BF16X3 : f16_fits ? PREC_FP16 : prec)
                                   : prec;
      prec_used = job.prec;
      job.q = v + in[0].p0 * d; job.ldq = d; job.b = C; job.ldb = d;
      job.out_idx = assign + in[0].p0; job.out_dis = dis + in[0].p0;
      // YAEL_GPU_KMEANS_DEFER=0 / 1: never / always defer (default: adaptive)
      static const int defer_mode = [] {
        const char *e = getenv("YAEL_GPU_KMEANS_DEFER");
        return e && *e ? atoi(e) : -1;
      }();
      job.defer = defer_mode == 1 ||
                  (defer_mode != 0 && last_rejected >= 0 && 100 * last_rejected < (long)job.nq);
      if (have_prev && job.prec != PREC_FP32) {
        float *kth;
        YG_CHECK(ws_get(ctx->ws, KS_PRIOR, (size_t)in[0].n, &kth));
        YG_CHECK(km_prior_bound(job.q, d, in[0].n, job.out_idx, C, kth, st));
        job.prior_kth = kth;
      }
      YG_CHECK(knn_device(job, ctx, st));
      have_prev = true;
      if (job.pending) {
        // the update queued next overwrites C: the rejected points are settled
        // against a copy of this iteration's centroids
        float *cprev;
        YG_CHECK(ws_get(ctx->ws, KS_CPREV, (size_t)k * d, &cprev));
        YG_CUDA(cudaMemcpyAsync(cprev, C, sizeof(float) * (size_t)k * d, cudaMemcpyDeviceToDevice,
                                st));
        job.b = cprev;
        pend = job;
      } else {
        count_assign(job);
      }
      return OK;
    }
    prec_used = PREC_FP32;
    return km_assign_small(work, nwork, v, d, C, k, active, assign, dis, st);
  }

  // one Lloyd iteration for every active instance (yael/kmeans.c:237-318)
  int iterate() {
    const int ni = (int)in.size();
    const long ncl = (long)ni * k;
    const double t_host0 = trace_enabled() ? wall_ms() : 0.0;
    for (auto &x : in)
      if (!x.done) {
        x.iters++;
        point_iters += x.n;
      }
    engine_iters++;
    cudaEvent_t e0, e1, e2;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventCreate(&e2);
    auto update_body = [&]() -> int {
      if (tc_fuse) {
        // the sums and counts came with the assignment; the counts, the error
        // flag and the objective's slice sums are written straight to the
        // pinned host buffers (no copies in the step)
        YG_CHECK(km_finalize(acc, counts, ncl, d, k, shift, active, C, st, ph_counts, tc_err,
                             ph_err));
        if (flags & YAEL_KMEANS_NORMALIZE_CENTS) YG_CHECK(km_normalize(C, ncl, d, k, active, st));
        YG_CHECK(km_slice_sums(slices, nsl, dis, ph_part, st));
        return OK;
      }
      if (tc) YG_CUDA(cudaMemcpyAsync(ph_err, tc_err, sizeof(int), cudaMemcpyDeviceToHost, st));
      YG_CUDA(cudaMemsetAsync(counts, 0, sizeof(int) * ncl, st));
      YG_CHECK(km_histogram(assign, pinst, ntot, k, active, counts, st));
      if (alt_mode()) {
        Workspace &ws = ctx->ws;
        int *keys, *keys2, *vals, *vals2, *offs2;
        float *tmp;
        void *sort_tmp;
        const size_t sb = km_alt_sort_bytes(ntot);
        YG_CHECK(ws_get(ws, KS_AKEYS, (size_t)ntot, &keys));
        YG_CHECK(ws_get(ws, KS_AKEYS2, (size_t)ntot, &keys2));
        YG_CHECK(ws_get(ws, KS_AVALS, (size_t)ntot, &vals));
        YG_CHECK(ws_get(ws, KS_AVALS2, (size_t)ntot, &vals2));
        YG_CHECK(ws_get(ws, KS_AOFFS, (size_t)k + 1, &offs2));
        YG_CHECK(ws_get(ws, KS_ATMP, (size_t)ntot * d, &tmp));
        YG_CHECK(ctx->ws.get(KS_ASORT, sb ? sb : 1, &sort_tmp));
        YG_CHECK(km_alt_update(assign, ntot, v, d, k, (flags & YAEL_KMEANS_L1) != 0, keys, keys2,
                               vals, vals2, offs2, tmp, sort_tmp, sb, C, st));
        if (flags & YAEL_KMEANS_NORMALIZE_CENTS) {
          if (flags & YAEL_KMEANS_L1) YG_CHECK(km_normalize_l1(C, ncl, d, st));
          else YG_CHECK(km_normalize(C, ncl, d, k, active, st));
        }
        YG_CHECK(km_slice_sums(slices, nsl, dis, part, st));
        YG_CUDA(cudaMemcpyAsync(ph_counts, counts, sizeof(int) * ncl, cudaMemcpyDeviceToHost, st));
        YG_CUDA(cudaMemcpyAsync(ph_part, part, sizeof(double) * nsl, cudaMemcpyDeviceToHost, st));
        return OK;
      }
      YG_CHECK(km_scan(counts, ncl, offs, cursor, st));
      YG_CHECK(km_scatter(assign, pinst, ntot, k, active, cursor, perm, st));
      YG_CHECK(km_update(perm, offs + ncl, ntot, assign, pinst, counts, v, d, ncl, k, shift,
                         active, acc, C, st));
      if (flags & YAEL_KMEANS_NORMALIZE_CENTS) YG_CHECK(km_normalize(C, ncl, d, k, active, st));
      YG_CHECK(km_slice_sums(slices, nsl, dis, part, st));
      YG_CUDA(cudaMemcpyAsync(ph_counts, counts, sizeof(int) * ncl, cudaMemcpyDeviceToHost, st));
      YG_CUDA(cudaMemcpyAsync(ph_part, part, sizeof(double) * nsl, cudaMemcpyDeviceToHost, st));
      return OK;
    };
    const bool probing = probe && probe->n_probe > 0 && ni == 1 && probe_t < probe->probe_iters;
    if (probing && probe->probe_centroids) {
      YG_CUDA(cudaMemcpyAsync(probe->probe_centroids + (size_t)probe_t * k * d, C,
                              sizeof(float) * (size_t)k * d, cudaMemcpyDeviceToHost, st));
      YG_CUDA(cudaStreamSynchronize(st));
    }
    const bool use_graphs = graphs_wanted() && eager_done;
    // the assignment is captured once its kernel variant is tuned (the
    // tuner's trials run eagerly)
    // (a run's first fused assignment starts its sums: eager, as it differs)
    const bool graph_assign =
        use_graphs && assign_graph_wanted() && assign_settled && !(tc_fuse && !tc_live);
    if (use_graphs && !g_update && !capture(update_body, &g_update, &g_update_n))
      graphs_failed = true;
    if (graph_assign && !g_assign && !graphs_failed &&
        !capture([&] { return assign_step(); }, &g_assign, &g_assign_n))
      graphs_failed = true;
    cudaEventRecord(e0, st);
    std::unique_ptr<NvtxRange> nv(new NvtxRange("kmeans.assign"));
    if (graph_assign && !graphs_failed) {
      YG_CUDA(cudaGraphLaunch(g_assign, st));
      count_launches(g_assign_n);
    } else {
      YG_CHECK(assign_step());
    }
    cudaEventRecord(e1, st);
    nv.reset(new NvtxRange("kmeans.update"));
    if (use_graphs && !graphs_failed) {
      YG_CUDA(cudaGraphLaunch(g_update, st));
      count_launches(g_update_n);
    } else {
      YG_CHECK(update_body());
    }
    eager_done = true;
    cudaEventRecord(e2, st);
    YG_CUDA(cudaStreamSynchronize(st));
    if (!g_assign) assign_settled = km_assign_tune_collect();
    if (pend.pending) {
      YG_CHECK(knn_resolve(pend, ctx, st));
      count_assign(pend);
      if (pend.n_band > 0) {  // some points were re-run: their clusters changed
        if (use_graphs && !graphs_failed) {
          YG_CUDA(cudaGraphLaunch(g_update, st));
          count_launches(g_update_n);
        } else {
          YG_CHECK(update_body());
        }
        YG_CUDA(cudaStreamSynchronize(st));
      }
    }
    if (tc && *ph_err) {
      set_error(E_TIMEOUT, "k-means tensor-core assignment gave up waiting (bounded wait expired)");
      return E_TIMEOUT;
    }
    std::copy(ph_counts, ph_counts + ncl, hcounts.begin());
    std::copy(ph_part, ph_part + nsl, hpart.begin());
    float a = 0, b = 0;
    cudaEventElapsedTime(&a, e0, e1);
    cudaEventElapsedTime(&b, e1, e2);
    ms_assign += a;
    ms_update += b;
    if (trace_enabled())
      fprintf(stderr, "[yael_gpu] kmeans iteration %ld: assign %.3f ms, update %.3f ms (events), "
              "%.3f ms on the host clock\n", engine_iters, a, b, wall_ms() - t_host0);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaEventDestroy(e2);

    // objective per instance: slice sums in point order
    std::vector<double> q(ni, 0.0);
    for (int s = 0; s < nsl; s++) q[hsl[s].inst] += hpart[s];
    if (probing) {
      probe_all.resize(ntot);
      YG_CUDA(cudaMemcpyAsync(probe_all.data(), assign, sizeof(int) * ntot,
                              cudaMemcpyDeviceToHost, st));
      YG_CUDA(cudaStreamSynchronize(st));
      int *dst = probe->probe_assign + (size_t)probe_t * probe->n_probe;
      for (int i = 0; i < probe->n_probe; i++) {
        const long r = probe->probe_rows[i];
        dst[i] = r >= 0 && r < ntot ? probe_all[r] : -1;
      }
      if (probe->probe_qerr) probe->probe_qerr[probe_t] = q[0];
      probe_t++;
    }

    nv.reset(new NvtxRange("kmeans.split_and_stop"));
    // the splits: planned per instance here, applied to the rows they touch
    // after the loop (an instance's steps touch its own rows only)
    std::vector<SplitStep> plan;
    std::vector<int> plan_inst, plan_at;  // instance, first step
    for (int i = 0; i < ni; i++) {
      Instance &x = in[i];
      if (x.done) continue;
      // empty clusters -> split (the draw happens every iteration)
      const unsigned sseed = rand_r(&x.core);
      const int *cnt = hcounts.data() + (long)i * k;
      bool empty = false;
      for (int c = 0; c < k; c++) empty |= cnt[c] == 0;
      int nre = 0;
      if (empty) {
        plan_inst.push_back(i);
        plan_at.push_back((int)plan.size());
        nre = split_plan(k, cnt, sseed, plan);
        if (nre > 0 && verbose)
          fprintf(stderr, "# kmeans warning: %d empty clusters -> split\n", nre);
      }
      x.tot_re += nre;
      if (x.tot_re > x.n / 100 && x.tot_re > 1000) {
        fprintf(stderr, "# kmeans: reassigned %d times, abandoning\n", x.tot_re);
        x.ret = -1;
        x.done = true;
        continue;
      }
      x.qerr_old = x.qerr;
      x.qerr = q[i];
      if (x.qerr_old == x.qerr && nre == 0) {
        x.done = true;
        continue;
      }
      if (verbose) {
        printf(" -> %.3f", x.qerr / x.n);
        fflush(stdout);
      }
      if (x.iters >= niter) x.done = true;
    }
    if (!plan.empty()) YG_CHECK(apply_splits(plan, plan_inst, plan_at));
    return set_active();
  }

  // the planned splits on the device centroids: the rows they touch
  // gathered, split on the host, put back
  int apply_splits(const std::vector<SplitStep> &plan, const std::vector<int> &pinst,
                   const std::vector<int> &pat) {
    SplitRows sr;
    split_rows(k, plan, pinst, pat, sr);
    const long m = (long)sr.rows.size();
    long *drows;
    float *dbuf;
    YG_CHECK(ws_get(ctx->ws, KS_SPLITROWS, (size_t)m, &drows));
    YG_CHECK(ws_get(ctx->ws, KS_SPLITBUF, (size_t)m * d, &dbuf));
    std::vector<float> R((size_t)m * d);
    YG_CUDA(cudaMemcpyAsync(drows, sr.rows.data(), sizeof(long) * m, cudaMemcpyHostToDevice, st));
    YG_CHECK(km_gather(C, d, drows, m, dbuf, st));
    YG_CUDA(cudaMemcpyAsync(R.data(), dbuf, sizeof(float) * m * d, cudaMemcpyDeviceToHost, st));
    YG_CUDA(cudaStreamSynchronize(st));
    split_apply_rows(d, k, plan, pinst, pat, sr, R.data());
    YG_CUDA(cudaMemcpyAsync(dbuf, R.data(), sizeof(float) * m * d, cudaMemcpyHostToDevice, st));
    scatter_rows64_kernel<<<(unsigned)ceil_div(m * d, 256), 256, 0, st>>>(dbuf, drows, m, d, C);
    YG_LAUNCH_CHECK();
    YG_CUDA(cudaStreamSynchronize(st));  // R and sr are stack buffers
    return OK;
  }

  bool all_done() const {
    for (auto &x : in)
      if (!x.done) return false;
    return true;
  }
};

// D2H of whichever outputs are requested (device or host destinations)
int copy_out(Ctx *ctx, cudaStream_t st, void *dst, const void *src, size_t bytes, bool dev) {
  if (!dst || bytes == 0) return OK;
  if (!dev) return copy_to_host(ctx, st, dst, src, bytes);
  YG_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, st));
  return OK;
}

// kmeans++ initialisation (yael/kmeans.c:27-82): squared distances to each
// newly selected point on the GPU (FP64, rounded to float), the sampling
// (normalisation and the sequential double subtraction) on the host
__global__ void kpp_kernel(const float *v, int d, long n, long newsel, float *best) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0;
  for (int c = 0; c < d; c++) {
    const double t = (double)v[i * d + c] - (double)v[newsel * d + c];
    s = add_sq64(s, t);
  }
  const float f = (float)s;
  if (f < best[i]) best[i] = f;
}

__global__ void fill_kernel(float *p, long n, float x) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = x;
}

int kmeanspp(Ctx *ctx, cudaStream_t st, const float *v, int d, int nsub, int k, bool verbose,
             unsigned seed, long *sel) {
  float *best;
  YG_CHECK(ws_get(ctx->ws, KS_TMP, (size_t)nsub, &best));
  fill_kernel<<<(unsigned)ceil_div(nsub, 256), 256, 0, st>>>(best, nsub, HUGE_VALF);
  YG_LAUNCH_CHECK();
  std::vector<float> h(nsub);
  sel[0] = rand_r(&seed) % k;  // the reference draws modulo k here
  for (int i = 1; i < k; i++) {
    if (verbose && i % 10 == 0) {
      printf("%d/%d\r", i, k);
      fflush(stdout);
    }
    kpp_kernel<<<(unsigned)ceil_div(nsub, 256), 256, 0, st>>>(v, d, nsub, sel[i - 1], best);
    YG_LAUNCH_CHECK();
    YG_CUDA(cudaMemcpyAsync(h.data(), best, sizeof(float) * nsub, cudaMemcpyDeviceToHost, st));
    YG_CUDA(cudaStreamSynchronize(st));
    mul_by(h.data(), nsub, 1. / l1(h.data(), nsub));
    double rd = drand_r_(&seed);
    long j;
    for (j = 0; j < nsub - 1; j++) {
      rd -= h[j];
      if (rd < 0) break;
    }
    sel[i] = j;
  }
  if (verbose) printf("\n");
  return OK;
}

}  // namespace

// kmeans() (yael/kmeans.c:332-447) on device or host buffers
int kmeans_run(int d, int n, int k, int niter, const float *v_in, int flags, long seed_in,
               int redo, float *C_out, float *dis_out, int *assign_out, int *nassign_out,
               int prec, bool dev, cudaStream_t st_in, float *ret_out, long *iters_out,
               long *fallback_out, long *second_out, float *ms_assign, float *ms_update,
               long *band_out = nullptr, yael_gpu_kmeans_opts *xo = nullptr) {
  Ctx *ctx;
  YG_CHECK(ctx_get(&ctx));
  cudaStream_t st = st_in ? st_in : ctx->stream;
  const bool verbose = !(flags & YAEL_KMEANS_QUIET);
  niter = niter == 0 ? 1000000 : niter;
  const bool user = (flags & YAEL_KMEANS_INIT_USER) != 0;
  if (user) {
    if (!C_out) {
      set_error(E_ARG, "kmeans: KMEANS_INIT_USER needs the initial centroids");
      return E_ARG;
    }
    redo = 1;
  }
  if (k > n || k < 1 || d < 1) {
    set_error(E_ARG, "kmeans: k=%d n=%d d=%d (the reference asserts k <= n)", k, n, d);
    return E_ARG;
  }
  const bool tr = trace_enabled();
  const double t_call = tr ? wall_ms() : 0.0;
  double t_init = 0.0, t_iter = 0.0;
  const float *v = v_in;
  if (!dev) {
    float *dv;
    YG_CHECK(ws_get(ctx->ws, KS_V, (size_t)n * d, &dv));
    YG_CUDA(cudaMemcpyAsync(dv, v_in, sizeof(float) * (size_t)n * d, cudaMemcpyHostToDevice, st));
    v = dv;
  }
  if (seed_in == 0) seed_in = lrand48();
  Engine E;
  E.ctx = ctx; E.st = st; E.d = d; E.k = k; E.niter = niter; E.flags = flags; E.prec = prec;
  E.verbose = verbose; E.v = v; E.ntot = n;
  E.in.resize(1);
  E.in[0].n = n;
  E.in[0].seed = (unsigned)seed_in;
  if (xo && xo->n_probe > 0) {
    if (!xo->probe_rows || !xo->probe_assign || xo->probe_iters < 0) {
      set_error(E_ARG, "kmeans: probe_rows and probe_assign are needed with n_probe > 0");
      return E_ARG;
    }
    E.probe = xo;
  }
  YG_CHECK(E.setup());
  if (tr) YG_CUDA(cudaStreamSynchronize(st));
  const double t_setup = tr ? wall_ms() : 0.0;
  double best = HUGE_VAL;
  long iter_tot = 0;
  int core_ret = 0;
  float *bC = nullptr, *bdis = nullptr;
  int *bassign = nullptr;
  std::vector<int> bnassign(k);
  for (int run = 0; run < redo; run++) {
    if (verbose) printf("<><><><> kmeans / run %d <><><><><>\n", run);
    const double t_r0 = tr ? wall_ms() : 0.0;
    Instance &x = E.in[0];
    if (user) {
      YG_CUDA(cudaMemcpyAsync(E.C, C_out, sizeof(float) * (size_t)k * d,
                              dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st));
    } else if (flags & YAEL_KMEANS_INIT_BERKELEY) {
      int nsub = n;
      if (n > k * 8 && n > 8192) {
        nsub = k * 8;
        if (verbose) printf("Restricting k-means++ initialization to %d points\n", nsub);
      }
      std::vector<long> sel(k);
      YG_CHECK(kmeanspp(ctx, st, v, d, nsub, k, verbose, rand_r(&x.seed), sel.data()));
      long *rows;
      YG_CHECK(ws_get(ctx->ws, KS_ROWS, (size_t)k, &rows));
      YG_CUDA(cudaMemcpyAsync(rows, sel.data(), sizeof(long) * k, cudaMemcpyHostToDevice, st));
      YG_CHECK(km_gather(v, d, rows, k, E.C, st));
      YG_CUDA(cudaStreamSynchronize(st));
    } else {
      YG_CHECK(E.init_random());
    }
    x.core = rand_r(&x.seed);
    x.tot_re = 0; x.iters = 0; x.ret = 0; x.done = false;
    E.have_prev = false;
    E.tc_live = false;
    x.qerr = HUGE_VAL; x.qerr_old = HUGE_VAL;
    YG_CHECK(E.set_active());
    if (tr) YG_CUDA(cudaStreamSynchronize(st));
    const double t_run = tr ? wall_ms() : 0.0;
    while (!E.all_done()) YG_CHECK(E.iterate());
    if (tr) {
      const double t_end = wall_ms();
      t_init += t_run - t_r0;
      t_iter += t_end - t_run;
    }
    if (verbose) printf("\n");
    iter_tot += x.iters;
    core_ret = x.ret;
    if (core_ret < 0) break;
    if (x.qerr < best) {
      best = x.qerr;
      if (redo > 1) {
        // keep this run's outputs on the device until a better run replaces them
        YG_CHECK(ws_get(ctx->ws, KS_BEST_C, (size_t)k * d, &bC));
        YG_CHECK(ws_get(ctx->ws, KS_BEST_DIS, (size_t)n, &bdis));
        YG_CHECK(ws_get(ctx->ws, KS_BEST_ASSIGN, (size_t)n, &bassign));
        YG_CUDA(cudaMemcpyAsync(bC, E.C, sizeof(float) * (size_t)k * d, cudaMemcpyDeviceToDevice, st));
        YG_CUDA(cudaMemcpyAsync(bdis, E.dis, sizeof(float) * n, cudaMemcpyDeviceToDevice, st));
        YG_CUDA(cudaMemcpyAsync(bassign, E.assign, sizeof(int) * n, cudaMemcpyDeviceToDevice, st));
      } else {
        bC = E.C; bdis = E.dis; bassign = E.assign;
      }
      bnassign.assign(E.hcounts.begin(), E.hcounts.begin() + k);
    }
  }
  const double t_loop = tr ? wall_ms() : 0.0;
  if (trace_enabled())
    fprintf(stderr,
            "[yael_gpu] kmeans n=%d k=%d d=%d iterations=%ld assign=%.3fms update=%.3fms "
            "graphs(assign=%d update=%d failed=%d) tc=%d fused=%d prec=%d\n",
            n, k, d, iter_tot, E.ms_assign, E.ms_update, E.g_assign != nullptr,
            E.g_update != nullptr, (int)E.graphs_failed, (int)E.tc, (int)E.tc_fuse, E.prec_used);
  if (verbose && core_ret >= 0) {
    printf("Total number of iterations: %ld\n", iter_tot);
    // unbalanced factor of the last iteration's counts (yael/vector.c:2301-2314)
    double tot = 0, uf = 0;
    for (int c = 0; c < k; c++) {
      tot += E.hcounts[c];
      uf += E.hcounts[c] * (double)E.hcounts[c];
    }
    printf("Unbalanced factor of last iteration: %g\n", uf * k / (tot * tot));
  }
  if (best < HUGE_VAL && bC) {
    YG_CHECK(copy_out(ctx, st, C_out, bC, sizeof(float) * (size_t)k * d, dev));
    YG_CHECK(copy_out(ctx, st, dis_out, bdis, sizeof(float) * (size_t)n, dev));
    YG_CHECK(copy_out(ctx, st, assign_out, bassign, sizeof(int) * (size_t)n, dev));
    if (nassign_out) {
      YG_CUDA(cudaMemcpyAsync(nassign_out, bnassign.data(), sizeof(int) * k,
                              dev ? cudaMemcpyHostToDevice : cudaMemcpyHostToHost, st));
    }
  }
  YG_CUDA(cudaStreamSynchronize(st));
  if (tr)
    fprintf(stderr,
            "[yael_gpu] kmeans call: set-up %.3f ms, init %.3f ms, iterations %.3f ms, wrap-up "
            "%.3f ms (host clock)\n",
            t_setup - t_call, t_init, t_iter, wall_ms() - t_loop);
  if (iters_out) *iters_out = iter_tot;
  if (fallback_out) *fallback_out = E.n_fallback;
  if (second_out) *second_out = E.n_second;
  if (band_out) *band_out = E.n_band;
  if (xo) xo->prec_used = E.prec_used;
  g_last_stats = yael_gpu_call_stats{iter_tot, E.point_iters, E.engine_iters, E.ms_assign,
                                     E.ms_update, E.prec_used};
  if (ms_assign) *ms_assign = E.ms_assign;
  if (ms_update) *ms_update = E.ms_update;
  *ret_out = core_ret < 0 ? -1.f : (float)(best / n);
  return OK;
}

// ---- hierarchical k-means (yael/hkm.c) -----------------------------------

__global__ void node_update_kernel(const long *perm_sorted, const int *child, long n, int bf,
                                   int *node) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const long p = perm_sorted[i];
  node[p] = node[p] * bf + child[i];
}

int hkm_run(int n, int d, int nlevel, int bf, const float *points, int niter, bool verbose,
            int prec, bool small_nodes, float **levels_out, int *assign_out, long *iters_out,
            float *ms_out) {
  Ctx *ctx;
  YG_CHECK(ctx_get(&ctx));
  cudaStream_t st = ctx->stream;
  float *dv, *vs;
  int *node;
  long *sorted;
  YG_CHECK(ws_get(ctx->ws, KS_V, (size_t)n * d, &dv));
  YG_CHECK(ws_get(ctx->ws, KS_VSORT, (size_t)n * d, &vs));
  YG_CHECK(ws_get(ctx->ws, KS_NODE, (size_t)n, &node));
  YG_CHECK(ws_get(ctx->ws, KS_TMP, (size_t)n * 2, &sorted));
  YG_CUDA(cudaMemcpyAsync(dv, points, sizeof(float) * (size_t)n * d, cudaMemcpyHostToDevice, st));
  YG_CUDA(cudaMemsetAsync(node, 0, sizeof(int) * n, st));
  long k = 1, iters = 0;
  yael_gpu_call_stats stats = {};
  cudaEvent_t t0, t1;
  cudaEventCreate(&t0);
  cudaEventCreate(&t1);
  cudaEventRecord(t0, st);
  for (int l = 0; l < nlevel; l++) {
    NvtxRange nv_level("hkm.level");
    const double tl0 = trace_enabled() ? wall_ms() : 0.0;
    // points grouped by parent, stable in point index (ivec_sort_index,
    // hkm.c:56-62), on the device; the nodes' first points come back
    std::vector<long> start(k + 1, 0);
    long *dstart;
    int *dpinst;
    YG_CHECK(ws_get(ctx->ws, KS_HSTART, (size_t)k + 1, &dstart));
    YG_CHECK(ws_get(ctx->ws, KS_HPINST, (size_t)n, &dpinst));
    YG_CHECK(km_group_by_key(node, n, (int)k, sorted, dstart, k > 1 ? dpinst : nullptr, ctx->ws,
                             KS_GCNT, KS_GTOT, st));
    YG_CUDA(cudaMemcpyAsync(start.data(), dstart, sizeof(long) * (size_t)(k + 1),
                            cudaMemcpyDeviceToHost, st));
    YG_CHECK(km_gather(dv, d, sorted, n, vs, st));
    YG_CUDA(cudaStreamSynchronize(st));  // start
    const double tla = trace_enabled() ? wall_ms() : 0.0;
    Engine E;
    E.ctx = ctx; E.st = st; E.d = d; E.k = bf; E.niter = niter == 0 ? 1000000 : niter;
    E.flags = YAEL_KMEANS_INIT_RANDOM | YAEL_KMEANS_QUIET;
    E.prec = prec; E.verbose = false; E.v = vs; E.ntot = n;
    E.pinst_given = k > 1 ? dpinst : nullptr;
    E.in.resize(k);
    for (long p = 0; p < k; p++) {
      const long na = start[p + 1] - start[p];
      if (verbose)
        fprintf(stderr, "[Level %d | Parent %ld] nassign=%ld | pos=%ld\n", l, p, na, start[p]);
      if (na == 0) {
        fprintf(stderr, "# Problem2: no enough vectors in a node\n");
        exit(1);
      }
      if (na < bf && !small_nodes) {
        set_error(E_ARG, "hkm: node %ld of level %d has %ld points < bf=%d (kmeans asserts k <= n)",
                  p, l, na, bf);
        return E_ARG;
      }
      Instance &x = E.in[p];
      x.p0 = start[p];
      x.n = (int)na;
      x.seed = (unsigned)lrand48();  // kmeans(..., seed 0, ...) per child, in parent order
      x.done = na < bf;              // small node: no k-means (see yael_gpu_hkm_learn_ex)
    }
    YG_CHECK(E.setup());
    const double tlb = trace_enabled() ? wall_ms() : 0.0;
    YG_CHECK(E.init_random());
    std::vector<int> iota(bf);
    for (int j = 0; j < bf; j++) iota[j] = j;
    for (auto &x : E.in) {
      x.core = rand_r(&x.seed);
      if (x.done)  // each point is its own child
        YG_CUDA(cudaMemcpyAsync(E.assign + x.p0, iota.data(), sizeof(int) * x.n,
                                cudaMemcpyHostToDevice, st));
    }
    YG_CUDA(cudaStreamSynchronize(st));
    YG_CHECK(E.set_active());
    const double tl1 = trace_enabled() ? wall_ms() : 0.0;
    while (!E.all_done()) YG_CHECK(E.iterate());
    const double tl2 = trace_enabled() ? wall_ms() : 0.0;
    for (auto &x : E.in) iters += x.iters;
    stats.point_iterations += E.point_iters;
    stats.level_iterations += E.engine_iters;
    stats.ms_assign += E.ms_assign;
    stats.ms_update += E.ms_update;
    stats.prec_used = E.prec_used;
    // centroids of this level, then node = node * bf + child
    node_update_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, st>>>(sorted, E.assign, n, bf, node);
    YG_LAUNCH_CHECK();
    YG_CHECK(copy_to_host(ctx, st, levels_out[l], E.C, sizeof(float) * (size_t)k * bf * d));
    if (trace_enabled())
      fprintf(stderr, "[yael_gpu] hkm level %d: %ld nodes, set-up %.3f ms (grouping %.3f, engine "
              "%.3f, init %.3f), iterations %.3f ms, wrap-up %.3f ms (host clock)\n", l, k,
              tl1 - tl0, tla - tl0, tlb - tla, tl1 - tlb, tl2 - tl1, wall_ms() - tl2);
    k *= bf;
  }
  cudaEventRecord(t1, st);
  YG_CUDA(cudaStreamSynchronize(st));
  if (ms_out) cudaEventElapsedTime(ms_out, t0, t1);
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  if (assign_out) YG_CHECK(copy_to_host(ctx, st, assign_out, node, sizeof(int) * (size_t)n));
  if (iters_out) *iters_out = iters;
  stats.instance_iterations = iters;
  g_last_stats = stats;
  return OK;
}

// greedy descent (yael/hkm.c:131-150) with exact L2 (FP32 + FP64 near ties)
__global__ void hkm_quantize_kernel(const float *cent, int nlevel, int bf, int d, long n,
                                    const float *v, int *idx) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float *x = v + i * d;
  const float rho = (float)(d + 4) * 5.9604645e-08f;
  long vw = 0, off = 0, k = bf;
  for (int l = 0; l < nlevel; l++) {
    const float *C = cent + off + vw * (long)bf * d;
    float b1 = 1e30f, b2 = 1e30f;
    int i1 = -1;
    for (int j = 0; j < bf; j++) {
      float s = 0.f;
      for (int c = 0; c < d; c++) {
        const float t = x[c] - C[(long)j * d + c];
        s = fmaf(t, t, s);
      }
      if (s < b1) { b2 = b1; b1 = s; i1 = j; } else if (s < b2) { b2 = s; }
    }
    if (i1 >= 0 && b2 < 1e30f && b2 - b1 <= rho * (b1 + b2)) {
      double best = INFINITY;
      for (int j = 0; j < bf; j++) {
        double s = 0;
        for (int c = 0; c < d; c++) {
          const double t = (double)x[c] - (double)C[(long)j * d + c];
          s = add_sq64(s, t);
        }
        if (s < best) { best = s; i1 = j; }
      }
    }
    vw = vw * bf + (i1 < 0 ? 0 : i1);
    off += k * d;
    k *= bf;
  }
  idx[i] = (int)vw;
}

int hkm_quantize_run(int nlevel, int bf, int d, float *const *levels, int n, const float *v,
                     int *idx) {
  if (n <= 0) return OK;
  Ctx *ctx;
  YG_CHECK(ctx_get(&ctx));
  cudaStream_t st = ctx->stream;
  long tot = 0, k = bf;
  for (int l = 0; l < nlevel; l++, k *= bf) tot += k * d;
  float *dc, *dv;
  int *di;
  YG_CHECK(ws_get(ctx->ws, KS_BEST_C, (size_t)tot, &dc));
  YG_CHECK(ws_get(ctx->ws, KS_V, (size_t)n * d, &dv));
  YG_CHECK(ws_get(ctx->ws, KS_ASSIGN, (size_t)n, &di));
  k = bf;
  long off = 0;
  for (int l = 0; l < nlevel; l++, k *= bf) {
    YG_CUDA(cudaMemcpyAsync(dc + off, levels[l], sizeof(float) * k * d, cudaMemcpyHostToDevice, st));
    off += k * d;
  }
  YG_CUDA(cudaMemcpyAsync(dv, v, sizeof(float) * (size_t)n * d, cudaMemcpyHostToDevice, st));
  hkm_quantize_kernel<<<(unsigned)ceil_div(n, 128), 128, 0, st>>>(dc, nlevel, bf, d, n, dv, di);
  YG_LAUNCH_CHECK();
  YG_CUDA(cudaMemcpyAsync(idx, di, sizeof(int) * n, cudaMemcpyDeviceToHost, st));
  YG_CUDA(cudaStreamSynchronize(st));
  return OK;
}

}  // namespace yg

using namespace yg;

static hkm_t *hkm_alloc(int d, int nlevel, int bf) {
  hkm_t *h = (hkm_t *)malloc(sizeof(hkm_t));
  h->nlevel = nlevel;
  h->bf = bf;
  h->d = d;
  h->centroids = (float **)malloc(sizeof(float *) * nlevel);
  long k = 1;
  for (int l = 0; l < nlevel; l++) {
    h->centroids[l] = (float *)malloc(sizeof(float) * k * bf * d);
    k *= bf;
  }
  h->k = (int)k;
  return h;
}

extern "C" {

int yael_gpu_last_stats(yael_gpu_call_stats *out) {
  if (!out) return YAEL_GPU_EARG;
  *out = g_last_stats;
  return YAEL_GPU_OK;
}

float yael_gpu_kmeans_ex(int d, int n, int k, int niter, const float *v, int flags, long seed,
                         int redo, float *centroids, float *dis, int *assign, int *nassign,
                         yael_gpu_kmeans_opts *opts) {
  int prec = default_precision();
  bool dev = false;
  cudaStream_t st = nullptr;
  if (opts) {
    if (explicit_precision(opts->precision))
      prec = opts->precision;
    dev = opts->device_ptrs != 0;
    st = (cudaStream_t)opts->stream;
  }
  float ret = -1;
  long iters = 0, fb = 0, sec = 0, bd = 0;
  float ma = 0, mu = 0;
  WaitLimitScope wls(opts ? opts->wait_limit_us : 0);
  const int rc = kmeans_run(d, n, k, niter, v, flags, seed, redo, centroids, dis, assign,
                            nassign, prec, dev, st, &ret, &iters, &fb, &sec, &ma, &mu, &bd,
                            opts);
  if (opts) {
    opts->status = rc;
    opts->iterations = iters;
    opts->n_fallback = fb;
    opts->n_second = sec;
    opts->n_band = bd;
    opts->ms_assign = ma;
    opts->ms_update = mu;
  }
  if (rc != OK) return -2.f;
  return ret;
}

float kmeans(int d, int n, int k, int niter, const float *v, int flags, long seed, int redo,
             float *centroids, float *dis, int *assign, int *nassign) {
  float ret = -1;
  if (kmeans_run(d, n, k, niter, v, flags, seed, redo, centroids, dis, assign, nassign,
                 default_precision(), false, nullptr, &ret, nullptr, nullptr, nullptr, nullptr,
                 nullptr) != OK)
    fatal_last("kmeans");
  return ret;
}

float *clustering_kmeans_assign_with_score(int n, int d, const float *points, int k,
                                           int nb_iter_max, double normalize, int n_thread,
                                           double *score_out, int **clust_assign_out) {
  (void)normalize;
  (void)score_out;  // never written by the reference either (yael/kmeans.c:452-482)
  float *centroids = (float *)malloc(sizeof(float) * (size_t)k * d);
  int *ca = clust_assign_out ? (int *)malloc(sizeof(int) * (size_t)n) : nullptr;
  int nredo = 1;
  if (nb_iter_max / 100000 != 0) {
    nredo = nb_iter_max / 100000;
    nb_iter_max = nb_iter_max % 100000;
  }
  const float ret = kmeans(d, n, k, nb_iter_max, points, n_thread | YAEL_KMEANS_INIT_RANDOM, 0,
                           nredo, centroids, nullptr, ca, nullptr);
  if (ret >= 0) {
    if (clust_assign_out) *clust_assign_out = ca;
    return centroids;
  }
  free(centroids);
  free(ca);
  if (clust_assign_out) *clust_assign_out = nullptr;
  return nullptr;
}

float *clustering_kmeans_assign(int n, int d, const float *points, int k, int nb_iter_max,
                                double normalize, int **clust_assign_out) {
  return clustering_kmeans_assign_with_score(n, d, points, k, nb_iter_max, normalize, 1,
                                             nullptr, clust_assign_out);
}

float *clustering_kmeans(int n, int d, const float *points, int k, int nb_iter_max,
                         double normalize) {
  int *ca = nullptr;
  float *c = clustering_kmeans_assign_with_score(n, d, points, k, nb_iter_max, normalize, 1,
                                                 nullptr, &ca);
  free(ca);
  return c;
}

hkm_t *hkm_learn(int n, int d, int nlevel, int bf, const float *v, int nb_iter_max, int nt,
                 int verbose, int **clust_assign_out) {
  (void)nt;  // the reference ignores it too (hkm.c:85)
  hkm_t *h = hkm_alloc(d, nlevel, bf);
  int *assign = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
  if (hkm_run(n, d, nlevel, bf, v, nb_iter_max, verbose != 0, default_precision(), false,
              h->centroids, assign, nullptr, nullptr) != OK)
    fatal_last("hkm_learn");
  if (clust_assign_out) *clust_assign_out = assign;
  else free(assign);
  return h;
}

int yael_gpu_hkm_learn_ex(int n, int d, int nlevel, int bf, const float *v, int nb_iter_max,
                          int small_nodes, float *centroids, int *assign, long *iterations,
                          float *ms) {
  std::vector<float *> lv(nlevel);
  long k = bf, off = 0;
  for (int l = 0; l < nlevel; l++, k *= bf) {
    lv[l] = centroids + off;
    off += k * d;
  }
  return hkm_run(n, d, nlevel, bf, v, nb_iter_max, false, default_precision(), small_nodes != 0,
                 lv.data(), assign, iterations, ms);
}

void hkm_delete(hkm_t *hkm) {
  for (int l = 0; l < hkm->nlevel; l++) free(hkm->centroids[l]);
  free(hkm->centroids);
  free(hkm);
}

void hkm_quantize(const hkm_t *hkm, int npt, const float *v, int *idx) {
  if (hkm_quantize_run(hkm->nlevel, hkm->bf, hkm->d, hkm->centroids, npt, v, idx) != OK)
    fatal_last("hkm_quantize");
}

float *hkm_get_centroids(const hkm_t *hkm, int l, int no) {
  return hkm->centroids[l] + (long)hkm->d * hkm->bf * no;
}

// file format of yael/hkm.c:181-232: int nlevel, bf, d, then per level one
// fvec record (int count, count floats) of bf^(l+1) * d centroids
void hkm_write(const char *filename, const hkm_t *hkm) {
  FILE *f = fopen(filename, "w");
  if (!f) {
    fprintf(stderr, "# Unable to write the hkm file %s\n", filename);
    return;
  }
  if (fwrite(&hkm->nlevel, sizeof(int), 1, f) != 1 || fwrite(&hkm->bf, sizeof(int), 1, f) != 1 ||
      fwrite(&hkm->d, sizeof(int), 1, f) != 1) {
    fprintf(stderr, "# Unable to write the hkm file %s\n", filename);
    fclose(f);
    return;
  }
  long k = hkm->bf;
  for (int l = 0; l < hkm->nlevel; l++, k *= hkm->bf) {
    const int cnt = (int)(k * hkm->d);
    if (fwrite(&cnt, sizeof(int), 1, f) != 1 ||
        fwrite(hkm->centroids[l], sizeof(float), cnt, f) != (size_t)cnt)
      perror("fvec_fwrite: write error");
  }
  fclose(f);
}

hkm_t *hkm_read(const char *filename) {
  FILE *f = fopen(filename, "r");
  int nlevel, bf, d;
  if (!f || fread(&nlevel, sizeof(int), 1, f) != 1 || fread(&bf, sizeof(int), 1, f) != 1 ||
      fread(&d, sizeof(int), 1, f) != 1 || nlevel < 1 || bf < 1 || d < 1) {
    fprintf(stderr, "# Unable to read the hkm file %s\n", filename);
    if (f) fclose(f);
    return nullptr;
  }
  hkm_t *h = hkm_alloc(d, nlevel, bf);
  long k = bf;
  for (int l = 0; l < nlevel; l++, k *= bf) {
    int cnt = 0;
    if (fread(&cnt, sizeof(int), 1, f) != 1 || cnt != k * d ||
        fread(h->centroids[l], sizeof(float), cnt, f) != (size_t)cnt) {
      fprintf(stderr, "# Unable to read the hkm file %s\n", filename);
      hkm_delete(h);
      fclose(f);
      return nullptr;
    }
  }
  fclose(f);
  return h;
}

}  // extern "C"
