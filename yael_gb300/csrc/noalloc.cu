// k-NN entry point that allocates no device memory.
//
// Some callers cannot let a library allocate GPU memory: a serving process
// that hands all of HBM to its own pool allocator at start-up (a cudaMalloc
// from here would fail or fragment that budget), or code on a latency-critical
// path where cudaMalloc / cudaFree synchronise the device.  For them
// yael_gpu_knn_noalloc computes the same exact k-NN as yael_gpu_knn_ex (the
// plain FP32 distance pass, the re-rank with its exactness certificate, the
// exhaustive FP64 fallback) with every scratch buffer carved from one
// file-scope __device__ array of kNoAllocScratchBytes.  The module loader
// reserves that array on each GPU that loads this library, for the life of
// the process.
//
// The array is shared by all calls and keeps the previous call's contents:
// each call clears what must start at zero.  Calls whose GPU work overlaps
// (other host threads, other streams) race on it and must be serialised by
// the caller.
#include "knn.cuh"
#include "../../include/yael_gpu.h"

namespace yg {

namespace {

constexpr size_t kNoAllocScratchBytes = (size_t)32 << 20;  // 32 MiB
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

struct NoAllocSmall {
  SetStats bs;
  int fail_cnt;
  int pad;
  unsigned long long n_cand;
};

// device address of the array on the current device.  The array's name is
// only a host-side stand-in for it; the lookup allocates nothing and is done
// on every call, so a context that was reset and reloaded is never handed a
// stale address.
int scratch_address(unsigned char **out) {
  void *p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || !p) {
    set_error(E_CUDA, "yael_gpu_knn_noalloc: cudaGetSymbolAddress failed: %s",
              cudaGetErrorString(e));
    return E_CUDA;
  }
  *out = static_cast<unsigned char *>(p);
  return OK;
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

int knn_noalloc(int nq, int nb, int d, int k, const float *b, const float *q, int *assign,
                float *dis, cudaStream_t st) {
  if (nq < 0 || nb < 1 || d < 1 || k < 1 || k > nb) {
    set_error(E_ARG, "yael_gpu_knn_noalloc: invalid sizes nq=%d nb=%d d=%d k=%d", nq, nb, d, k);
    return E_ARG;
  }
  if (k > 16) {
    set_error(E_ARG, "yael_gpu_knn_noalloc: k=%d above its maximum of 16", k);
    return E_ARG;
  }
  if (nq == 0) return OK;
  int C = 1;
  while (C < 2 * k) C <<= 1;  // room for the certificate on non-integer data
  const int nqt = (int)ceil_div(nq, 128), ntb = (int)ceil_div(nb, SIMT_TILE_N);
  int num_sms = 0, dev = 0;
  YG_CUDA(cudaGetDevice(&dev));
  YG_CUDA(cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev));
  const size_t fixed = align256(sizeof(NoAllocSmall)) + align256((size_t)nb * 4) +
                       align256((size_t)nq * 8) + 2 * align256((size_t)nq) +
                       align256((size_t)nq * 4) + align256((size_t)nq * 4) +
                       align256(exhaustive_bytes_per_query(nb));
  auto lists = [&](int nch) { return 2 * align256((size_t)nch * nq * C * 4); };
  if (fixed + lists(1) > kNoAllocScratchBytes) {
    set_error(E_ARG,
              "yael_gpu_knn_noalloc: nq=%d nb=%d k=%d needs %zu bytes of scratch, the static "
              "scratch holds %zu; use yael_gpu_knn_ex",
              nq, nb, k, fixed + lists(1), kNoAllocScratchBytes);
    return E_ARG;
  }
  int nchunk = imin(choose_chunks(nqt, ntb, num_sms, 1, 4), kMaxCandidates / C);
  while (nchunk > 1 && fixed + lists(nchunk) > kNoAllocScratchBytes) nchunk--;
  const int tpc = (int)ceil_div(ntb, nchunk);
  nchunk = (int)ceil_div(ntb, tpc);

  unsigned char *base;
  YG_CHECK(scratch_address(&base));
  size_t off = 0;
  auto take = [&](size_t bytes) {
    unsigned char *p = base + off;
    off += align256(bytes);
    return p;
  };
  NoAllocSmall *small = reinterpret_cast<NoAllocSmall *>(take(sizeof(NoAllocSmall)));
  float *bn32 = reinterpret_cast<float *>(take((size_t)nb * 4));
  double *qn64 = reinterpret_cast<double *>(take((size_t)nq * 8));
  unsigned char *qflag = take((size_t)nq);
  unsigned char *qexact = take((size_t)nq);
  float *eps = reinterpret_cast<float *>(take((size_t)nq * 4));
  int *fail_list = reinterpret_cast<int *>(take((size_t)nq * 4));
  ScanSel sel;
  sel.mode = SCAN_TOPC;
  sel.C = C;
  sel.nchunk = nchunk;
  sel.tiles_per_chunk = tpc;
  sel.topv = reinterpret_cast<float *>(take((size_t)nchunk * nq * C * 4));
  sel.topi = reinterpret_cast<int *>(take((size_t)nchunk * nq * C * 4));
  // the exhaustive fallback gets the rest of the array (at least one query's
  // worth, by the size check above), so rejected queries are batched
  void *rows = base + off;
  const size_t rows_bytes = kNoAllocScratchBytes - off;

  // once work is queued, every return waits for it: the next call reuses the
  // array and must not race with kernels of this one
  auto queued = [&]() -> int {
    // everything that must start at zero: the statistics and counters
    NoAllocSmall h{};
    h.bs.all_exact = 1;
    YG_CUDA(cudaMemcpyAsync(small, &h, sizeof(h), cudaMemcpyHostToDevice, st));
    YG_CHECK(prep_rows(b, d, nb, d, 1.f, nullptr, bn32, nullptr, nullptr, nullptr, 0, nullptr, 0,
                       &small->bs, st));
    YG_CHECK(prep_rows(q, d, nq, d, 1.f, qn64, nullptr, qflag, nullptr, nullptr, 0, nullptr, 0,
                       nullptr, st));
    YG_CHECK(compute_eps(nq, d, PREC_FP32, METRIC_L2, qn64, nullptr, qflag, &small->bs, eps,
                         qexact, st));
    YG_CHECK(simt_scan(q, d, nq, b, d, nb, d, bn32, 1, METRIC_L2, sel, st));
    RerankArgs ra;
    ra.nq = nq; ra.nb = nb; ra.d = d; ra.k = k; ra.metric = METRIC_L2;
    ra.q = q; ra.ldq = d; ra.b = b; ra.ldb = d;
    ra.qn64 = qn64; ra.eps = eps; ra.qexact = qexact; ra.bstats = &small->bs;
    ra.sel = sel;
    ra.out_idx = assign; ra.out_dis = dis;
    ra.fail_list = fail_list; ra.fail_cnt = &small->fail_cnt; ra.n_cand = &small->n_cand;
    YG_CHECK(rerank(ra, st));
    int nfail = 0;
    YG_CUDA(cudaMemcpyAsync(&nfail, &small->fail_cnt, sizeof(int), cudaMemcpyDeviceToHost, st));
    YG_CUDA(cudaStreamSynchronize(st));
    if (nfail > 0)
      YG_CHECK(exhaustive(nfail, fail_list, nb, d, k, METRIC_L2, q, d, b, d, nullptr, assign, dis,
                          rows, rows_bytes, st));
    YG_CUDA(cudaStreamSynchronize(st));
    return OK;
  };
  const int rc = queued();
  if (rc != OK) (void)cudaStreamSynchronize(st);
  return rc;
}

}  // namespace

}  // namespace yg

extern "C" int yael_gpu_knn_noalloc(int nq, int nb, int d, int k, const float *b,
                                    const float *q, int *assign, float *dis, void *stream) {
  return yg::knn_noalloc(nq, nb, d, k, b, q, assign, dis, (cudaStream_t)stream);
}
