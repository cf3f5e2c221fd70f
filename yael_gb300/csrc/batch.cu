// Batched exact k-NN over many independent (queries, base) pairs of uneven
// sizes (yael_gpu_knn_batch).  Device arrays with the BF16 pass and k >= 9 go
// through the grouped pipeline (group.cu: one launch per pass over all the
// pairs).  Otherwise the pairs run concurrently on a persistent pool of host
// workers; each worker owns a context (stream + grow-only workspace,
// runtime.cu) that lives as long as the process, so repeated batches reuse
// their buffers.  Pairs are handed out largest first (nq * nb) from an atomic
// cursor, which balances the uneven sizes; the calling thread works too.
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "autotune.cuh"
#include "knn.cuh"

namespace yg {
namespace {

struct BatchTask {
  const yael_gpu_knn_pair *pairs = nullptr;
  std::vector<int> order;  // pair indices, largest first
  int d = 0, k = 0, metric = METRIC_L2, prec = PREC_FP32, device_ptrs = 0, device = 0;
  std::atomic<int> next{0};
  std::atomic<long long> n_fallback{0}, n_band{0}, n_second{0}, n_cand{0};
  std::atomic<int> all_exact{1};
  std::mutex m;
  int err = OK;
  std::string msg;
};

void run_pairs(BatchTask *t) {
  tune_set_thread_enabled(false);  // concurrent pairs: timings not comparable
  if (cudaSetDevice(t->device) != cudaSuccess) {
    std::lock_guard<std::mutex> g(t->m);
    if (t->err == OK) { t->err = E_CUDA; t->msg = "cudaSetDevice failed in a batch worker"; }
    return;
  }
  for (;;) {
    const int i = t->next.fetch_add(1);
    if (i >= (int)t->order.size()) break;
    {
      std::lock_guard<std::mutex> g(t->m);
      if (t->err != OK) break;  // stop at the first error
    }
    const yael_gpu_knn_pair &p = t->pairs[t->order[i]];
    yael_gpu_knn_opts o;
    memset(&o, 0, sizeof(o));
    o.device_ptrs = t->device_ptrs;  // o.stream = NULL: this worker's stream
    const int rc = knn_host(t->metric, p.nq, p.nb, t->d, t->k, p.b, p.q, nullptr, p.assign,
                            p.dis, t->prec, &o);
    if (rc != OK) {
      std::lock_guard<std::mutex> g(t->m);
      if (t->err == OK) {
        t->err = rc;
        t->msg = std::string("pair ") + std::to_string(t->order[i]) + ": " + last_message();
      }
      break;
    }
    t->n_fallback += o.n_fallback;
    t->n_band += o.n_band;
    t->n_second += o.n_second;
    t->n_cand += o.n_candidates;
    if (!o.exact_class) t->all_exact = 0;
  }
}

// Persistent workers (never joined: they live for the process, like the
// per-thread contexts they own).
class Pool {
 public:
  static Pool &get() {
    static Pool *p = new Pool();
    return *p;
  }

  void run(BatchTask *t, int nworkers) {
    std::lock_guard<std::mutex> one_batch_at_a_time(run_m_);
    {
      std::unique_lock<std::mutex> lk(m_);
      while ((int)threads_.size() < nworkers - 1) {
        const int id = (int)threads_.size();
        threads_.emplace_back([this, id] { worker(id); });
        threads_.back().detach();
      }
      task_ = t;
      want_ = nworkers - 1;
      pending_ = want_;
      gen_++;
    }
    cv_.notify_all();
    run_pairs(t);  // the caller is one of the workers
    std::unique_lock<std::mutex> lk(m_);
    done_cv_.wait(lk, [&] { return pending_ == 0; });
    task_ = nullptr;
  }

 private:
  void worker(int id) {
    long seen = 0;
    std::unique_lock<std::mutex> lk(m_);
    for (;;) {
      cv_.wait(lk, [&] { return gen_ != seen; });
      seen = gen_;
      if (id >= want_) continue;
      BatchTask *t = task_;
      lk.unlock();
      run_pairs(t);
      lk.lock();
      if (--pending_ == 0) done_cv_.notify_all();
    }
  }

  std::mutex run_m_, m_;
  std::condition_variable cv_, done_cv_;
  std::vector<std::thread> threads_;
  BatchTask *task_ = nullptr;
  long gen_ = 0;
  int want_ = 0, pending_ = 0;
};

int workers_default() {
  const char *e = getenv("YAEL_GPU_BATCH_WORKERS");
  const int n = e ? atoi(e) : 0;
  return n > 0 ? (n > 64 ? 64 : n) : 8;
}

}  // namespace
}  // namespace yg

using namespace yg;

extern "C" int yael_gpu_knn_batch(int npairs, const yael_gpu_knn_pair *pairs, int d, int k,
                                  yael_gpu_knn_opts *opts) {
  if (npairs < 0 || (npairs > 0 && !pairs) || d < 1 || k < 1) {
    set_error(E_ARG, "knn_batch: invalid arguments npairs=%d d=%d k=%d", npairs, d, k);
    return E_ARG;
  }
  BatchTask t;
  t.pairs = pairs;
  t.d = d;
  t.k = k;
  t.prec = default_precision();
  if (opts) {
    if (explicit_precision(opts->precision))
      t.prec = opts->precision;
    if (opts->metric == 16) t.metric = METRIC_DOT;
    else if (opts->metric && opts->metric != 2 && opts->metric != 12) {
      set_error(E_UNSUPPORTED, "knn_batch: distance_type %d not supported", opts->metric);
      return E_UNSUPPORTED;
    }
    t.device_ptrs = opts->device_ptrs;
  }
  for (int i = 0; i < npairs; i++) {
    if (pairs[i].nq < 0 || pairs[i].nb < k) {
      set_error(E_ARG, "knn_batch: pair %d has nq=%d nb=%d (need nq >= 0, nb >= k=%d)", i,
                pairs[i].nq, pairs[i].nb, k);
      return E_ARG;
    }
  }
  if (cudaGetDevice(&t.device) != cudaSuccess) {
    set_error(E_CUDA, "knn_batch: no CUDA device");
    return E_CUDA;
  }
  if (t.device_ptrs) {
    // the inputs were produced on the caller's stream
    const cudaError_t e = cudaStreamSynchronize(opts ? (cudaStream_t)opts->stream : nullptr);
    if (e != cudaSuccess) {
      set_error(E_CUDA, "knn_batch: cudaStreamSynchronize: %s", cudaGetErrorString(e));
      return E_CUDA;
    }
  }
  if (npairs > 0 && knn_grouped_eligible(d, k, t.prec, t.device_ptrs)) {
    Ctx *ctx;
    YG_CHECK(ctx_get(&ctx));
    GroupCounters gc;
    const int rc = knn_grouped(npairs, pairs, d, k, t.metric, ctx->stream, &gc);
    if (rc == OK) {
      if (opts) {
        opts->n_fallback = (int)std::min<long long>(gc.n_fallback, 0x7fffffff);
        opts->n_band = (int)std::min<long long>(gc.n_band, 0x7fffffff);
        opts->n_second = (int)std::min<long long>(gc.n_second, 0x7fffffff);
        opts->n_candidates = (int)std::min<long long>(gc.n_cand, 0x7fffffff);
        opts->exact_class = gc.all_exact;
      }
      return OK;
    }
    if (rc != E_NOMEM) return rc;  // out of memory: the per-pair pool below
    (void)cudaGetLastError();
  }
  t.order.resize(npairs);
  for (int i = 0; i < npairs; i++) t.order[i] = i;
  std::stable_sort(t.order.begin(), t.order.end(), [&](int a, int b) {
    return (double)pairs[a].nq * pairs[a].nb > (double)pairs[b].nq * pairs[b].nb;
  });
  const int nw = std::max(1, std::min(workers_default(), npairs));
  if (npairs > 0) Pool::get().run(&t, nw);
  if (opts) {
    opts->n_fallback = (int)std::min<long long>(t.n_fallback.load(), 0x7fffffff);
    opts->n_band = (int)std::min<long long>(t.n_band.load(), 0x7fffffff);
    opts->n_second = (int)std::min<long long>(t.n_second.load(), 0x7fffffff);
    opts->n_candidates = (int)std::min<long long>(t.n_cand.load(), 0x7fffffff);
    opts->exact_class = t.all_exact.load();
  }
  if (t.err != OK) {
    set_error(t.err, "knn_batch: %s", t.msg.c_str());
    return t.err;
  }
  return OK;
}
