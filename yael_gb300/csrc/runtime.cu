// Runtime pieces: per-thread error state, per-thread stream and workspace,
// configuration from the environment.
#include <stdarg.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <map>
#include <mutex>
#include <string>
#include <utility>

#include "common.cuh"
#include "../../include/yael_gpu.h"

namespace yg {

static std::atomic<long> g_launches{0};
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
void count_launches(long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
long launch_count() { return g_launches.load(); }

static thread_local int t_code = OK;
static thread_local char t_msg[1024] = "";

void set_error(int code, const char *fmt, ...) {
  t_code = code;
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(t_msg, sizeof(t_msg), fmt, ap);
  va_end(ap);
}
int last_code() { return t_code; }
const char *last_message() { return t_msg; }

void fatal_last(const char *where) {
  fprintf(stderr, "yael_gb300: %s failed: %s\n", where, t_msg[0] ? t_msg : "(no message)");
  fflush(stderr);
  abort();
}

int Workspace::get(int slot, size_t bytes, void **out) {
  if (slot >= (int)bufs.size()) bufs.resize(slot + 1);
  Buf &b = bufs[slot];
  if (bytes == 0) bytes = 256;
  if (b.n < bytes) {
    if (b.p) {
      cudaError_t e = host ? cudaFreeHost(b.p) : cudaFree(b.p);
      b.p = nullptr;
      b.n = 0;
      if (e != cudaSuccess) {
        set_error(E_CUDA, "cudaFree: %s", cudaGetErrorString(e));
        return E_CUDA;
      }
    }
    size_t n = bytes + bytes / 8;  // headroom so slowly growing sizes do not thrash
    n = (n + 255) & ~(size_t)255;
    cudaError_t e = test_fail_alloc() ? cudaErrorMemoryAllocation
                    : host            ? cudaMallocHost(&b.p, n)
                                      : cudaMalloc(&b.p, n);
    if (e != cudaSuccess) {
      (void)cudaGetLastError();
      b.p = nullptr;
      set_error(E_NOMEM, "%s(%zu bytes, workspace slot %d): %s",
                host ? "cudaMallocHost" : "cudaMalloc", n, slot, cudaGetErrorString(e));
      return E_NOMEM;
    }
    b.n = n;
  }
  *out = b.p;
  return OK;
}

void Workspace::release_all() {
  for (auto &b : bufs)
    if (b.p) {
      if (host) cudaFreeHost(b.p);
      else cudaFree(b.p);
    }
  bufs.clear();
}

Workspace::~Workspace() { release_all(); }

static thread_local Ctx *t_ctx = nullptr;

int ctx_get(Ctx **out) {
  if (t_ctx) {
    *out = t_ctx;
    return OK;
  }
  Ctx *c = new Ctx();
  cudaError_t e = cudaGetDevice(&c->device);
  if (e != cudaSuccess) {
    delete c;
    set_error(E_CUDA, "no CUDA device: %s", cudaGetErrorString(e));
    return E_CUDA;
  }
  cudaDeviceProp p;
  e = cudaGetDeviceProperties(&p, c->device);
  if (e != cudaSuccess) {
    delete c;
    set_error(E_CUDA, "cudaGetDeviceProperties: %s", cudaGetErrorString(e));
    return E_CUDA;
  }
  c->num_sms = p.multiProcessorCount;
  c->cc_major = p.major;
  c->cc_minor = p.minor;
  c->smem_optin = p.sharedMemPerBlockOptin;
  c->pinned.host = true;
  e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete c;
    set_error(E_CUDA, "cudaStreamCreate: %s", cudaGetErrorString(e));
    return E_CUDA;
  }
  t_ctx = c;
  *out = c;
  return OK;
}

int ctx_pinned_status(Ctx *c, void **out) {
  if (!c->pinned_status) {
    cudaError_t e = cudaMallocHost(&c->pinned_status, kPinnedStatusBytes);
    if (e != cudaSuccess) {
      (void)cudaGetLastError();
      c->pinned_status = nullptr;
      set_error(E_NOMEM, "cudaMallocHost(%zu): %s", kPinnedStatusBytes, cudaGetErrorString(e));
      return E_NOMEM;
    }
  }
  *out = c->pinned_status;
  return OK;
}

int copy_to_host(Ctx *c, cudaStream_t st, void *dst, const void *src, size_t bytes) {
  if (!dst || bytes == 0) return OK;
  cudaPointerAttributes at;
  const cudaError_t ea = cudaPointerGetAttributes(&at, dst);
  if (ea != cudaSuccess) (void)cudaGetLastError();
  if (ea == cudaSuccess && at.type != cudaMemoryTypeUnregistered) {
    YG_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, st));
    YG_CUDA(cudaStreamSynchronize(st));
    return OK;
  }
  constexpr size_t kPiece = (size_t)4 << 20;
  void *stage[2];
  for (int i = 0; i < 2; i++)
    YG_CHECK(c->pinned.get(kPinnedStageSlot + i, std::min(bytes, kPiece), &stage[i]));
  cudaEvent_t ev[2];
  for (int i = 0; i < 2; i++) YG_CUDA(cudaEventCreateWithFlags(&ev[i], cudaEventDisableTiming));
  int rc = OK;
  size_t prev_off = 0, prev_len = 0;
  int i = 0;
  for (size_t off = 0; off < bytes && rc == OK; off += kPiece, i++) {
    const size_t len = std::min(kPiece, bytes - off);
    cudaError_t e = cudaMemcpyAsync(stage[i & 1], static_cast<const char *>(src) + off, len,
                                    cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaEventRecord(ev[i & 1], st);
    if (e == cudaSuccess && i > 0) e = cudaEventSynchronize(ev[(i - 1) & 1]);
    if (e != cudaSuccess) {
      set_error(E_CUDA, "copy_to_host: %s", cudaGetErrorString(e));
      rc = E_CUDA;
      break;
    }
    if (i > 0) memcpy(static_cast<char *>(dst) + prev_off, stage[(i - 1) & 1], prev_len);
    prev_off = off;
    prev_len = len;
  }
  if (rc == OK && prev_len) {
    const cudaError_t e = cudaEventSynchronize(ev[(i - 1) & 1]);
    if (e != cudaSuccess) {
      set_error(E_CUDA, "copy_to_host: %s", cudaGetErrorString(e));
      rc = E_CUDA;
    } else {
      memcpy(static_cast<char *>(dst) + prev_off, stage[(i - 1) & 1], prev_len);
    }
  }
  if (rc != OK) (void)cudaStreamSynchronize(st);  // nothing in flight into the stage
  for (int j = 0; j < 2; j++) cudaEventDestroy(ev[j]);
  return rc;
}

int default_precision() {
  const char *s = getenv("YAEL_GPU_PRECISION");
  if (!s || !*s) return PREC_FP32;
  if (!strcmp(s, "bf16") || !strcmp(s, "BF16") || !strcmp(s, "1")) return PREC_BF16;
  if (!strcmp(s, "bf16x3") || !strcmp(s, "BF16X3") || !strcmp(s, "2")) return PREC_BF16X3;
  if (!strcmp(s, "fp16") || !strcmp(s, "FP16") || !strcmp(s, "3")) return PREC_FP16;
  return PREC_FP32;
}

int ensure_smem(const void *func, size_t bytes) {
  static std::mutex m;
  static std::map<std::pair<const void *, int>, size_t> done;
  int dev = 0;
  YG_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> g(m);
  size_t &cur = done[std::make_pair(func, dev)];
  if (bytes <= cur || bytes <= 48 * 1024) return OK;
  YG_CUDA(cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  cur = bytes;
  return OK;
}

// YAEL_GPU_TEST_FAIL_ALLOC=n (n >= 1, read at every workspace growth): the
// n-th growth of the calling thread counted from the moment the variable
// changed value fails as an out-of-memory cudaMalloc would (the call is not
// made).  A host-side test hook for the E_NOMEM path.
static thread_local long t_fail_seen = 0;
static thread_local std::string t_fail_env;
bool test_fail_alloc() {
  const char *s = getenv("YAEL_GPU_TEST_FAIL_ALLOC");
  const std::string cur = s ? s : "";
  if (cur != t_fail_env) {
    t_fail_env = cur;
    t_fail_seen = 0;
  }
  const long n = cur.empty() ? 0 : atol(cur.c_str());
  if (n <= 0) return false;
  return ++t_fail_seen == n;
}

static thread_local unsigned long long t_wait_ns = 0;
unsigned long long wait_limit_ns() { return t_wait_ns; }
WaitLimitScope::WaitLimitScope(int limit_us) : saved(t_wait_ns) {
  if (limit_us > 0) t_wait_ns = (unsigned long long)limit_us * 1000ull;
}
WaitLimitScope::~WaitLimitScope() { t_wait_ns = saved; }

bool test_withhold_loads() {
  const char *s = getenv("YAEL_GPU_TEST_WITHHOLD_LOADS");
  return s && s[0] == '1';
}

bool trace_enabled() {
  static const bool on = [] {
    const char *s = getenv("YAEL_GPU_TRACE");
    return s && *s && strcmp(s, "0") != 0;
  }();
  return on;
}

}  // namespace yg

extern "C" const char *yael_gpu_last_error(void) { return yg::last_message(); }

extern "C" int yael_gpu_version(void) { return YAEL_GPU_ABI_VERSION; }

extern "C" long yael_gpu_launch_count(void) { return yg::launch_count(); }
