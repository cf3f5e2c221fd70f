// Shared definitions for the GB300 (sm_103a) implementation of yael's
// distance-GEMM path: error handling, the per-thread stream, the grow-only
// workspace, small device helpers.
#pragma once

#include <nvtx3/nvToolsExt.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include <cstddef>
#include <string>
#include <vector>

namespace yg {

// ---------------------------------------------------------------------------
// errors.  yael signals failure by assert()/abort() (nn.c:456, vector.c:34-41);
// the drop-in entry points keep that convention (message on stderr, abort),
// the *_ex entry points return a status and leave the message for
// yael_gpu_last_error().
enum Status : int {
  OK = 0,
  E_CUDA = 1,
  E_ARG = 2,
  E_UNSUPPORTED = 3,
  E_NOMEM = 4,
  E_TIMEOUT = 5,
};

void set_error(int code, const char *fmt, ...);
int last_code();
const char *last_message();
[[noreturn]] void fatal_last(const char *where);

#define YG_CUDA(call)                                                      \
  do {                                                                     \
    cudaError_t _e = (call);                                               \
    if (_e != cudaSuccess) {                                               \
      ::yg::set_error(::yg::E_CUDA, "%s:%d %s: %s", __FILE__, __LINE__,    \
                      #call, cudaGetErrorString(_e));                      \
      return ::yg::E_CUDA;                                                 \
    }                                                                      \
  } while (0)

#define YG_CHECK(expr)                 \
  do {                                 \
    int _s = (expr);                   \
    if (_s != ::yg::OK) return _s;     \
  } while (0)

void count_launch();
void count_launches(long n);  // kernels replayed by a CUDA graph launch
long launch_count();
#define YG_LAUNCH_CHECK()          \
  do {                             \
    ::yg::count_launch();          \
    YG_CUDA(cudaGetLastError());   \
  } while (0)

// ---------------------------------------------------------------------------
// execution context: one device per process (the current device at first
// use), one non-blocking stream per calling host thread, one grow-only device
// workspace per host thread.  Callers may run concurrently from several host
// threads (the reference is reentrant, yael.swg:140-144).
struct Workspace {
  struct Buf {
    void *p = nullptr;
    size_t n = 0;
  };
  std::vector<Buf> bufs;
  bool host = false;  // pinned host memory (cudaMallocHost) instead of device memory
  // slot-addressed scratch: the same slot is reused by every call.
  int get(int slot, size_t bytes, void **out);
  void release_all();
  ~Workspace();
};

struct Ctx {
  int device = 0;
  int num_sms = 0;
  int cc_major = 0, cc_minor = 0;
  size_t smem_optin = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t copy_stream = nullptr;  // host uploads overlapped with passes (lazy)
  Workspace ws;
  Workspace pinned;  // grow-only pinned host buffers (host = true), by slot
  void *pinned_status = nullptr;  // kPinnedStatusBytes of pinned host memory (lazy)
};

constexpr size_t kPinnedStatusBytes = 4096;
// the context's pinned status buffer: small device -> host reads stay async
int ctx_pinned_status(Ctx *c, void **out);

// pinned slots 3 and 4: the staging pieces of copy_to_host
constexpr int kPinnedStageSlot = 3;
// Device -> host copy into caller memory, complete on return (the stream is
// synchronised): pinned or registered memory directly, pageable memory
// through two 4 MB pinned pieces of the context (the copy of one piece runs
// while the host copies the previous one out), several times faster than the
// driver's own staging of a pageable destination.
int copy_to_host(Ctx *c, cudaStream_t st, void *dst, const void *src, size_t bytes);

// returns the calling thread's context (created on first use)
int ctx_get(Ctx **out);

// precision of the distance pass
// PREC_BF16X3: the tensor cores on a 3xBF16 split of the operands
// (x = hi + lo), about 2^-16 relative error instead of 2^-8
// PREC_FP16: the tensor cores on fp16 operands (2^-11 relative rounding at the
// bf16 rate), for data fp16 can hold (|x| < 16384, ||x||^2 < 2^15 for base
// rows); rows it cannot hold get an infinite error bound and are settled by
// the later passes
// s + t * t and s + a * b with the product rounded before the sum, as C
// without floating-point contraction computes them (the oracle is built with
// -ffp-contract=off): FP64 distances agree with it bit for bit on any host
__device__ __forceinline__ double add_sq64(double s, double t) {
  return __dadd_rn(s, __dmul_rn(t, t));
}
__device__ __forceinline__ double add_mul64(double s, double a, double b) {
  return __dadd_rn(s, __dmul_rn(a, b));
}

enum Precision : int { PREC_FP32 = 0, PREC_BF16 = 1, PREC_BF16X3 = 2, PREC_FP16 = 3 };
int default_precision();  // from YAEL_GPU_PRECISION (fp32 | bf16 | bf16x3 | fp16), default fp32
// p is one of the YAEL_GPU_PREC_* values a caller may pass explicitly
inline bool explicit_precision(int p) { return p >= PREC_FP32 && p <= PREC_FP16; }
// Bound of the waits inside the tensor-core kernels launched by the calling
// thread, in ns (0: the kernels' own 2 s); set for the duration of a call by
// WaitLimitScope from a caller's wait_limit_us option.
unsigned long long wait_limit_ns();
struct WaitLimitScope {
  unsigned long long saved;
  explicit WaitLimitScope(int limit_us);
  ~WaitLimitScope();
};
// YAEL_GPU_TEST_WITHHOLD_LOADS=1 (read at every launch): the tensor-core
// kernels' producers issue no load, so the consumers' bounded waits expire
// and the call returns YAEL_GPU_ETIMEOUT with the context still usable.  A
// test hook for that path; nothing is faulted and nothing hangs.
bool test_withhold_loads();
// YAEL_GPU_TEST_FAIL_ALLOC=n: the n-th workspace growth after the variable
// was set fails as an out-of-memory cudaMalloc (host-side test hook)
bool test_fail_alloc();
// YAEL_GPU_TRACE set (and not "0"): every k-NN pass is timed with CUDA events
// and reported on stderr, one line per pass
bool trace_enabled();

// An NVTX range over a host scope: the phases of the pipeline (packing,
// distance pass, re-rank, later passes, update, split) appear by name on a
// profiler's timeline; without a tool attached a push / pop costs nothing.
struct NvtxRange {
  explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange &) = delete;
  NvtxRange &operator=(const NvtxRange &) = delete;
};

// A device array owned by the host scope that holds it (freed on
// destruction).  get() grows it to at least `want` elements, dropping the
// contents; an allocation failure records E_NOMEM and aborts through
// fatal_last(where), the convention of the drop-in entry points.
template <typename T>
struct DevArray {
  T *p = nullptr;
  long n = 0;
  DevArray() = default;
  DevArray(const DevArray &) = delete;
  DevArray &operator=(const DevArray &) = delete;
  ~DevArray() {
    if (p) cudaFree(p);
  }
  T *get(const char *where, long want) {
    if (want > n) {
      if (p) cudaFree(p);
      p = nullptr;
      n = 0;
      const size_t bytes = sizeof(T) * (size_t)(want > 1 ? want : 1);
      const cudaError_t e = cudaMalloc((void **)&p, bytes);
      if (e != cudaSuccess) {
        p = nullptr;
        set_error(E_NOMEM, "cudaMalloc of %zu bytes: %s", bytes, cudaGetErrorString(e));
        fatal_last(where);
      }
      n = want;
    }
    return p;
  }
};

// Raises kernel func's dynamic shared-memory limit to at least bytes on the
// current device, once per (kernel, device, size); thread safe.
int ensure_smem(const void *func, size_t bytes);

// ---------------------------------------------------------------------------
// device helpers
__host__ __device__ inline long long ceil_div(long long a, long long b) { return (a + b - 1) / b; }
__host__ __device__ inline int imin(int a, int b) { return a < b ? a : b; }
__host__ __device__ inline int imax(int a, int b) { return a > b ? a : b; }

// order-preserving map float -> uint32 (NaN sorts above +inf for +NaN)
__device__ __forceinline__ uint32_t f2ord(float f) {
  uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord2f(uint32_t u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}
__device__ __forceinline__ unsigned long long d2ord(double f) {
  unsigned long long u = __double_as_longlong(f);
  return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
}

}  // namespace yg
