// Device kernels of the k-means Lloyd step (see kmeans.cuh).
#include <math.h>

#include "kmeans.cuh"

namespace yg {

namespace {

constexpr float kU = 5.9604645e-08f;  // 2^-24

template <int K>
__global__ void __launch_bounds__(256)
    assign_small_kernel(const KmWork *__restrict__ work, const float *__restrict__ v, int d,
                        const float *__restrict__ C, int k, const unsigned char *active,
                        int *assign, float *dis) {
  extern __shared__ float cs[];  // the instance's k x d centroids
  const KmWork w = work[blockIdx.x];
  if (!active[w.inst]) return;
  const float *Ci = C + (long)w.inst * k * d;
  for (int i = threadIdx.x; i < k * d; i += blockDim.x) cs[i] = Ci[i];
  __syncthreads();
  const float rho = (float)(d + 4) * kU;
  for (int pi = threadIdx.x; pi < w.n; pi += blockDim.x) {
    const long p = w.p0 + pi;
    const float *x = v + p * d;
    float acc[K];
#pragma unroll
    for (int j = 0; j < K; j++) acc[j] = 0.f;
    for (int c = 0; c < d; c++) {
      const float xv = __ldg(x + c);
#pragma unroll
      for (int j = 0; j < K; j++) {
        if (j < k) {
          const float t = xv - cs[j * d + c];
          acc[j] = fmaf(t, t, acc[j]);
        }
      }
    }
    // strict '<' from 1e30 over increasing j (yael/nn.c:404-435)
    float b1 = 1e30f, b2 = 1e30f;
    int i1 = -1;
#pragma unroll
    for (int j = 0; j < K; j++) {
      if (j < k) {
        const float a = acc[j];
        if (a < b1) {
          b2 = b1;
          b1 = a;
          i1 = j;
        } else if (a < b2) {
          b2 = a;
        }
      }
    }
    float out = b1;
    if (i1 >= 0 && b2 < 1e30f && b2 - b1 <= rho * (b1 + b2)) {
      // near tie: FP64, sequential over coordinates, lowest index on equality
      double best = INFINITY;
      int bi = -1;
      for (int j = 0; j < k; j++) {
        double s = 0;
        for (int c = 0; c < d; c++) {
          const double t = (double)x[c] - (double)cs[j * d + c];
          s += t * t;
        }
        if (s < best) {
          best = s;
          bi = j;
        }
      }
      i1 = bi;
      out = (float)best;
    }
    assign[p] = i1;
    dis[p] = out;
  }
}

__global__ void hist_kernel(const int *assign, const int *pinst, long n, int k,
                            const unsigned char *active, int *counts) {
  const long p = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const int inst = pinst ? pinst[p] : 0;
  const int a = assign[p];
  if (a < 0 || !active[inst]) return;
  const long g = (long)inst * k + a;
  const unsigned peers = __match_any_sync(__activemask(), g);
  const int leader = __ffs(peers) - 1;
  if ((threadIdx.x & 31) == leader) atomicAdd(counts + g, __popc(peers));
}

__global__ void scan_kernel(const int *counts, long ncl, long *offs, long *cursor) {
  // offs has ncl + 1 entries: offs[ncl] = total
  // one block: contiguous chunks per thread, then a scan of the chunk sums
  __shared__ long part[1024];
  const int t = threadIdx.x, nt = blockDim.x;
  const long per = (ncl + nt - 1) / nt;
  const long a = (long)t * per, b = a + per < ncl ? a + per : ncl;
  long s = 0;
  for (long i = a; i < b; i++) s += counts[i];
  part[t] = s;
  __syncthreads();
  if (t == 0) {
    long run = 0;
    for (int i = 0; i < nt; i++) {
      const long x = part[i];
      part[i] = run;
      run += x;
    }
  }
  __syncthreads();
  long run = part[t];
  for (long i = a; i < b; i++) {
    offs[i] = run;
    cursor[i] = run;
    run += counts[i];
  }
  if (t == nt - 1) offs[ncl] = part[nt - 1] + s;
}

__global__ void scatter_kernel(const int *assign, const int *pinst, long n, int k,
                               const unsigned char *active, long *cursor, long *perm) {
  const long p = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const int inst = pinst ? pinst[p] : 0;
  const int a = assign[p];
  if (a < 0 || !active[inst]) return;
  const long g = (long)inst * k + a;
  const unsigned peers = __match_any_sync(__activemask(), g);
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(peers) - 1;
  long base = 0;
  if (lane == leader) base = atomicAdd((unsigned long long *)(cursor + g),
                                       (unsigned long long)__popc(peers));
  base = __shfl_sync(peers, base, leader);
  perm[base + __popc(peers & ((1u << lane) - 1))] = p;
}

// warps walk contiguous runs of the cluster-sorted point list, accumulating
// exact integer sums in registers and flushing at cluster boundaries
template <int NDR>
__global__ void __launch_bounds__(256)
    segsum_kernel(const long *perm, const long *total, const int *assign, const int *pinst,
                  const float *__restrict__ v, int d, int k, const int *shift,
                  long long *acc) {
  constexpr int RUN = 32;
  const int lane = threadIdx.x & 31;
  const long wglob = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long nsorted = *total;
  const long s0 = wglob * RUN;
  if (s0 >= nsorted) return;
  const long s1 = s0 + RUN < nsorted ? s0 + RUN : nsorted;
  const int dbase = blockIdx.y * NDR * 32;
  long long part[NDR];
#pragma unroll
  for (int r = 0; r < NDR; r++) part[r] = 0;
  long gcur = -1;
  for (long s = s0; s < s1; s++) {
    const long p = perm[s];
    const int inst = pinst ? pinst[p] : 0;
    const long g = (long)inst * k + assign[p];
    if (g != gcur) {
      if (gcur >= 0) {
#pragma unroll
        for (int r = 0; r < NDR; r++) {
          const int c = dbase + r * 32 + lane;
          if (c < d && part[r])
            atomicAdd((unsigned long long *)(acc + gcur * d + c), (unsigned long long)part[r]);
          part[r] = 0;
        }
      }
      gcur = g;
    }
    const double sc = ldexp(1.0, shift[inst]);
#pragma unroll
    for (int r = 0; r < NDR; r++) {
      const int c = dbase + r * 32 + lane;
      if (c < d) part[r] += __double2ll_rn((double)__ldg(v + p * d + c) * sc);
    }
  }
  if (gcur >= 0) {
#pragma unroll
    for (int r = 0; r < NDR; r++) {
      const int c = dbase + r * 32 + lane;
      if (c < d && part[r])
        atomicAdd((unsigned long long *)(acc + gcur * d + c), (unsigned long long)part[r]);
    }
  }
}

__global__ void finalize_kernel(const long long *acc, const int *counts, long ncl, int d,
                                int k, const int *shift, const unsigned char *active,
                                float *C) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ncl * d) return;
  const long g = i / d;
  const int inst = (int)(g / k);
  if (!active[inst]) return;
  const double inv = ldexp(1.0, -shift[inst]);
  const double r = 1.0 / (double)counts[g];
  C[i] = __double2float_rn(__ll2double_rn(acc[i]) * inv * r);
}

__global__ void normalize_kernel(float *C, long ncl, int d, int k, const unsigned char *active) {
  const long g = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= ncl || !active[g / k]) return;
  float *row = C + g * d;
  double s = 0;
  for (int c = 0; c < d; c++) s += (double)(row[c] * row[c]);
  const double inv = 1. / sqrt(s);
  for (int c = 0; c < d; c++) row[c] = (float)((double)row[c] * inv);
}

__global__ void absmax_kernel(const KmSlice *sl, const float *v, int d, float *out) {
  const KmSlice s = sl[blockIdx.x];
  float m = 0.f;
  for (long i = threadIdx.x; i < (long)s.n * d; i += blockDim.x) m = fmaxf(m, fabsf(v[s.p0 * d + i]));
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  __shared__ float wm[8];
  if ((threadIdx.x & 31) == 0) wm[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); w++) m = fmaxf(m, wm[w]);
    m = fmaxf(m, wm[0]);
    atomicMax((unsigned int *)out + s.inst, __float_as_uint(m));
  }
}

__global__ void slice_sum_kernel(const KmSlice *sl, const float *dis, double *out) {
  const KmSlice s = sl[blockIdx.x];
  __shared__ double red[256];
  double acc = 0;
  for (int i = threadIdx.x; i < s.n; i += blockDim.x) acc += (double)dis[s.p0 + i];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = red[0];
}

__global__ void gather_kernel(const float *v, int d, const long *rows, long nrows, float *C) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nrows * d) return;
  const long r = i / d;
  C[i] = v[rows[r] * d + (i - r * d)];
}

template <int K>
int launch_assign(const KmWork *work, int nwork, const float *v, int d, const float *C, int k,
                  const unsigned char *active, int *assign, float *dis, cudaStream_t st) {
  const size_t smem = (size_t)k * d * sizeof(float);
  static size_t attr = 48 * 1024;
  if (smem > attr) {
    YG_CUDA(cudaFuncSetAttribute(assign_small_kernel<K>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr = smem;
  }
  assign_small_kernel<K><<<nwork, 256, smem, st>>>(work, v, d, C, k, active, assign, dis);
  YG_LAUNCH_CHECK();
  return OK;
}

}  // namespace

int km_assign_small(const KmWork *work, int nwork, const float *v, int d, const float *C,
                    int k, const unsigned char *active, int *assign, float *dis,
                    cudaStream_t st) {
  if (nwork <= 0) return OK;
  if ((size_t)k * d * 4 > 200 * 1024) {
    set_error(E_UNSUPPORTED, "grouped assignment: k*d=%ld too large for shared memory",
              (long)k * d);
    return E_UNSUPPORTED;
  }
  if (k <= 16) return launch_assign<16>(work, nwork, v, d, C, k, active, assign, dis, st);
  if (k <= 32) return launch_assign<32>(work, nwork, v, d, C, k, active, assign, dis, st);
  if (k <= 64) return launch_assign<64>(work, nwork, v, d, C, k, active, assign, dis, st);
  set_error(E_ARG, "grouped assignment: k=%d > %d", k, kSmallK);
  return E_ARG;
}

int km_histogram(const int *assign, const int *pinst, long n, int k,
                 const unsigned char *active, int *counts, cudaStream_t st) {
  if (n <= 0) return OK;
  hist_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, st>>>(assign, pinst, n, k, active, counts);
  YG_LAUNCH_CHECK();
  return OK;
}

int km_scan(const int *counts, long ncl, long *offs, long *cursor, cudaStream_t st) {
  scan_kernel<<<1, 1024, 0, st>>>(counts, ncl, offs, cursor);
  YG_LAUNCH_CHECK();
  return OK;
}

int km_scatter(const int *assign, const int *pinst, long n, int k,
               const unsigned char *active, long *cursor, long *perm, cudaStream_t st) {
  if (n <= 0) return OK;
  scatter_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, st>>>(assign, pinst, n, k, active,
                                                             cursor, perm);
  YG_LAUNCH_CHECK();
  return OK;
}

int km_update(const long *perm, const long *total, long nmax, const int *assign,
              const int *pinst, const int *counts, const float *v, int d, long ncl, int k,
              const int *shift, const unsigned char *active, long long *acc, float *C,
              cudaStream_t st) {
  YG_CUDA(cudaMemsetAsync(acc, 0, sizeof(long long) * ncl * d, st));
  if (nmax > 0) {
    const long warps = ceil_div(nmax, 32);
    const int nd = d <= 32 ? 1 : d <= 64 ? 2 : d <= 128 ? 4 : 8;
    dim3 grid((unsigned)ceil_div(warps * 32, 256), (unsigned)ceil_div(d, nd * 32));
    switch (nd) {
      case 1: segsum_kernel<1><<<grid, 256, 0, st>>>(perm, total, assign, pinst, v, d, k, shift, acc); break;
      case 2: segsum_kernel<2><<<grid, 256, 0, st>>>(perm, total, assign, pinst, v, d, k, shift, acc); break;
      case 4: segsum_kernel<4><<<grid, 256, 0, st>>>(perm, total, assign, pinst, v, d, k, shift, acc); break;
      default: segsum_kernel<8><<<grid, 256, 0, st>>>(perm, total, assign, pinst, v, d, k, shift, acc); break;
    }
    YG_LAUNCH_CHECK();
  }
  finalize_kernel<<<(unsigned)ceil_div(ncl * d, 256), 256, 0, st>>>(acc, counts, ncl, d, k, shift,
                                                                     active, C);
  YG_LAUNCH_CHECK();
  return OK;
}

int km_normalize(float *C, long ncl, int d, int k, const unsigned char *active,
                 cudaStream_t st) {
  normalize_kernel<<<(unsigned)ceil_div(ncl, 128), 128, 0, st>>>(C, ncl, d, k, active);
  YG_LAUNCH_CHECK();
  return OK;
}

int km_absmax(const KmSlice *sl, int nsl, const float *v, int d, float *out,
                     cudaStream_t st) {
  if (nsl <= 0) return OK;
  absmax_kernel<<<nsl, 256, 0, st>>>(sl, v, d, out);
  YG_LAUNCH_CHECK();
  return OK;
}

int km_slice_sums(const KmSlice *sl, int nsl, const float *dis, double *out, cudaStream_t st) {
  if (nsl <= 0) return OK;
  slice_sum_kernel<<<nsl, 256, 0, st>>>(sl, dis, out);
  YG_LAUNCH_CHECK();
  return OK;
}

int km_gather(const float *v, int d, const long *rows, long nrows, float *C, cudaStream_t st) {
  if (nrows <= 0) return OK;
  gather_kernel<<<(unsigned)ceil_div(nrows * d, 256), 256, 0, st>>>(v, d, rows, nrows, C);
  YG_LAUNCH_CHECK();
  return OK;
}

}  // namespace yg
