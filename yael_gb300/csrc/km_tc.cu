// The exact nearest-centroid step of k-means for k <= 256 on the tensor cores
// (yael/kmeans.c:242-244: knn_full with k = 1 against the centroids, which the
// reference runs through sgemm; its nearest-index rule is yael/nn.c:404-435),
// fused with the fixed-point centroid sums of the update (yael/kmeans.c:277-288,
// exact integer sums here) when they fit shared memory.
//
// One persistent CTA per SM walks a contiguous range of units (128-point
// tiles of one instance), so consecutive units mostly share an instance:
//   warp 0      TMA producer: a ring of S stages, each the tile's packed
//               16-bit points (Kp/64 blocks of 128 rows x 128 B, 128B swizzle)
//               and their 16-column side block of ones; the instance's packed
//               centroids (and their norm parts) in one resident slot,
//               reloaded when the instance changes and its last MMA is done.
//   warp 1      TMEM owner (two 128 x N FP32 accumulators) and MMA issuer:
//               Kp/16 tcgen05.mma 128xNx16 per tile plus one K = 16 step over
//               the side blocks, so the accumulator holds
//               v_j = ||c_j||^2 - 2 x.c_j of every centroid j.
//   warps 2-9   epilogue.  Warps 2-5 (one TMEM lane quadrant each, a thread
//               per point) find the smallest v and list the band of centroids
//               within 2 eps of it (eps: the rigorous error bound of the
//               16-bit products, the k-NN certificate's bound); all eight
//               warps then take the points one at a time (a lane per four
//               coordinates): FP32 direct differences over the band, FP64 on
//               near ties, the winner's fixed-point row added to the shared
//               memory sums of its centroid.
// Every wait is bounded (tc_ptx.cuh); on expiry *err is set, every role leaves
// its loop, the copies and MMAs already issued are waited for, and TMEM is
// freed.
#include <cudaTypedefs.h>
#include <limits.h>
#include <math.h>

#include "kmeans.cuh"
#include "tc_kernel.cuh"

namespace yg {
namespace kmtc {
using namespace ptx;

constexpr int NT = 320;
constexpr int BMAX = 8;  // band entries kept per point; more: every centroid is re-checked
constexpr int A_BLK = 128 * 128;  // 128 rows x 64 16-bit columns
constexpr int A_SIDE = 128 * 32;  // 128 rows x 16 16-bit columns

struct Lay {
  int nkb, N, S, fuse, csm;
  size_t stage_bytes, b_off, bside_off, cf_off, band_off, acc_off, cnt_off, bar_off, total;
};

__host__ __device__ inline Lay make_lay(int nkb, int N, int S, int fuse, int k, int d,
                                       int csm) {
  Lay L;
  L.nkb = nkb; L.N = N; L.S = S; L.fuse = fuse; L.csm = csm;
  size_t off = 0;
  L.stage_bytes = (size_t)nkb * A_BLK + A_SIDE;  // a multiple of 1024
  off += (size_t)S * L.stage_bytes;
  L.b_off = off;     off += (size_t)nkb * N * 128;  // N % 32 == 0: 1024-aligned blocks
  L.bside_off = off; off += (size_t)N * 32;
  L.cf_off = off;    off += csm ? (size_t)N * d * 4 : 0;  // FP32 centroid rows (d % 4 == 0)
  L.band_off = off;  off += (size_t)2 * 128 * (BMAX + 1) * 4;
  off = (off + 15) & ~(size_t)15;
  L.acc_off = off;   off += fuse ? (size_t)k * d * 8 : 0;
  L.cnt_off = off;   off += fuse ? (size_t)k * 4 : 0;
  off = (off + 15) & ~(size_t)15;
  L.bar_off = off;   off += (size_t)(2 * S + 8) * 8 + 16;
  L.total = off + 1024;  // alignment slack of the 1024-byte aligned base
  return L;
}

struct Params {
  const KmTcUnit *units;
  int nunits;
  int d, k, N, Kp, f16;
  const float *v, *C;
  const double *xn64;
  const float *xres;
  const SetStats *cs;
  const unsigned char *active;
  int *assign;
  float *dis;
  long long *acc;
  int *counts;
  const int *shift;
  int *err;
  int acc_global;              // sums added straight to acc / counts (k * d too large
                               // for shared memory)
  int csm;                     // the instance's FP32 centroid rows staged in shared memory
  unsigned long long wait_ns;  // bound of every wait (0: kWaitLimitNs)
  int withhold;                // test switch: the producer issues no load
};

__device__ __forceinline__ float warp_sum(float x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

constexpr int G = 8;  // rows a warp of the epilogue takes at once in phase B

// a float4 of a centroid row: shared memory (staged) or global (read-only path)
__device__ __forceinline__ float4 cload(const float *p, bool sm) {
  return sm ? *reinterpret_cast<const float4 *>(p) : __ldg(reinterpret_cast<const float4 *>(p));
}

template <int ND4>
__device__ __forceinline__ float row_dist(const float4 (&x)[ND4], const float4 (&c)[ND4],
                                          int lane, int d4) {
  float s = 0.f;
#pragma unroll
  for (int q = 0; q < ND4; q++) {
    if (lane + 32 * q < d4) {
      float t = x[q].x - c[q].x;
      s = fmaf(t, t, s);
      t = x[q].y - c[q].y;
      s = fmaf(t, t, s);
      t = x[q].z - c[q].z;
      s = fmaf(t, t, s);
      t = x[q].w - c[q].w;
      s = fmaf(t, t, s);
    }
  }
  return warp_sum(s);
}

// Phase B for one point (the whole warp): the band's exact decision, the
// outputs, and the point's fixed-point row added to its centroid's sums.  c0
// holds the first band member's row (or centroid 0's when the band
// overflowed its list); Ci the instance's centroid rows (staged or global).
template <int ND4>
__device__ __forceinline__ void finish_row(const Params &P, const int *bl, int r0, long p,
                                           const float *Ci, const float4 (&x)[ND4],
                                           const float4 (&c0)[ND4], int lane, int d, int d4,
                                           int k, float rho, bool fuse,
                                           unsigned long long *sacc, int *scnt, int sh,
                                           int inst) {
  const int cnt = bl[r0 * (BMAX + 1)];
  const int nm = cnt > BMAX ? k : cnt;  // an overflowing band: every centroid
  float e1 = INFINITY, e2 = INFINITY;
  int j1 = -1;
  for (int m = 0; m < nm; m++) {
    const int j = cnt > BMAX ? m : bl[r0 * (BMAX + 1) + 1 + m];
    float e;
    if (m == 0) {
      e = row_dist<ND4>(x, c0, lane, d4);
    } else {
      float4 c[ND4];
#pragma unroll
      for (int q = 0; q < ND4; q++) {
        const int c4 = lane + 32 * q;
        c[q] = c4 < d4 ? cload(Ci + (long)j * d + 4 * c4, P.csm != 0)
                       : make_float4(0.f, 0.f, 0.f, 0.f);
      }
      e = row_dist<ND4>(x, c, lane, d4);
    }
    // members come in increasing index order: strict '<' keeps the lower
    // index on equal values
    if (e < e1) { e2 = e1; e1 = e; j1 = j; } else if (e < e2) { e2 = e; }
  }
  int oj = -1;
  float od = 1e30f;
  if (j1 >= 0 && e1 < 1e30f) {
    oj = j1;
    od = e1;
    if (e2 < INFINITY && e2 - e1 <= rho * (e1 + e2)) {
      // near tie: FP64 over the members, sequential over coordinates, a lane
      // per member; lowest index on equal values
      double best = INFINITY;
      int bj = INT_MAX;
      for (int m = lane; m < nm; m += 32) {
        const int j = cnt > BMAX ? m : bl[r0 * (BMAX + 1) + 1 + m];
        const float *cr = Ci + (long)j * d, *xr = P.v + p * d;
        double s = 0;
        for (int c = 0; c < d; c++) {
          const double t = (double)xr[c] - (double)cr[c];
          s += t * t;
        }
        if (s < best || (s == best && j < bj)) { best = s; bj = j; }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const double ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int oj2 = __shfl_xor_sync(0xffffffffu, bj, o);
        if (ob < best || (ob == best && oj2 < bj)) { best = ob; bj = oj2; }
      }
      if (bj != INT_MAX && best < 1e30) { oj = bj; od = (float)best; }
      else { oj = -1; od = 1e30f; }
    }
  }
  if (lane == 0) {
    P.assign[p] = oj;
    P.dis[p] = od;
  }
  if (fuse && oj >= 0) {
    // the instance's shared-memory sums, or the global ones directly
    const long g = (long)inst * k + oj;
    unsigned long long *row_acc =
        P.acc_global ? reinterpret_cast<unsigned long long *>(P.acc) + g * d
                     : sacc + (long)oj * d;
#pragma unroll
    for (int q = 0; q < ND4; q++) {
      const int c4 = lane + 32 * q;
      if (c4 < d4) {
        atomicAdd(row_acc + 4 * c4 + 0, (unsigned long long)fixed_of(x[q].x, sh));
        atomicAdd(row_acc + 4 * c4 + 1, (unsigned long long)fixed_of(x[q].y, sh));
        atomicAdd(row_acc + 4 * c4 + 2, (unsigned long long)fixed_of(x[q].z, sh));
        atomicAdd(row_acc + 4 * c4 + 3, (unsigned long long)fixed_of(x[q].w, sh));
      }
    }
    if (lane == 0) {
      if (P.acc_global) atomicAdd(P.counts + g, 1);
      else atomicAdd(scnt + oj, 1);
    }
  }
}

template <int ND4>
__global__ void __launch_bounds__(NT, 1)
    km_tc_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapAs,
                 const __grid_constant__ CUtensorMap mapB, const __grid_constant__ CUtensorMap mapBs,
                 const __grid_constant__ CUtensorMap mapC, int S, Params P) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t *base = reinterpret_cast<uint8_t *>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  const int nkb = P.Kp / 64, N = P.N, k = P.k, d = P.d;
  const bool fuse = P.acc != nullptr;
  const bool sfuse = fuse && !P.acc_global;  // shared-memory sums
  const Lay lay = make_lay(nkb, N, S, sfuse ? 1 : 0, k, d, P.csm);
  uint8_t *Stg = base;
  uint8_t *Bs = base + lay.b_off;
  uint8_t *Bside = base + lay.bside_off;
  float *Cf = reinterpret_cast<float *>(base + lay.cf_off);
  int *band = reinterpret_cast<int *>(base + lay.band_off);  // [2][128][BMAX + 1]
  unsigned long long *sacc = reinterpret_cast<unsigned long long *>(base + lay.acc_off);
  int *scnt = reinterpret_cast<int *>(base + lay.cnt_off);
  uint64_t *bars = reinterpret_cast<uint64_t *>(base + lay.bar_off);
  uint64_t *full = bars, *empty = bars + S, *tfull = bars + 2 * S, *tempty = bars + 2 * S + 2;
  uint64_t *bfull = bars + 2 * S + 4, *bempty = bars + 2 * S + 5, *mdone = bars + 2 * S + 6;
  uint64_t *cempty = bars + 2 * S + 7;  // the staged FP32 centroids read by the epilogue
  uint32_t *tmem_holder = reinterpret_cast<uint32_t *>(bars + 2 * S + 8);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_holder + 1);
  const uint64_t wl = P.wait_ns ? (uint64_t)P.wait_ns : kWaitLimitNs;
  const uint32_t tcols = N * 2 <= 32 ? 32u : N * 2 <= 64 ? 64u : N * 2 <= 128 ? 128u
                         : N * 2 <= 256 ? 256u : 512u;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // this CTA's contiguous range of units
  const int w0 = (int)((long)blockIdx.x * P.nunits / gridDim.x);
  const int w1 = (int)((long)(blockIdx.x + 1) * P.nunits / gridDim.x);

  if (threadIdx.x == 0) {
    for (int s = 0; s < S; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int a = 0; a < 2; a++) {
      mbar_init(&tfull[a], 1);
      mbar_init(&tempty[a], 4);  // the four lane-quadrant warps of the epilogue
    }
    mbar_init(bfull, 1);
    mbar_init(bempty, 1);
    mbar_init(mdone, 1);
    mbar_init(cempty, 8);  // the eight epilogue warps
    *abort_flag = 0;
    fence_mbar_init();
  }
  if (warp == 1) {
    tmem_alloc(tmem_holder, tcols);
    tmem_relinquish();
  }
  if (sfuse && warp >= 2) {
    for (int i = threadIdx.x - 64; i < k * d; i += 256) sacc[i] = 0ull;
    for (int i = threadIdx.x - 64; i < k; i += 256) scnt[i] = 0;
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_holder;

  if (warp == 0) {
    // ---------------- TMA producer
    if (lane == 0 && !P.withhold) {
      int sn = 0;
      uint32_t phn = 0;
      uint32_t issued = 0, last_par = 0;  // per stage: issued at least once, parity of the last
      int cur = -1, nbl = 0;
      bool ok = true;
      const uint32_t abytes = (uint32_t)(nkb * A_BLK + A_SIDE);
      const uint32_t bbytes = (uint32_t)(nkb * N * 128 + N * 32 + (P.csm ? N * d * 4 : 0));
      for (int w = w0; w < w1 && ok; w++) {
        const KmTcUnit u = P.units[w];
        if (!P.active[u.inst]) continue;
        if (u.inst != cur) {
          // the previous instance's centroids are free once its MMAs are done
          if (nbl > 0 && !mbar_wait(bempty, (uint32_t)((nbl - 1) & 1), abort_flag, wl)) {
            ok = false;
            break;
          }
          // and the staged FP32 rows once the epilogue is done with them
          if (nbl > 0 && P.csm && !mbar_wait(cempty, (uint32_t)((nbl - 1) & 1), abort_flag, wl)) {
            ok = false;
            break;
          }
          mbar_arrive_expect_tx(bfull, bbytes);
          for (int kb = 0; kb < nkb; kb++)
            tma_load_2d(&mapB, bfull, Bs + (size_t)kb * N * 128, kb * 64, u.inst * k);
          tma_load_2d(&mapBs, bfull, Bside, 0, u.inst * k);
          if (P.csm) tma_load_2d(&mapC, bfull, Cf, 0, u.inst * k);
          nbl++;
          cur = u.inst;
        }
        const int s = sn;
        const uint32_t ph = phn;
        if (++sn == S) { sn = 0; phn ^= 1; }
        if (!mbar_wait(&empty[s], ph ^ 1, abort_flag, wl)) { ok = false; break; }
        uint8_t *sp = Stg + (size_t)s * lay.stage_bytes;
        mbar_arrive_expect_tx(&full[s], abytes);
        for (int kb = 0; kb < nkb; kb++)
          tma_load_2d(&mapA, &full[s], sp + (size_t)kb * A_BLK, kb * 64, (int)u.p0);
        tma_load_2d(&mapAs, &full[s], sp + (size_t)nkb * A_BLK, 0, (int)u.p0);
        issued |= 1u << s;
        last_par = (last_par & ~(1u << s)) | (ph << s);
      }
      // every copy issued has landed before the CTA's shared memory is released
      for (int s = 0; s < S; s++)
        if (issued >> s & 1) mbar_wait_drain(&full[s], last_par >> s & 1);
      if (nbl > 0) mbar_wait_drain(bfull, (uint32_t)((nbl - 1) & 1));
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer
    if (lane == 0) {
      const uint32_t idesc = idesc_16_f32(128, N, P.f16 != 0);
      int sn = 0;
      uint32_t phn = 0;
      int it = 0, cur = -1, nbl = 0;
      bool ok = true, any = false;
      for (int w = w0; w < w1 && ok; w++) {
        const KmTcUnit u = P.units[w];
        if (!P.active[u.inst]) continue;
        if (u.inst != cur) {
          if (nbl > 0) umma_commit(bempty);  // the previous centroids' last reads done
          if (!mbar_wait(bfull, (uint32_t)(nbl & 1), abort_flag, wl)) { ok = false; break; }
          nbl++;
          cur = u.inst;
        }
        const int a = it & 1;
        const uint32_t uu = (uint32_t)(it >> 1);
        if (!mbar_wait(&tempty[a], (uu & 1) ^ 1, abort_flag, wl)) { ok = false; break; }
        const int s = sn;
        const uint32_t ph = phn;
        if (++sn == S) { sn = 0; phn ^= 1; }
        if (!mbar_wait(&full[s], ph, abort_flag, wl)) { ok = false; break; }
        tc_fence_after();
        const uint32_t dt = tmem + (uint32_t)(a * N);
        const uint32_t sa = smem_u32(Stg + (size_t)s * lay.stage_bytes);
        const uint32_t sb = smem_u32(Bs);
        for (int kb = 0; kb < nkb; kb++) {
          const uint64_t da = desc_k_sw128(sa + (uint32_t)(kb * A_BLK));
          const uint64_t db = desc_k_sw128(sb + (uint32_t)(kb * N * 128));
#pragma unroll
          for (int kk = 0; kk < 4; kk++)
            umma_bf16(dt, da + (uint64_t)(kk * 2), db + (uint64_t)(kk * 2), idesc,
                      (kb > 0 || kk > 0) ? 1u : 0u);
        }
        umma_bf16(dt, desc_k_sw32(sa + (uint32_t)(nkb * A_BLK)), desc_k_sw32(smem_u32(Bside)),
                  idesc, 1u);
        any = true;
        umma_commit(&empty[s]);
        umma_commit(&tfull[a]);
        it++;
      }
      // every MMA issued has finished with TMEM and shared memory
      if (any) {
        umma_commit(mdone);
        mbar_wait_drain(mdone, 0);
      }
    }
  } else {
    // ---------------- epilogue
    const int ew = warp - 2;       // 0..7
    const int grp = warp & 3;      // TMEM lane quadrant (warps 2-5 read TMEM)
    const int row = grp * 32 + lane;
    const uint32_t lane_base = (uint32_t)(grp * 32) << 16;
    const float u24 = 5.9604645e-08f;
    const float rho = (float)(d + 4) * u24;
    const float B = __uint_as_float(P.cs->max_norm_bits);
    const float dB = __uint_as_float(P.cs->max_resid_bits);
    const float Kt = (float)(P.Kp + 16);
    const float un = (float)((d + 31) / 32 + 6) * u24;
    const int d4 = d >> 2;
    int it = 0, cur = -1;
    bool ok = true;
    auto flush = [&](int inst) {
      asm volatile("bar.sync 1, 256;" ::: "memory");
      const long g0 = (long)inst * k;
      for (int i = threadIdx.x - 64; i < k * d; i += 256) {
        const unsigned long long x = sacc[i];
        if (x) atomicAdd((unsigned long long *)(P.acc + g0 * d + i), x);
        sacc[i] = 0ull;
      }
      for (int i = threadIdx.x - 64; i < k; i += 256) {
        if (scnt[i]) atomicAdd(P.counts + g0 + i, scnt[i]);
        scnt[i] = 0;
      }
      asm volatile("bar.sync 1, 256;" ::: "memory");
    };
    int nbl = 0;  // centroid tiles seen (the staged FP32 rows' bfull phases)
    for (int w = w0; w < w1 && ok; w++) {
      const KmTcUnit u = P.units[w];
      if (!P.active[u.inst]) continue;
      if (u.inst != cur) {
        if (sfuse && cur >= 0) flush(cur);
        // the previous instance's staged rows are no longer read by this warp
        if (P.csm && cur >= 0 && lane == 0) mbar_arrive(cempty);
        if (P.csm) {
          // the new instance's rows have landed (the MMA warp waits on the same
          // phase of bfull before its first MMA of the instance)
          ok = mbar_wait(bfull, (uint32_t)(nbl & 1), abort_flag, wl);
          __syncwarp();
          ok = __all_sync(0xffffffffu, ok);
        }
        nbl++;
        cur = u.inst;
      }
      const int a = it & 1;
      int *bl = band + a * 128 * (BMAX + 1);
      if (ew < 4) {
        const uint32_t uu = (uint32_t)(it >> 1);
        ok = ok && mbar_wait(&tfull[a], uu & 1, abort_flag, wl);
        __syncwarp();
        ok = __all_sync(0xffffffffu, ok);
        if (ok) {
          tc_fence_after();
          const bool rv = row < u.np;
          const long p = u.p0 + row;
          float eps = 0.f;
          if (rv) {
            const float qn = sqrtf(fmaxf((float)P.xn64[p], 0.f)) * (1.f + 1e-5f);
            const float dq = P.xres[p];
            const float dot = dq * (B + dB) + qn * dB;
            const float accb = Kt * 2.f * u24 * (2.f * (qn + dq) * (B + dB) + 1.001f * B * B);
            eps = (2.f * dot + u24 * B * B + accb + un * (qn * qn + B * B)) * 1.1f + 1e-30f;
          }
          const uint32_t tc = tmem + lane_base + (uint32_t)(a * N);
          uint32_t r[32];
          float vmin = INFINITY;
          for (int c0 = 0; c0 < N; c0 += 32) {
            tmem_ld32(tc + (uint32_t)c0, r);
            tmem_ld_wait(r);
#pragma unroll
            for (int i = 0; i < 32; i++)
              if (c0 + i < k) vmin = fminf(vmin, __uint_as_float(r[i]));
          }
          const float lim = vmin + 2.f * eps;
          int cnt = 0;
          for (int c0 = 0; c0 < N; c0 += 32) {
            tmem_ld32(tc + (uint32_t)c0, r);
            tmem_ld_wait(r);
#pragma unroll
            for (int i = 0; i < 32; i++) {
              if (c0 + i < k && __uint_as_float(r[i]) <= lim) {
                if (cnt < BMAX) bl[row * (BMAX + 1) + 1 + cnt] = c0 + i;
                cnt++;
              }
            }
          }
          tc_fence_before();
          bl[row * (BMAX + 1)] = (rv && vmin < INFINITY) ? cnt : 0;
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&tempty[a]);
      }
      // the band lists of this tile are written (and the other buffer's were
      // read by every warp before it): one barrier per tile, all warps agree
      ok = bar_red_and_256(ok);
      if (!ok) break;
      // phase B: a warp takes rows ew, ew + 8, ..., eight at a time, with the
      // point rows and each point's first band member loaded for all eight
      // before any is used (the loads are the latency of this phase)
      const int sh = fuse ? P.shift[u.inst] : 0;
      const float *Ci = P.csm ? Cf : P.C + (long)u.inst * k * d;
#pragma unroll 1
      for (int i0 = 0; i0 < 128 / 8; i0 += G) {
        if (ew + 8 * i0 >= u.np) break;  // uniform over the warp
        float4 xb[G][ND4], cb[G][ND4];
#pragma unroll
        for (int g = 0; g < G; g++) {
          const int r0 = ew + 8 * (i0 + g);
          const bool val = r0 < u.np;
          const int cnt = val ? bl[r0 * (BMAX + 1)] : 0;
          const int j0 = cnt > BMAX ? 0 : cnt > 0 ? bl[r0 * (BMAX + 1) + 1] : 0;
          const long p = u.p0 + r0;
#pragma unroll
          for (int q = 0; q < ND4; q++) {
            const int c4 = lane + 32 * q;
            const bool in = val && c4 < d4;
            xb[g][q] = in ? __ldg(reinterpret_cast<const float4 *>(P.v + p * d) + c4)
                          : make_float4(0.f, 0.f, 0.f, 0.f);
            cb[g][q] = in && cnt > 0 ? cload(Ci + (long)j0 * d + 4 * c4, P.csm != 0)
                                     : make_float4(0.f, 0.f, 0.f, 0.f);
          }
        }
#pragma unroll
        for (int g = 0; g < G; g++) {
          const int r0 = ew + 8 * (i0 + g);
          if (r0 < u.np)
            finish_row<ND4>(P, bl, r0, u.p0 + r0, Ci, xb[g], cb[g], lane, d, d4, k, rho, fuse,
                            sacc, scnt, sh, u.inst);
        }
      }
      it++;
    }
    if (sfuse && ok && cur >= 0) flush(cur);
  }

  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 1) {
    __syncwarp();
    tmem_dealloc(tmem, tcols);
  }
  if (threadIdx.x == 0 && *abort_flag && P.err) atomicExch(P.err, 1);
}

}  // namespace kmtc

namespace {
// a tensor map over FP32 rows, no swizzle (box: cols x rows)
int make_map_f32(CUtensorMap *m, const void *ptr, uint64_t cols, uint64_t rows, uint32_t box_cols,
                 uint32_t box_rows) {
  YG_CHECK(tck::get_encode());
  if (!ptr || (reinterpret_cast<uintptr_t>(ptr) & 15) || ((cols * 4) & 15) || rows == 0) {
    set_error(E_ARG, "tensor map (f32): null / misaligned operand");
    return E_ARG;
  }
  cuuint64_t dims[2] = {cols, rows};
  cuuint64_t strides[1] = {cols * 4};
  cuuint32_t box[2] = {box_cols, box_rows};
  cuuint32_t es[2] = {1, 1};
  CUresult r = tck::g_encode(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void *>(ptr), dims,
                             strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                             CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error(E_CUDA, "cuTensorMapEncodeTiled (f32) failed (%d)", (int)r);
    return E_CUDA;
  }
  return OK;
}
}  // namespace

bool km_tc_supported(int d, int k, const float *v, const float *C) {
  if (!(d >= 4 && d % 4 == 0 && d <= 256 && k >= 1 && k <= kTcMaxK &&
        (reinterpret_cast<uintptr_t>(v) & 15) == 0 && (reinterpret_cast<uintptr_t>(C) & 15) == 0))
    return false;
  // a ring of two stages beside the centroid tile, without staging or
  // shared-memory sums, must fit (not so for d > 128 with k > 224)
  const int Kp = ((d + 63) / 64) * 64, N = ((k + 31) / 32) * 32;
  return kmtc::make_lay(Kp / 64, N, 2, 0, k, d, 0).total <= 227 * 1024;
}

bool km_tc_fuses(int d, int k) { return (size_t)k * d * 8 <= 48 * 1024; }

int km_tc_assign(const KmTcUnit *units, int nunits, const KmTcPoints &P, const float *v, int d,
                 const float *C, int ninst, int k, void *cpk, void *cside, float *cres,
                 SetStats *cstats, const unsigned char *active, int *assign, float *dis,
                 long long *acc, int *counts, const int *shift, int *err, cudaStream_t st) {
  using namespace kmtc;
  if (nunits <= 0) return OK;
  if (!km_tc_supported(d, k, v, C) || P.Kp != ((d + 63) / 64) * 64) {
    set_error(E_UNSUPPORTED, "km_tc_assign: d=%d k=%d Kp=%d", d, k, P.Kp);
    return E_UNSUPPORTED;
  }
  const int N = ((k + 31) / 32) * 32, nkb = P.Kp / 64;
  const long ncl = (long)ninst * k;
  // the centroids, packed as the points are (same 16-bit format)
  YG_CHECK(stats_reset(cstats, st));
  YG_CHECK(prep_rows(C, d, (int)ncl, d, 1.f, nullptr, nullptr, nullptr, cres,
                     (__nv_bfloat16 *)cpk, P.Kp, (__nv_bfloat16 *)cside, 1, cstats, st, 8, P.f16));
  // the sums go through shared memory when an instance's k x d fit, else
  // straight to the global accumulators; the instance's FP32 centroid rows
  // are staged when they are few.  Both give way, staging first, when a ring
  // of two stages would not fit beside them.
  int acc_global = acc != nullptr && !km_tc_fuses(d, k);
  int fuse = acc != nullptr && !acc_global;
  int csm = (size_t)N * d * 4 <= 32 * 1024;
  auto fits = [&](int S_) {
    return make_lay(nkb, N, S_, fuse, k, d, csm).total <= 227 * 1024;
  };
  if (!fits(2)) csm = 0;
  if (!fits(2) && fuse) {
    fuse = 0;
    acc_global = 1;
  }
  int S = 6;
  while (S > 2 && !fits(S)) S--;
  const Lay lay = make_lay(nkb, N, S, fuse, k, d, csm);
  if (lay.total > 227 * 1024) {
    set_error(E_UNSUPPORTED, "km_tc_assign: shared memory %zu too large (d=%d k=%d)", lay.total,
              d, k);
    return E_UNSUPPORTED;
  }
  auto kern = d <= 128 ? km_tc_kernel<1> : km_tc_kernel<2>;
  YG_CHECK(ensure_smem((const void *)kern, lay.total));
  CUtensorMap mA, mAs, mB, mBs, mC;
  YG_CHECK(tck::make_map(&mA, P.pk, P.Kp, P.n, (uint64_t)P.Kp * 2, 64, 128,
                         CU_TENSOR_MAP_SWIZZLE_128B));
  YG_CHECK(tck::make_map(&mAs, P.side, 16, P.n, 32, 16, 128, CU_TENSOR_MAP_SWIZZLE_32B));
  YG_CHECK(tck::make_map(&mB, cpk, P.Kp, ncl, (uint64_t)P.Kp * 2, 64, (uint32_t)N,
                         CU_TENSOR_MAP_SWIZZLE_128B));
  YG_CHECK(tck::make_map(&mBs, cside, 16, ncl, 32, 16, (uint32_t)N, CU_TENSOR_MAP_SWIZZLE_32B));
  if (csm) YG_CHECK(make_map_f32(&mC, C, d, ncl, (uint32_t)d, (uint32_t)N));
  else mC = mBs;
  int dev = 0, nsm = 0;
  YG_CUDA(cudaGetDevice(&dev));
  YG_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  Params p;
  p.units = units; p.nunits = nunits; p.d = d; p.k = k; p.N = N; p.Kp = P.Kp; p.f16 = P.f16;
  p.v = v; p.C = C; p.xn64 = P.xn64; p.xres = P.xres; p.cs = cstats; p.active = active;
  p.assign = assign; p.dis = dis; p.acc = acc; p.counts = counts; p.shift = shift; p.err = err;
  p.acc_global = acc_global;
  p.csm = csm;
  p.wait_ns = wait_limit_ns();
  p.withhold = test_withhold_loads() ? 1 : 0;
  const unsigned g = (unsigned)(nunits < nsm ? nunits : nsm);
  kern<<<g, NT, lay.total, st>>>(mA, mAs, mB, mBs, mC, S, p);
  YG_LAUNCH_CHECK();
  return OK;
}

}  // namespace yg
