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
  int nkb, N, S, fuse;
  size_t stage_bytes, b_off, bside_off, band_off, acc_off, cnt_off, bar_off, total;
};

__host__ __device__ inline Lay make_lay(int nkb, int N, int S, int fuse, int k, int d) {
  Lay L;
  L.nkb = nkb; L.N = N; L.S = S; L.fuse = fuse;
  size_t off = 0;
  L.stage_bytes = (size_t)nkb * A_BLK + A_SIDE;  // a multiple of 1024
  off += (size_t)S * L.stage_bytes;
  L.b_off = off;     off += (size_t)nkb * N * 128;  // N % 32 == 0: 1024-aligned blocks
  L.bside_off = off; off += (size_t)N * 32;
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
  unsigned long long wait_ns;  // bound of every wait (0: kWaitLimitNs)
  int withhold;                // test switch: the producer issues no load
};

__device__ __forceinline__ float warp_sum(float x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

__global__ void __launch_bounds__(NT, 1)
    km_tc_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapAs,
                 const __grid_constant__ CUtensorMap mapB, const __grid_constant__ CUtensorMap mapBs,
                 int S, Params P) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t *base = reinterpret_cast<uint8_t *>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  const int nkb = P.Kp / 64, N = P.N, k = P.k, d = P.d;
  const bool fuse = P.acc != nullptr;
  const Lay lay = make_lay(nkb, N, S, fuse ? 1 : 0, k, d);
  uint8_t *Stg = base;
  uint8_t *Bs = base + lay.b_off;
  uint8_t *Bside = base + lay.bside_off;
  int *band = reinterpret_cast<int *>(base + lay.band_off);  // [2][128][BMAX + 1]
  unsigned long long *sacc = reinterpret_cast<unsigned long long *>(base + lay.acc_off);
  int *scnt = reinterpret_cast<int *>(base + lay.cnt_off);
  uint64_t *bars = reinterpret_cast<uint64_t *>(base + lay.bar_off);
  uint64_t *full = bars, *empty = bars + S, *tfull = bars + 2 * S, *tempty = bars + 2 * S + 2;
  uint64_t *bfull = bars + 2 * S + 4, *bempty = bars + 2 * S + 5, *mdone = bars + 2 * S + 6;
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
    *abort_flag = 0;
    fence_mbar_init();
  }
  if (warp == 1) {
    tmem_alloc(tmem_holder, tcols);
    tmem_relinquish();
  }
  if (fuse && warp >= 2) {
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
      const uint32_t bbytes = (uint32_t)(nkb * N * 128 + N * 32);
      for (int w = w0; w < w1 && ok; w++) {
        const KmTcUnit u = P.units[w];
        if (!P.active[u.inst]) continue;
        if (u.inst != cur) {
          // the previous instance's centroids are free once its MMAs are done
          if (nbl > 0 && !mbar_wait(bempty, (uint32_t)((nbl - 1) & 1), abort_flag, wl)) {
            ok = false;
            break;
          }
          mbar_arrive_expect_tx(bfull, bbytes);
          for (int kb = 0; kb < nkb; kb++)
            tma_load_2d(&mapB, bfull, Bs + (size_t)kb * N * 128, kb * 64, u.inst * k);
          tma_load_2d(&mapBs, bfull, Bside, 0, u.inst * k);
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
    for (int w = w0; w < w1 && ok; w++) {
      const KmTcUnit u = P.units[w];
      if (!P.active[u.inst]) continue;
      if (fuse && u.inst != cur) {
        if (cur >= 0) flush(cur);
        cur = u.inst;
      }
      cur = u.inst;
      const int a = it & 1;
      int *bl = band + a * 128 * (BMAX + 1);
      if (ew < 4) {
        const uint32_t uu = (uint32_t)(it >> 1);
        ok = mbar_wait(&tfull[a], uu & 1, abort_flag, wl);
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
      const int sh = fuse ? P.shift[u.inst] : 0;
      for (int r0 = ew; r0 < u.np; r0 += 8) {
        const long p = u.p0 + r0;
        const int cnt = bl[r0 * (BMAX + 1)];
        float4 x4[2];
#pragma unroll
        for (int q = 0; q < 2; q++) {
          const int c4 = lane + 32 * q;
          x4[q] = c4 < d4 ? __ldg(reinterpret_cast<const float4 *>(P.v + p * d) + c4)
                          : make_float4(0.f, 0.f, 0.f, 0.f);
        }
        const int nm = cnt > BMAX ? k : cnt;  // an overflowing band: every centroid
        const float *Ci = P.C + (long)u.inst * k * d;
        float e1 = INFINITY, e2 = INFINITY;
        int j1 = -1;
        for (int m = 0; m < nm; m++) {
          const int j = cnt > BMAX ? m : bl[r0 * (BMAX + 1) + 1 + m];
          float sacc_ = 0.f;
#pragma unroll
          for (int q = 0; q < 2; q++) {
            const int c4 = lane + 32 * q;
            if (c4 < d4) {
              const float4 cv = __ldg(reinterpret_cast<const float4 *>(Ci + (long)j * d) + c4);
              float t = x4[q].x - cv.x;
              sacc_ = fmaf(t, t, sacc_);
              t = x4[q].y - cv.y;
              sacc_ = fmaf(t, t, sacc_);
              t = x4[q].z - cv.z;
              sacc_ = fmaf(t, t, sacc_);
              t = x4[q].w - cv.w;
              sacc_ = fmaf(t, t, sacc_);
            }
          }
          const float e = warp_sum(sacc_);
          if (e < e1) { e2 = e1; e1 = e; j1 = j; } else if (e < e2) { e2 = e; }
        }
        int oj = -1;
        float od = 1e30f;
        if (j1 >= 0 && e1 < 1e30f) {
          oj = j1;
          od = e1;
          if (e2 < INFINITY && e2 - e1 <= rho * (e1 + e2)) {
            // near tie: FP64 over the members, sequential over coordinates, a
            // lane per member; lowest index on equal values
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
          unsigned long long *row_acc = sacc + (long)oj * d;
#pragma unroll
          for (int q = 0; q < 2; q++) {
            const int c4 = lane + 32 * q;
            if (c4 < d4) {
              atomicAdd(row_acc + 4 * c4 + 0, (unsigned long long)fixed_of(x4[q].x, sh));
              atomicAdd(row_acc + 4 * c4 + 1, (unsigned long long)fixed_of(x4[q].y, sh));
              atomicAdd(row_acc + 4 * c4 + 2, (unsigned long long)fixed_of(x4[q].z, sh));
              atomicAdd(row_acc + 4 * c4 + 3, (unsigned long long)fixed_of(x4[q].w, sh));
            }
          }
          if (lane == 0) atomicAdd(scnt + oj, 1);
        }
      }
      it++;
    }
    if (fuse && ok && cur >= 0) flush(cur);
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

bool km_tc_supported(int d, int k, const float *v, const float *C) {
  return d >= 4 && d % 4 == 0 && d <= 256 && k >= 1 && k <= kTcMaxK &&
         (reinterpret_cast<uintptr_t>(v) & 15) == 0 && (reinterpret_cast<uintptr_t>(C) & 15) == 0;
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
  const int fuse = acc != nullptr;
  if (fuse && !km_tc_fuses(d, k)) {
    set_error(E_UNSUPPORTED, "km_tc_assign: fused sums of k*d=%ld need too much shared memory",
              (long)k * d);
    return E_UNSUPPORTED;
  }
  int S = 6;
  while (S > 2 && make_lay(nkb, N, S, fuse, k, d).total > 227 * 1024) S--;
  const Lay lay = make_lay(nkb, N, S, fuse, k, d);
  if (lay.total > 227 * 1024) {
    set_error(E_UNSUPPORTED, "km_tc_assign: shared memory %zu too large (d=%d k=%d)", lay.total,
              d, k);
    return E_UNSUPPORTED;
  }
  YG_CHECK(ensure_smem((const void *)km_tc_kernel, lay.total));
  CUtensorMap mA, mAs, mB, mBs;
  YG_CHECK(tck::make_map(&mA, P.pk, P.Kp, P.n, (uint64_t)P.Kp * 2, 64, 128,
                         CU_TENSOR_MAP_SWIZZLE_128B));
  YG_CHECK(tck::make_map(&mAs, P.side, 16, P.n, 32, 16, 128, CU_TENSOR_MAP_SWIZZLE_32B));
  YG_CHECK(tck::make_map(&mB, cpk, P.Kp, ncl, (uint64_t)P.Kp * 2, 64, (uint32_t)N,
                         CU_TENSOR_MAP_SWIZZLE_128B));
  YG_CHECK(tck::make_map(&mBs, cside, 16, ncl, 32, 16, (uint32_t)N, CU_TENSOR_MAP_SWIZZLE_32B));
  int dev = 0, nsm = 0;
  YG_CUDA(cudaGetDevice(&dev));
  YG_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  Params p;
  p.units = units; p.nunits = nunits; p.d = d; p.k = k; p.N = N; p.Kp = P.Kp; p.f16 = P.f16;
  p.v = v; p.C = C; p.xn64 = P.xn64; p.xres = P.xres; p.cs = cstats; p.active = active;
  p.assign = assign; p.dis = dis; p.acc = acc; p.counts = counts; p.shift = shift; p.err = err;
  p.wait_ns = wait_limit_ns();
  p.withhold = test_withhold_loads() ? 1 : 0;
  const unsigned g = (unsigned)(nunits < nsm ? nunits : nsm);
  km_tc_kernel<<<g, NT, lay.total, st>>>(mA, mAs, mB, mBs, S, p);
  YG_LAUNCH_CHECK();
  return OK;
}

}  // namespace yg
