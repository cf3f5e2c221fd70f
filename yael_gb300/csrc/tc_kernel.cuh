// The tcgen05 16-bit (bf16 or fp16) distance + selection kernel and its host launcher, as
// templates instantiated by tc_scan.cu / tc_scan_r2.cu (query tile resident in
// shared memory) and tc_scan_qs.cu / tc_scan_qs2.cu (query tile streamed with
// every K block, any Kp).
//
// One CTA = one 128-row query tile x one chunk of 256-row base tiles.
//   warp 0      TMA producer: a ring of S stages, each one 64-column K block of
//               a base tile (plus the matching query block when streamed) or
//               the 16-column norm block, 128B / 32B swizzled.
//   warp 1      TMEM owner (512 columns = two 128x256 FP32 accumulators) and
//               MMA issuer: Kp/16 (+1) tcgen05.mma 128x256x16 per base tile.
//   warps 2-9   selection: TMEM lane = query row; warps 2-5 read columns
//               0-127 and warps 6-9 columns 128-255 of each accumulator with
//               tcgen05.ld 32x32b.x32, filter against a running bound and
//               update the per-row list (TOPC / TOPV) or append candidates
//               (THRESH).
// The accumulators are double-buffered so the selection of tile t overlaps the
// MMAs of tile t+1.
//
// PAIR: the CTAs of a query-tile pair form a cluster and run one 256x256x16
// MMA per K step over both SMs (tcgen05 cta_group::2): each CTA holds its own
// 128 query rows and loads only half (128 rows) of every base block, and the
// leader CTA's MMA warp drives both tensor cores.  Per SM this halves the
// shared-memory traffic of the base operand (read by the MMA and written by
// TMA), which bounds the single-CTA form.  Pair protocol: the stage-full and
// query-full barriers of the leader collect both CTAs' TMA bytes; the leader's
// commits arrive on the stage-empty / accumulator-full barriers of both CTAs;
// the selection warps of both CTAs arrive on the leader's accumulator-empty
// barriers.
//
// All waits are bounded (tc_ptx.cuh); on expiry the kernel sets *err, every
// role leaves its loop and TMEM is freed.
#pragma once
#include <cudaTypedefs.h>
#include <limits.h>
#include <math.h>

#include "tc_ptx.cuh"
#include "tc_scan.cuh"

namespace yg {
namespace tck {
using namespace ptx;

constexpr int NT_TC = 320;
constexpr int N_EPI = 256;               // selection threads
constexpr int STAGE_BYTES = 256 * 128;   // 256 rows x 64 bf16
constexpr int QBLK_BYTES = 128 * 128;    // 128 rows x 64 bf16
constexpr int QN_BYTES = 4096;           // 128 rows x 16 bf16 (padded to 4 KB)
constexpr int BN_BYTES = 256 * 32;       // 256 rows x 16 bf16
constexpr int TMEM_COLS = 512;

struct Layout {
  int nkb, S, C, mode;
  size_t q_off, qn_off, stg_off, stage_bytes, list_off, bar_off, total;
};

// qs: the query tile is streamed with each K block (stage = B block + A block)
// instead of staying resident for the whole chunk; pair: a stage holds this
// CTA's half of the base block
__host__ __device__ inline Layout make_layout(int nkb, int S, int mode, int C, bool qs,
                                              bool pair) {
  Layout L;
  L.nkb = nkb; L.S = S; L.mode = mode; L.C = C;
  size_t off = 0;
  L.q_off = off;   off += qs ? 0 : (size_t)nkb * QBLK_BYTES;
  L.qn_off = off;  off += qs ? 0 : QN_BYTES;
  // a stage: this CTA's base block, the query block when streamed, and room
  // for the norm blocks that travel with the last K block of a tile
  L.stage_bytes = (pair ? STAGE_BYTES / 2 : STAGE_BYTES) + BN_BYTES +
                  (qs ? QBLK_BYTES + QN_BYTES : 0);
  L.stg_off = off; off += (size_t)S * L.stage_bytes;
  L.list_off = off;
  if (mode != SCAN_THRESH) off += (size_t)(C > 16 ? N_EPI : 128) * C * 8;
  off = (off + 15) & ~(size_t)15;
  L.bar_off = off; off += (size_t)(2 * S + 8) * 8 + 16;
  L.total = off + 1024;  // alignment slack for the 1024-byte aligned base
  return L;
}

__device__ __forceinline__ float fmin3(float a, float b, float c) {
  float r;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}

// sorted insertion of (x, j) into an ascending register list; the caller has
// Upper bound of the C-th smallest value of a thread's 128 columns (four
// 32-column register sets): the largest of the minima of C equal column
// blocks, each block holding a value <= it.  A block without a number (all
// NaN) or holding +inf gives +inf, i.e. no bound.
template <int C>
__device__ __forceinline__ float cth_bound(const uint32_t (&r0)[32], const uint32_t (&r1)[32],
                                           const uint32_t (&r2)[32], const uint32_t (&r3)[32]) {
  constexpr int BS = 128 / C;  // block width in columns, a multiple of 8
  float B = -INFINITY, run = INFINITY;
  auto chunk = [&](const uint32_t (&r)[32], int c) {
#pragma unroll
    for (int g = 0; g < 4; g++) {
      const uint32_t *x = r + 8 * g;
      run = fminf(run, fmin3(fmin3(__uint_as_float(x[0]), __uint_as_float(x[1]),
                                   __uint_as_float(x[2])),
                             fmin3(__uint_as_float(x[3]), __uint_as_float(x[4]),
                                   __uint_as_float(x[5])),
                             fminf(__uint_as_float(x[6]), __uint_as_float(x[7]))));
      if ((c * 32 + 8 * g + 8) % BS == 0) {
        B = fmaxf(B, run);
        run = INFINITY;
      }
    }
  };
  chunk(r0, 0);
  chunk(r1, 1);
  chunk(r2, 2);
  chunk(r3, 3);
  return B;
}

// checked x < L[C-1].  Equal values keep their earlier (smaller) ids first.
template <int C>
__device__ __forceinline__ void reg_insert(float (&L)[C], int (&I)[C], float x, int j) {
  int p = 0;
#pragma unroll
  for (int s = 0; s < C; s++) p += (L[s] <= x);
#pragma unroll
  for (int s = C - 1; s >= 0; s--) {
    const float lv = (s > 0) ? L[s - 1] : 0.f;
    const int li = (s > 0) ? I[s - 1] : 0;
    const bool shift = s > p;
    const bool here = s == p;
    L[s] = shift ? lv : (here ? x : L[s]);
    I[s] = shift ? li : (here ? j : I[s]);
  }
}

template <int MODE, int C, bool L2, bool QS, bool PAIR>
__global__ void __launch_bounds__(NT_TC, 1)
    tc_scan_kernel(const __grid_constant__ CUtensorMap mapQ,
                   const __grid_constant__ CUtensorMap mapQn,
                   const __grid_constant__ CUtensorMap mapB,
                   const __grid_constant__ CUtensorMap mapBn, int nq, int nb, int nkb,
                   int S, ScanSel sel, int *err) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  // aligned by pointer arithmetic on smem_raw (not through an integer), so
  // that the compiler keeps these pointers in the shared address space
  uint8_t *base = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
  const Layout lay = make_layout(nkb, S, MODE, C, QS, PAIR);
  const size_t SB = lay.stage_bytes;
  constexpr int BHALF = PAIR ? STAGE_BYTES / 2 : STAGE_BYTES;  // base bytes per stage, this CTA
  constexpr int BNHALF = PAIR ? BN_BYTES / 2 : BN_BYTES;
  uint8_t *Qs = base + lay.q_off;
  uint8_t *Qn = base + lay.qn_off;
  uint8_t *Stg = base + lay.stg_off;
  float *Lv = reinterpret_cast<float *>(base + lay.list_off);
  uint64_t *bars = reinterpret_cast<uint64_t *>(base + lay.bar_off);
  uint64_t *full = bars, *empty = bars + S, *tfull = bars + 2 * S, *tempty = bars + 2 * S + 2;
  uint64_t *qfull = bars + 2 * S + 4;
  uint64_t *qempty = bars + 2 * S + 5;  // resident query tile released (grouped)
  uint32_t *tmem_holder = reinterpret_cast<uint32_t *>(bars + 2 * S + 6);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_holder + 1);
  uint64_t *mdone = bars + 2 * S + 7;  // the MMAs issued have finished (exit)
  const uint64_t wl = sel.wait_ns ? (uint64_t)sel.wait_ns : kWaitLimitNs;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ntb = (int)ceil_div(nb, TC_TILE_N);
  const int nks = nkb;  // stages per base tile (the norm block rides with the last)
  // Work units are (query tile, chunk of base tiles).  With streamed queries a
  // CTA keeps no per-unit state in shared memory, so single CTAs run a 1D
  // persistent grid that walks the units with stride gridDim.x (ring position,
  // accumulator buffer and barrier phases carry over from unit to unit); else
  // one unit per CTA from the 2D grid (query tile, chunk).
  // A grouped pass (sel.units) takes its units from the table: query rows and
  // valid columns end at the unit's pair, and ids are relative to its base.
  // A grouped pass with a resident query tile is persistent too: the tile is
  // reloaded per unit once the previous unit's MMAs have released it (qempty).
  const bool grouped = !PAIR && sel.units != nullptr;
  const bool PERSIST = !PAIR && (QS || grouped);
  const int nqt = (int)ceil_div(nq, TC_TILE_M);
  const int nunits = grouped ? sel.nunits : PERSIST ? nqt * sel.nchunk : 1;
  const int w0 = PERSIST ? (int)blockIdx.x : 0, wstep = PERSIST ? (int)gridDim.x : 1;
  struct UnitInfo {
    long q0, qend;
    int t_begin, t_end, bend, chunk, pair;
  };
  auto unit_info = [&](int w) -> UnitInfo {
    UnitInfo u;
    if (grouped) {
      const GroupUnit g = sel.units[w];
      u.q0 = g.q0; u.qend = g.qend; u.t_begin = g.t_begin; u.t_end = g.t_end;
      u.bend = g.bend; u.chunk = g.chunk; u.pair = g.pair;
      return u;
    }
    u.q0 = PERSIST ? (long)(w % nqt) * TC_TILE_M : (long)blockIdx.x * TC_TILE_M;
    u.qend = nq;
    u.chunk = PERSIST ? w / nqt : (int)blockIdx.y;
    u.t_begin = u.chunk * sel.tiles_per_chunk;
    u.t_end = imin(ntb, u.t_begin + sel.tiles_per_chunk);
    u.bend = nb;
    u.pair = -1;
    return u;
  };
  const uint32_t crank = PAIR ? cluster_ctarank() : 0;
  const bool leader = crank == 0;

  if (threadIdx.x == 0) {
    for (int s = 0; s < S; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int a = 0; a < 2; a++) {
      mbar_init(&tfull[a], 1);
      // the leader's MMA waits for the selection warps of both CTAs
      mbar_init(&tempty[a], (PAIR ? 2 : 1) * (N_EPI / 32));
    }
    mbar_init(qfull, 1);
    mbar_init(qempty, 1);
    mbar_init(mdone, 1);
    *abort_flag = 0;
    fence_mbar_init();
  }
  if (warp == 1) {
    if (PAIR) {
      tmem_alloc_pair(tmem_holder, TMEM_COLS);
      tmem_relinquish_pair();
    } else {
      tmem_alloc(tmem_holder, TMEM_COLS);
      tmem_relinquish();
    }
  }
  tc_fence_before();
  __syncthreads();
  if (PAIR) cluster_sync();  // both CTAs' barriers exist before any remote signal
  tc_fence_after();
  const uint32_t tmem = *tmem_holder;
  // barriers of the leader, as shared::cluster addresses (PAIR)
  const uint32_t full_l = PAIR ? mapa_shared(smem_u32(full), 0) : 0;
  const uint32_t qfull_l = PAIR ? mapa_shared(smem_u32(qfull), 0) : 0;
  const uint32_t tempty_l = PAIR ? mapa_shared(smem_u32(tempty), 0) : 0;

  if (warp == 0) {
    // ---------------- TMA producer (every CTA loads its own query tile and
    // its part of each base block)
    if (lane == 0 && !(sel.withhold && !PAIR)) {
      // ring position: stage sn, phase parity phn (advanced at every use)
      int sn = 0;
      uint32_t phn = 0;
      bool ok = true;
      int ui = 0;  // units done by this CTA
      uint32_t issued = 0, last_par = 0;  // per stage: loaded at least once, last parity
      int qloads = 0;
      for (int w = w0; w < nunits && ok; w += wstep, ui++) {
      const UnitInfo un = unit_info(w);
      const long q0 = un.q0;
      if (!QS) {
        // the resident tile of the previous unit is free once its MMAs are done
        if (ui > 0 && !mbar_wait(qempty, (uint32_t)((ui - 1) & 1), abort_flag, wl)) {
          ok = false;
          break;
        }
        const uint32_t qbytes = (uint32_t)(nkb * QBLK_BYTES + (L2 ? 128 * 32 : 0));
        if (PAIR) {
          if (leader) mbar_arrive_expect_tx(qfull, 2 * qbytes);
          for (int kb = 0; kb < nkb; kb++)
            tma_load_2d_pair(&mapQ, qfull_l, Qs + kb * QBLK_BYTES, kb * 64, (int)q0);
          if (L2) tma_load_2d_pair(&mapQn, qfull_l, Qn, 0, (int)q0);
        } else {
          mbar_arrive_expect_tx(qfull, qbytes);
          for (int kb = 0; kb < nkb; kb++)
            tma_load_2d(&mapQ, qfull, Qs + kb * QBLK_BYTES, kb * 64, (int)q0);
          if (L2) tma_load_2d(&mapQn, qfull, Qn, 0, (int)q0);
        }
        qloads++;
      }
      for (int t = un.t_begin; t < un.t_end && ok; t++) {
        const int brow = t * TC_TILE_N + (int)crank * (TC_TILE_N / 2) * (PAIR ? 1 : 0);
        for (int ks = 0; ks < nks; ks++) {
          const int s = sn;
          const uint32_t ph = phn;
          if (++sn == S) { sn = 0; phn ^= 1; }
          if (!mbar_wait(&empty[s], ph ^ 1, abort_flag, wl)) { ok = false; break; }
          uint8_t *sp = Stg + (size_t)s * SB;
          const bool lastk = L2 && ks == nkb - 1;
          const uint32_t tx = (uint32_t)(BHALF + (QS ? QBLK_BYTES : 0)) +
                              (lastk ? (uint32_t)(BNHALF + (QS ? 128 * 32 : 0)) : 0u);
          // the norm blocks travel with the last K block (base norms first,
          // then, when streamed, the query norms BN_BYTES further)
          uint8_t *np_ = sp + BHALF + (QS ? QBLK_BYTES : 0);
          if (PAIR) {
            const uint32_t fb = full_l + (uint32_t)(s * 8);
            if (leader) mbar_arrive_expect_tx(&full[s], 2 * tx);
            tma_load_2d_pair(&mapB, fb, sp, ks * 64, brow);
            if (QS) tma_load_2d_pair(&mapQ, fb, sp + BHALF, ks * 64, (int)q0);
            if (lastk) {
              tma_load_2d_pair(&mapBn, fb, np_, 0, brow);
              if (QS) tma_load_2d_pair(&mapQn, fb, np_ + BN_BYTES, 0, (int)q0);
            }
          } else {
            mbar_arrive_expect_tx(&full[s], tx);
            tma_load_2d(&mapB, &full[s], sp, ks * 64, brow);
            if (QS) tma_load_2d(&mapQ, &full[s], sp + BHALF, ks * 64, (int)q0);
            if (lastk) {
              tma_load_2d(&mapBn, &full[s], np_, 0, brow);
              if (QS) tma_load_2d(&mapQn, &full[s], np_ + BN_BYTES, 0, (int)q0);
            }
            issued |= 1u << s;
            last_par = (last_par & ~(1u << s)) | (ph << s);
          }
        }
      }
      }
      // the last unit's tile release has landed before the CTA exits
      if (!QS && PERSIST && ok && ui > 0) ok = mbar_wait(qempty, (uint32_t)((ui - 1) & 1), abort_flag, wl);
      if (!PAIR) {
        // every copy this CTA issued has landed before its shared memory is
        // released (immediate unless a bounded wait gave up)
        for (int s = 0; s < S; s++)
          if (issued >> s & 1) mbar_wait_drain(&full[s], last_par >> s & 1);
        if (qloads > 0) mbar_wait_drain(qfull, (uint32_t)((qloads - 1) & 1));
      }
      if (PAIR) {
        // every stage released by the leader's MMAs: no commit is still on its
        // way to this CTA when the pair exits
        for (int e = 0; e < S && ok; e++) {
          const int s = sn;
          const uint32_t ph = phn;
          if (++sn == S) { sn = 0; phn ^= 1; }
          if (!mbar_wait(&empty[s], ph ^ 1, abort_flag, wl)) ok = false;
        }
      }
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer (the leader's, for a pair)
    if (lane == 0 && leader) {
      const uint32_t idesc = idesc_16_f32(PAIR ? 2 * TC_TILE_M : TC_TILE_M, TC_TILE_N, sel.f16 != 0);
      bool ok = true, any = false;
      int sn = 0;
      uint32_t phn = 0;
      int it = 0, ui = 0;
      for (int w = w0; w < nunits && ok; w += wstep, ui++) {
      const UnitInfo un = unit_info(w);
      if (!QS) {
        if (!mbar_wait(qfull, (uint32_t)(ui & 1), abort_flag, wl)) { ok = false; break; }
        tc_fence_after();
      }
      for (int t = un.t_begin; t < un.t_end && ok; t++, it++) {
        const int a = it & 1;
        const uint32_t u = (uint32_t)(it >> 1);
        if (!mbar_wait(&tempty[a], (u & 1) ^ 1, abort_flag, wl)) { ok = false; break; }
        tc_fence_after();
        const uint32_t dt = tmem + (uint32_t)(a * TC_TILE_N);
        for (int ks = 0; ks < nks; ks++) {
          const int s = sn;
          const uint32_t ph = phn;
          if (++sn == S) { sn = 0; phn ^= 1; }
          // TMA data: its arrival is tracked by the barrier's transaction
          // count, no tcgen05 fence is needed (a fence here would stall the
          // MMA pipe once per stage)
          if (!mbar_wait(&full[s], ph, abort_flag, wl)) { ok = false; break; }
          const uint32_t sb = smem_u32(Stg + (size_t)s * SB);
          // a descriptor's start address field is addr >> 4 in its low 14 bits
          // (shared addresses < 256 KB): offsets are added to a base descriptor
          {
            const uint32_t sa = QS ? sb + BHALF : smem_u32(Qs + ks * QBLK_BYTES);
            const uint64_t da = desc_k_sw128(sa), db = desc_k_sw128(sb);
#pragma unroll
            for (int kk = 0; kk < 4; kk++) {
              const uint32_t acc = (ks > 0 || kk > 0) ? 1u : 0u;
              if (PAIR)
                umma_bf16_pair(dt, da + (uint64_t)(kk * 2), db + (uint64_t)(kk * 2), idesc, acc);
              else
                umma_bf16(dt, da + (uint64_t)(kk * 2), db + (uint64_t)(kk * 2), idesc, acc);
            }
            if (L2 && ks == nkb - 1) {  // the norm fold: one more K=16 step
              const uint32_t sn_ = sb + BHALF + (QS ? QBLK_BYTES : 0);
              const uint64_t dq = desc_k_sw32(QS ? sn_ + BN_BYTES : smem_u32(Qn));
              const uint64_t dbn = desc_k_sw32(sn_);
              if (PAIR)
                umma_bf16_pair(dt, dq, dbn, idesc, 1u);
              else
                umma_bf16(dt, dq, dbn, idesc, 1u);
            }
          }
          any = true;
          if (PAIR)
            umma_commit_pair_mc(&empty[s], 3);
          else
            umma_commit(&empty[s]);
        }
        if (!ok) break;
        if (PAIR)
          umma_commit_pair_mc(&tfull[a], 3);
        else
          umma_commit(&tfull[a]);
      }
      // release the resident query tile once this unit's MMAs are done
      if (!QS && PERSIST && ok) umma_commit(qempty);
      }
      if (!PAIR && any) {
        // every MMA issued has finished with TMEM and shared memory
        umma_commit(mdone);
        mbar_wait_drain(mdone, 0);
      }
      if (PAIR) {
        // the last two accumulators released by the selection warps of both
        // CTAs: no remote arrival is still on its way when the pair exits
        for (int e = it; e < it + 2 && ok; e++) {
          const int a = e & 1;
          const uint32_t u = (uint32_t)(e >> 1);
          if (!mbar_wait(&tempty[a], (u & 1) ^ 1, abort_flag, wl)) ok = false;
        }
      }
    }
  } else {
    // ---------------- selection warps
    const int ew = warp - 2;               // 0..7
    const int grp = warp & 3;              // TMEM lane group this warp may access
    const int half = ew >> 2;              // column half
    const int row = grp * 32 + lane;
    const int tslot = ew * 32 + lane;      // 0..255
    const uint32_t lane_base = (uint32_t)(grp * 32) << 16;
    int it = 0;
    bool ok = true;
    for (int w = w0; w < nunits && ok; w += wstep) {
    const UnitInfo un = unit_info(w);
    const long qrow = un.q0 + row;
    const int chunk = un.chunk;
    const int t_begin = un.t_begin, t_end = un.t_end;
    const int nbv = un.bend;  // columns at or past nbv are not the unit's
    const bool rvalid = qrow < un.qend;
    float lmax = INFINITY, thr = NAN;
    constexpr int CR = (C <= 16) ? C : 1;  // register lists up to 16 entries
    float RL[CR];
    int RI[CR];
#pragma unroll
    for (int s = 0; s < CR; s++) { RL[s] = INFINITY; RI[s] = 0x7fffffff; }
    int *Li = reinterpret_cast<int *>(Lv + (MODE != SCAN_THRESH && C > 16 ? N_EPI * C : 0));
    if (MODE != SCAN_THRESH && C > 16) {
      for (int s = 0; s < C; s++) { Lv[s * N_EPI + tslot] = INFINITY; Li[s * N_EPI + tslot] = 0x7fffffff; }
    }
    if (MODE == SCAN_THRESH && rvalid) thr = sel.thr[qrow];
    int rcount = 0;  // THRESH: hits of this thread's region (chunk, half, query)
    float tb = INFINITY;  // lists: bound of the current half tile's C-th smallest
    // THRESH region of this thread: counter index and first slot
    long rbase = (long)(chunk * 2 + half) * nq + qrow, cbase;
    int cap = sel.cap, id_off = sel.id_off;
    if (grouped && MODE == SCAN_THRESH) {
      const GroupPair &gp = sel.gpairs[un.pair];
      const long rl = (long)(chunk * 2 + half) * gp.nq + (qrow - gp.qoff);
      rbase = gp.cnt_off + rl;
      cbase = gp.cand_off + rl * gp.cap;
      cap = gp.cap;
      id_off = -gp.boff;
    } else {
      cbase = rbase * cap;
    }

    // per-element update of one value (the rare path)
    auto update = [&](float x, int j) {
      if (MODE == SCAN_TOPV) {
        if (x < lmax) {  // min/max bubble, values only
#pragma unroll
          for (int z = 0; z < CR; z++) {
            const float lo = fminf(RL[z], x);
            x = fmaxf(RL[z], x);
            RL[z] = lo;
          }
          lmax = RL[CR - 1];
        }
      } else if (MODE == SCAN_TOPC) {
        if (x < lmax) {
          if (C <= 16) {
            reg_insert<CR>(RL, RI, x, j);
            lmax = RL[CR - 1];
          } else {
            int p = C - 1;
            while (p > 0 && Lv[(p - 1) * N_EPI + tslot] > x) {
              Lv[p * N_EPI + tslot] = Lv[(p - 1) * N_EPI + tslot];
              Li[p * N_EPI + tslot] = Li[(p - 1) * N_EPI + tslot];
              p--;
            }
            Lv[p * N_EPI + tslot] = x;
            Li[p * N_EPI + tslot] = j;
            lmax = Lv[(C - 1) * N_EPI + tslot];
          }
        }
      } else {
        if (x <= thr) {
          if (rcount < cap) {
            sel.candv[cbase + rcount] = x;
            sel.candi[cbase + rcount] = j + id_off;
          }
          rcount++;
        }
      }
    };

    // One 32-column chunk already in registers.  The loop body must stay small
    // (the selection warps run it from the instruction cache): a min tree and
    // one warp vote per chunk; only when some lane's chunk minimum passes its
    // bound (true when min < bound or min is NaN) does the warp build each
    // lane's hit mask and walk its hits, extracting each value with a select
    // tree instead of unrolled per-element code.
    auto process = [&](const uint32_t (&r)[32], int jc) {
      float v[32];
#pragma unroll
      for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
      if (jc + 32 > nbv) {
#pragma unroll
        for (int i = 0; i < 32; i++)
          if (jc + i >= nbv) v[i] = NAN;
      }
      float m8[4];
#pragma unroll
      for (int g = 0; g < 4; g++)
        m8[g] = fmin3(fmin3(v[8 * g], v[8 * g + 1], v[8 * g + 2]),
                      fmin3(v[8 * g + 3], v[8 * g + 4], v[8 * g + 5]),
                      fminf(v[8 * g + 6], v[8 * g + 7]));
      const float mc = fminf(fminf(m8[0], m8[1]), fminf(m8[2], m8[3]));
      // lists: a superset filter (update() keeps the strict x < lmax)
      const float bnd = MODE == SCAN_THRESH ? thr : fminf(lmax, tb);
      const bool pass = rvalid && !(mc > bnd);
      if (!__any_sync(0xffffffffu, pass)) return;
      if (!pass) return;
      uint32_t bits = 0;
#pragma unroll
      for (int i = 0; i < 32; i++) {
        bits |= !(v[i] > bnd) ? (1u << i) : 0u;
      }
#pragma unroll 1
      while (bits) {
        const int i = __ffs(bits) - 1;
        bits &= bits - 1;
        float t16[16], t8[8], t4[4], t2[2];
#pragma unroll
        for (int z = 0; z < 16; z++) t16[z] = (i & 1) ? v[2 * z + 1] : v[2 * z];
#pragma unroll
        for (int z = 0; z < 8; z++) t8[z] = (i & 2) ? t16[2 * z + 1] : t16[2 * z];
#pragma unroll
        for (int z = 0; z < 4; z++) t4[z] = (i & 4) ? t8[2 * z + 1] : t8[2 * z];
#pragma unroll
        for (int z = 0; z < 2; z++) t2[z] = (i & 8) ? t4[2 * z + 1] : t4[2 * z];
        update((i & 16) ? t2[1] : t2[0], jc + i);
      }
    };

    for (int t = t_begin; t < t_end; t++, it++) {
      const int a = it & 1;
      const uint32_t u = (uint32_t)(it >> 1);
      ok = mbar_wait(&tfull[a], u & 1, abort_flag, wl);
      __syncwarp();
      if (!__all_sync(0xffffffffu, ok)) { ok = false; break; }
      tc_fence_after();
      const uint32_t tcol = tmem + lane_base + (uint32_t)(a * TC_TILE_N + half * 128);
      const int j0 = t * TC_TILE_N + half * 128;
      // two register sets: the load of chunk c+1 is in flight while chunk c is
      // scanned; the loop keeps one copy of the chunk code per register set
      uint32_t r0[32], r1[32], r2[32], r3[32];
      tmem_ld32(tcol, r0);
      tmem_ld32(tcol + 32, r1);
      tmem_ld32(tcol + 64, r2);
      tmem_ld32(tcol + 96, r3);
      tmem_ld_wait(r0);
      tmem_ld_wait(r1);
      tmem_ld_wait(r2);
      tmem_ld_wait(r3);
      tc_fence_before();
      __syncwarp();
      if (lane == 0) {
        if (PAIR)
          mbar_arrive_cluster(tempty_l + (uint32_t)(a * 8));
        else
          mbar_arrive(&tempty[a]);
      }
      // first tile of a unit: the lists are empty and every value would be a
      // hit; a bound of this half tile's C-th smallest filters them instead
      if (MODE != SCAN_THRESH && C <= 16) {
        tb = INFINITY;
        if (t == t_begin && j0 + 128 <= nbv) tb = cth_bound<C>(r0, r1, r2, r3);
      }
      process(r0, j0);
      process(r1, j0 + 32);
      process(r2, j0 + 64);
      process(r3, j0 + 96);
    }
    // a failed wait ends this unit's scan; the merge below still runs, so that
    // every selection warp reaches each named barrier
    if (MODE == SCAN_THRESH && rvalid) sel.cnt[rbase] = rcount;
    if (MODE != SCAN_THRESH) {
      // merge the two column halves of each row
      int *Xi = reinterpret_cast<int *>(Lv + 128 * C);
      if (C <= 16 && half == 1) {
#pragma unroll
        for (int s = 0; s < CR; s++) { Lv[row * C + s] = RL[s]; Xi[row * C + s] = RI[s]; }
      }
      asm volatile("bar.sync 1, 256;" ::: "memory");
      if (half == 0 && rvalid) {
        const long o = ((long)chunk * nq + qrow) * C;
        int ia = 0, ib = 0;
        for (int s = 0; s < C; s++) {
          float va, vb;
          int xa, xb;
          if (C <= 16) {
            va = INFINITY; xa = 0x7fffffff;
#pragma unroll
            for (int z = 0; z < CR; z++) if (z == ia) { va = RL[z]; xa = RI[z]; }
            vb = ib < C ? Lv[row * C + ib] : INFINITY;
            xb = ib < C ? Xi[row * C + ib] : 0x7fffffff;
          } else {
            const int pt = tslot + 128;
            va = ia < C ? Lv[ia * N_EPI + tslot] : INFINITY;
            xa = ia < C ? Li[ia * N_EPI + tslot] : 0x7fffffff;
            vb = ib < C ? Lv[ib * N_EPI + pt] : INFINITY;
            xb = ib < C ? Li[ib * N_EPI + pt] : 0x7fffffff;
          }
          const bool takeA = ia < C && (ib >= C || va < vb || (va == vb && xa <= xb));
          const float vo = takeA ? va : vb;
          const int xo = takeA ? xa : xb;
          sel.topv[o + s] = vo;
          sel.topi[o + s] = (xo == 0x7fffffff) ? -1 : xo + id_off;
          if (takeA) ia++; else ib++;
        }
      }
    }
    // the next unit's half 1 rewrites the rows only after they are merged, and
    // all selection warps leave the unit loop together (any failed wait ends it)
    if (PERSIST) ok = bar_red_and_256(ok);
    }
  }

  tc_fence_before();
  __syncthreads();
  if (PAIR) cluster_sync();  // no peer signal is still on its way
  tc_fence_after();
  if (warp == 1) {
    __syncwarp();
    if (PAIR)
      tmem_dealloc_pair(tmem, TMEM_COLS);
    else
      tmem_dealloc(tmem, TMEM_COLS);
  }
  if (PAIR) cluster_sync();  // the pair's collective free is done before either CTA exits
  if (threadIdx.x == 0 && *abort_flag && err) atomicExch(err, 1);
}

// ---------------- host side

static PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

static int get_encode() {
  if (g_encode) return OK;
  void *fn = nullptr;
  cudaDriverEntryPointQueryResult qr;
  cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000,
                                                   cudaEnableDefault, &qr);
  if (e != cudaSuccess || qr != cudaDriverEntryPointSuccess || !fn) {
    set_error(E_CUDA, "cuTensorMapEncodeTiled unavailable (%s)", cudaGetErrorString(e));
    return E_CUDA;
  }
  g_encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
  return OK;
}

static int make_map(CUtensorMap *m, const void *ptr, uint64_t cols, uint64_t rows,
             uint64_t row_bytes, uint32_t box_cols, uint32_t box_rows,
             CUtensorMapSwizzle sw) {
  YG_CHECK(get_encode());
  if (!ptr || (reinterpret_cast<uintptr_t>(ptr) & 15) || (row_bytes & 15) || rows == 0) {
    set_error(E_ARG, "tensor map: null / misaligned operand (ptr=%p pitch=%llu rows=%llu)", ptr,
              (unsigned long long)row_bytes, (unsigned long long)rows);
    return E_ARG;
  }
  cuuint64_t dims[2] = {cols, rows};
  cuuint64_t strides[1] = {row_bytes};
  cuuint32_t box[2] = {box_cols, box_rows};
  cuuint32_t es[2] = {1, 1};
  CUresult r = g_encode(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(ptr), dims,
                        strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, sw,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error(E_CUDA, "cuTensorMapEncodeTiled failed (%d): cols=%llu rows=%llu pitch=%llu",
              (int)r, (unsigned long long)cols, (unsigned long long)rows,
              (unsigned long long)row_bytes);
    return E_CUDA;
  }
  return OK;
}

template <int MODE, int C, bool L2, bool QS, bool PAIR>
int launch(const TcOperands &op, int nq, int nb, const ScanSel &sel, cudaStream_t st) {
  const int nkb = op.Kp / 64;
  int S = 12;
  while (S > 2 && make_layout(nkb, S, MODE, C, QS, PAIR).total > 227 * 1024) S--;
  const Layout lay = make_layout(nkb, S, MODE, C, QS, PAIR);
  if (!QS && lay.q_off + (size_t)nkb * QBLK_BYTES > 227 * 1024) {
    set_error(E_UNSUPPORTED, "tc_scan: resident query tile too large (Kp=%d)", op.Kp);
    return E_UNSUPPORTED;
  }
  if (lay.total > 227 * 1024) {
    set_error(E_UNSUPPORTED, "tc_scan: shared memory %zu too large (Kp=%d C=%d)", lay.total,
              op.Kp, C);
    return E_UNSUPPORTED;
  }
  YG_CHECK(ensure_smem((const void *)tc_scan_kernel<MODE, C, L2, QS, PAIR>, lay.total));
  CUtensorMap mq, mqn, mb, mbn;
  YG_CHECK(make_map(&mq, op.q, op.Kp, nq, (uint64_t)op.Kp * 2, 64, 128,
                    CU_TENSOR_MAP_SWIZZLE_128B));
  // a pair CTA loads 128 of the 256 rows of each base block
  const uint32_t brows = PAIR ? TC_TILE_N / 2 : TC_TILE_N;
  YG_CHECK(make_map(&mb, op.b, op.Kp, nb, (uint64_t)op.Kp * 2 * op.b_step, 64, brows,
                    CU_TENSOR_MAP_SWIZZLE_128B));
  if (L2) {
    YG_CHECK(make_map(&mqn, op.qn, 16, nq, 32, 16, 128, CU_TENSOR_MAP_SWIZZLE_32B));
    YG_CHECK(make_map(&mbn, op.bn, 16, nb, (uint64_t)32 * op.b_step, 16, brows,
                      CU_TENSOR_MAP_SWIZZLE_32B));
  } else {
    mqn = mq;
    mbn = mb;
  }
  if (!PAIR && (QS || sel.units)) {
    // persistent: one CTA per SM (the ring fills shared memory), units strided
    int dev = 0, nsm = 0;
    YG_CUDA(cudaGetDevice(&dev));
    YG_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    const long nunits = sel.units ? (long)sel.nunits : ceil_div(nq, TC_TILE_M) * (long)sel.nchunk;
    if (nunits > INT_MAX) {
      set_error(E_UNSUPPORTED, "tc_scan: %ld work units", nunits);
      return E_UNSUPPORTED;
    }
    if (sel.max_ctas > 0 && sel.max_ctas < nsm) nsm = sel.max_ctas;
    const unsigned g = (unsigned)(nunits < nsm ? nunits : nsm);
    tc_scan_kernel<MODE, C, L2, QS, PAIR><<<g, NT_TC, lay.total, st>>>(mq, mqn, mb, mbn, nq, nb,
                                                                        nkb, S, sel, op.err);
  } else if (!PAIR) {
    dim3 grid((unsigned)ceil_div(nq, TC_TILE_M), (unsigned)sel.nchunk);
    tc_scan_kernel<MODE, C, L2, QS, PAIR><<<grid, NT_TC, lay.total, st>>>(
        mq, mqn, mb, mbn, nq, nb, nkb, S, sel, op.err);
  } else {
    // query tiles padded to whole pairs (a padding CTA has no valid rows)
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(ceil_div(ceil_div(nq, TC_TILE_M), 2) * 2), (unsigned)sel.nchunk);
    cfg.blockDim = dim3(NT_TC);
    cfg.dynamicSmemBytes = lay.total;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = 2;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    YG_CUDA(cudaLaunchKernelEx(&cfg, tc_scan_kernel<MODE, C, L2, QS, PAIR>, mq, mqn, mb, mbn, nq,
                               nb, nkb, S, sel, op.err));
  }
  YG_LAUNCH_CHECK();
  return OK;
}

template <bool L2, bool QS, bool PAIR>
int dispatch(const TcOperands &op, int nq, int nb, const ScanSel &sel, cudaStream_t st) {
  if (sel.mode == SCAN_THRESH) return launch<SCAN_THRESH, 1, L2, QS, PAIR>(op, nq, nb, sel, st);
  switch (sel.C) {
    case 1: return launch<SCAN_TOPC, 1, L2, QS, PAIR>(op, nq, nb, sel, st);
    case 2: return launch<SCAN_TOPC, 2, L2, QS, PAIR>(op, nq, nb, sel, st);
    case 4: return launch<SCAN_TOPC, 4, L2, QS, PAIR>(op, nq, nb, sel, st);
    case 8: return launch<SCAN_TOPC, 8, L2, QS, PAIR>(op, nq, nb, sel, st);
    case 16:
      if (sel.mode == SCAN_TOPV) return launch<SCAN_TOPV, 16, L2, QS, PAIR>(op, nq, nb, sel, st);
      return launch<SCAN_TOPC, 16, L2, QS, PAIR>(op, nq, nb, sel, st);
  }
  set_error(E_ARG, "tc_scan: unsupported list length C=%d", sel.C);
  return E_ARG;
}

// one instantiation per translation unit (they compile in parallel)
template <bool QS, bool PAIR>
int dispatch_metric(const TcOperands &op, int nq, int nb, const ScanSel &sel, cudaStream_t st) {
  if (op.metric == METRIC_L2) return dispatch<true, QS, PAIR>(op, nq, nb, sel, st);
  return dispatch<false, QS, PAIR>(op, nq, nb, sel, st);
}

}  // namespace tck

// the four instantiations: query tile resident (r) or streamed (s), single
// CTAs (1) or CTA pairs (2)
int tc_dispatch_r1(const TcOperands &op, int nq, int nb, const ScanSel &sel, cudaStream_t st);
int tc_dispatch_r2(const TcOperands &op, int nq, int nb, const ScanSel &sel, cudaStream_t st);
int tc_dispatch_s1(const TcOperands &op, int nq, int nb, const ScanSel &sel, cudaStream_t st);
int tc_dispatch_s2(const TcOperands &op, int nq, int nb, const ScanSel &sel, cudaStream_t st);

}  // namespace yg
