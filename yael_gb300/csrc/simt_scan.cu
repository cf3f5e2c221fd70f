// FP32 CUDA-core distance tiles with fused per-query selection (the plain
// drop-in path).  128 queries x 128 base rows per tile, 256 threads, 8x8 FFMA
// micro-tiles; the finished tile is staged in shared memory so that each query
// row is scanned by two threads in increasing base order (see scan.cuh for the
// selection contract).
#include <math.h>

#include "scan.cuh"
#include "simt_tile.cuh"

namespace yg {

namespace {
using namespace simt;

template <int MODE, int C>
__global__ void __launch_bounds__(NT, 1)
    simt_scan_kernel(const float *__restrict__ Q, long ldq, int nq,
                     const float *__restrict__ B, long ldb, int nb, int d,
                     const float *__restrict__ bn, long bn_stride, int metric,
                     ScanSel sel) {
  extern __shared__ __align__(16) float smem[];
  float *St = smem + kOperandFloats;          // [BM][ST_LD]
  float *Lv = St + BM * ST_LD;                // [C][NT]  (TOPC)
  int *Li = reinterpret_cast<int *>(Lv + (MODE == SCAN_TOPC ? C * NT : 0));

  const int tid = threadIdx.x;
  const long q0 = (long)blockIdx.x * BM;
  const int ntb = (int)ceil_div(nb, BN);
  const int t_begin = blockIdx.y * sel.tiles_per_chunk;
  const int t_end = imin(ntb, t_begin + sel.tiles_per_chunk);

  // selection role: row sr, column half sh
  const int sr = tid & (BM - 1), sh = tid >> 7;
  const long qrow = q0 + sr;
  float lmax = INFINITY, thr = NAN;
  int rcount = 0;  // THRESH: hits of this thread's region
  const long rbase = ((long)(blockIdx.y * 2 + sh) * nq + qrow);
  if (MODE == SCAN_TOPC) {
#pragma unroll
    for (int s = 0; s < C; s++) {
      Lv[s * NT + tid] = INFINITY;
      Li[s * NT + tid] = -1;
    }
  } else {
    if (qrow < nq) thr = sel.thr[qrow];
  }
  const int tx = tid & 15, ty = tid >> 4;

  for (int t = t_begin; t < t_end; ++t) {
    const long j0 = (long)t * BN;
    float acc[8][8];
    tile_mainloop(Q, ldq, nq, q0, B, ldb, nb, j0, d, smem, acc);

    // epilogue: v = ||b||^2 - 2 q.b (or q.b) into the staging tile
#pragma unroll
    for (int j = 0; j < 8; j++) {
      const int col = col_of(j, tx);
      const long jg = j0 + col;
      const bool ok = jg < nb;
      const float bnj = (ok && metric == METRIC_L2) ? __ldg(bn + jg * bn_stride) : 0.f;
#pragma unroll
      for (int i = 0; i < 8; i++) {
        const int row = row_of(i, ty);
        const float v = metric == METRIC_L2 ? fmaf(-2.f, acc[i][j], bnj) : acc[i][j];
        St[row * ST_LD + col] = ok ? v : NAN;
      }
    }
    __syncthreads();

    // selection: row sr, columns [sh*64, sh*64+64), increasing base index
    if (qrow < nq) {
      const float *srow = St + sr * ST_LD + sh * 64;
      const int jbase = (int)(j0 + sh * 64);
      for (int c = 0; c < 64; c++) {
        const float v = srow[c];
        if (MODE == SCAN_TOPC) {
          if (v < lmax) {
            int p = C - 1;
            while (p > 0 && Lv[(p - 1) * NT + tid] > v) {
              Lv[p * NT + tid] = Lv[(p - 1) * NT + tid];
              Li[p * NT + tid] = Li[(p - 1) * NT + tid];
              p--;
            }
            Lv[p * NT + tid] = v;
            Li[p * NT + tid] = jbase + c;
            lmax = Lv[(C - 1) * NT + tid];
          }
        } else {
          if (v <= thr) {
            if (rcount < sel.cap) {
              sel.candv[rbase * sel.cap + rcount] = v;
              sel.candi[rbase * sel.cap + rcount] = jbase + c + sel.id_off;
            }
            rcount++;
          }
        }
      }
    }
    __syncthreads();  // staging tile is rewritten by the next tile
  }

  if (MODE == SCAN_THRESH && qrow < nq) sel.cnt[rbase] = rcount;
  if (MODE == SCAN_TOPC) {
    if (sh == 0 && qrow < nq) {
      // merge the two half-row lists, lexicographic (v, id)
      int ia = 0, ib = 0;
      const long o = ((long)blockIdx.y * nq + qrow) * C;
      for (int s = 0; s < C; s++) {
        const float va = ia < C ? Lv[ia * NT + tid] : INFINITY;
        const float vb = ib < C ? Lv[ib * NT + tid + 128] : INFINITY;
        const int xa = ia < C ? Li[ia * NT + tid] : -1;
        const int xb = ib < C ? Li[ib * NT + tid + 128] : -1;
        const bool takeA =
            (ia < C) && (ib >= C || va < vb || (va == vb && (unsigned)xa <= (unsigned)xb));
        if (takeA) {
          sel.topv[o + s] = va;
          sel.topi[o + s] = xa < 0 ? xa : xa + sel.id_off;
          ia++;
        } else {
          sel.topv[o + s] = vb;
          sel.topi[o + s] = xb < 0 ? xb : xb + sel.id_off;
          ib++;
        }
      }
    }
  }
}

template <int MODE, int C>
int launch(const float *q, long ldq, int nq, const float *b, long ldb, int nb, int d,
           const float *bn, long bn_stride, int metric, const ScanSel &sel,
           cudaStream_t st) {
  const size_t smem = sizeof(float) * (kOperandFloats + BM * ST_LD) +
                      (MODE == SCAN_TOPC ? (size_t)C * NT * 8 : 0);
  YG_CHECK(ensure_smem((const void *)simt_scan_kernel<MODE, C>, smem));
  dim3 grid((unsigned)ceil_div(nq, BM), (unsigned)sel.nchunk);
  simt_scan_kernel<MODE, C><<<grid, NT, smem, st>>>(q, ldq, nq, b, ldb, nb, d, bn,
                                                     bn_stride, metric, sel);
  YG_LAUNCH_CHECK();
  return OK;
}
}  // namespace

int simt_scan(const float *q, long ldq, int nq, const float *b, long ldb, int nb,
              int d, const float *bn, long bn_stride, int metric, const ScanSel &sel,
              cudaStream_t st) {
  if (nq <= 0 || nb <= 0) return OK;
  // (SCAN_TOPV runs as SCAN_TOPC here: the ids are simply also written)
  if (sel.mode == SCAN_THRESH)
    return launch<SCAN_THRESH, 1>(q, ldq, nq, b, ldb, nb, d, bn, bn_stride, metric, sel, st);
  switch (sel.C) {
    case 1: return launch<SCAN_TOPC, 1>(q, ldq, nq, b, ldb, nb, d, bn, bn_stride, metric, sel, st);
    case 2: return launch<SCAN_TOPC, 2>(q, ldq, nq, b, ldb, nb, d, bn, bn_stride, metric, sel, st);
    case 4: return launch<SCAN_TOPC, 4>(q, ldq, nq, b, ldb, nb, d, bn, bn_stride, metric, sel, st);
    case 8: return launch<SCAN_TOPC, 8>(q, ldq, nq, b, ldb, nb, d, bn, bn_stride, metric, sel, st);
    case 16: return launch<SCAN_TOPC, 16>(q, ldq, nq, b, ldb, nb, d, bn, bn_stride, metric, sel, st);
    case 32: return launch<SCAN_TOPC, 32>(q, ldq, nq, b, ldb, nb, d, bn, bn_stride, metric, sel, st);
  }
  set_error(E_ARG, "simt_scan: unsupported list length C=%d", sel.C);
  return E_ARG;
}

int choose_chunks(int n_query_tiles, int n_base_tiles, int num_sms, int ctas_per_sm,
                  int min_tiles_per_chunk) {
  const int slots = num_sms * ctas_per_sm;
  int maxc = n_base_tiles / imax(1, min_tiles_per_chunk);
  if (maxc < 1) maxc = 1;
  if (n_query_tiles >= 4 * slots) return 1;
  int best = 1;
  double best_eff = -1;
  for (int c = 1; c <= maxc && c <= 4096; c++) {
    const long total = (long)n_query_tiles * c;
    const long waves = (total + slots - 1) / slots;
    const double eff = (double)total / (double)(waves * slots);
    if (total >= slots && eff >= 0.9) return c;
    if (eff > best_eff + 1e-9) {
      best_eff = eff;
      best = c;
    }
    if (total >= 8L * slots) break;
  }
  return best;
}

}  // namespace yg
