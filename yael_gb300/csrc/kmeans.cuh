// Device kernels of the k-means Lloyd step (yael/kmeans.c:213-329), written for
// many independent instances at once (hierarchical k-means runs every child
// clustering of a level together).  Instance i owns points [p0_i, p0_i + n_i)
// of one contiguous point array and centroids [i*k, (i+1)*k) of one centroid
// array; global cluster id = i*k + local id.
#pragma once
#include "common.cuh"
#include "prep.cuh"

namespace yg {

// llrint(x * 2^S) (round to nearest, ties to even) of a float x, with integer
// operations only (the FP64 pipe of this GPU is narrow).  The caller's shift
// keeps |x| 2^S < 2^62; non-finite x gives 0.
__device__ __forceinline__ long long fixed_of(float x, int S) {
  const unsigned u = __float_as_uint(x);
  const int ex = (int)((u >> 23) & 0xffu);
  if (ex == 0xff) return 0;
  unsigned long long m = u & 0x7fffffu;
  int e = -149;  // x = +-m 2^e
  if (ex != 0) {
    m |= 0x800000u;
    e = ex - 150;
  }
  const int sh = e + S;
  unsigned long long r;
  if (sh >= 0) {
    r = m << sh;
  } else if (-sh > 24) {
    r = 0;  // m < 2^24 <= half of the unit in the last place kept
  } else {
    const int rs = -sh;
    const unsigned long long q = m >> rs;
    const unsigned long long rem = m & ((1ull << rs) - 1);
    const unsigned long long half = 1ull << (rs - 1);
    r = q + ((rem > half || (rem == half && (q & 1))) ? 1 : 0);
  }
  return (u >> 31) ? -(long long)r : (long long)r;
}

// fixed_of(x, S) for -126 <= S <= 127, with scale = 2^S (a normal float):
// x * 2^S is then exact (the shift keeps |x| 2^S below 2^62; a product that
// underflows is below 1/2, and both forms give 0 for it), and the conversion
// rounds to nearest even as fixed_of does
__device__ __forceinline__ long long fixed_of_scaled(float x, float scale) {
  if ((__float_as_uint(x) & 0x7f800000u) == 0x7f800000u) return 0;
  return __float2ll_rn(x * scale);
}

struct KmWork {      // one block of the grouped assignment kernel
  int inst;          // instance
  long p0;           // first point (global index)
  int n;             // points in this block (<= kAssignChunk)
};
constexpr int kAssignChunk = 1024;
constexpr int kSmallK = 64;  // largest k of the direct grouped assignment

// assign[p] = local argmin_j ||v_p - C_{inst,j}||^2 (ties to the lowest j),
// dis[p] = that distance.  FP32 direct differences; when the two best are
// closer than their rounding bound all k are recomputed in FP64.  Points with
// a NaN distance everywhere get assign -1, dis 1e30 (yael/nn.c:404-407).
// active[inst] == 0 skips the instance.
int km_assign_small(const KmWork *work, int nwork, const float *v, int d, const float *C,
                    int k, const unsigned char *active, int *assign, float *dis,
                    cudaStream_t st);

// ---- the 16-bit tensor-core assignment for k <= 256 (km_tc.cu) -------------
// A unit is one tile of up to 128 consecutive points of one instance.
struct KmTcUnit {
  int inst;
  int np;   // points in the tile
  long p0;  // first point (global index)
};
constexpr int kTcMaxK = 256;

// The points of a run (or of an hkm level) packed once: 16-bit -2x in
// [n][Kp] with a [n][16] side block of ones (the norm fold), ||x||^2 in FP64
// and the packing's error norm ||x - 16(x)|| per point.
struct KmTcPoints {
  void *pk = nullptr, *side = nullptr;
  double *xn64 = nullptr;
  float *xres = nullptr;
  long n = 0;
  int Kp = 0, f16 = 0;
  // with mu != null every packed row is translated first: the points by
  // their instance's row of mu (mu: ninst x d), the centroids likewise, so
  // the packing errors scale with the spread of an instance, not with its
  // distance from the origin (distances do not change under a translation)
  const float *mu = nullptr;
  // per unit of the unit table, per point of its tile: (||x'|| rounded up,
  // ||x' - 16(x')||), copied with the tile (km_tc_tile_side fills it)
  float2 *tside = nullptr;
};

// tside[w][r] for the unit table (0 past a tile's points)
int km_tc_tile_side(const KmTcUnit *units, int nunits, const double *xn64, const float *xres,
                    float2 *tside, cudaStream_t st);

// shapes the kernel takes: d % 4 == 0, d <= 256, k <= 256, 16-byte aligned rows
bool km_tc_supported(int d, int k, const float *v, const float *C);

// Nearest centroid of every point of the listed units, exact: the tensor
// cores give every centroid's distance within a rigorous bound eps of the
// point (the certificate bound of the k-NN pass); every centroid within 2 eps
// of the smallest is re-evaluated by FP32 direct differences, and by FP64 when
// the best two are closer than their rounding bound (ties to the lowest
// index).  Points whose distances are all NaN get -1 / 1e30.  The centroids
// are packed here (cpk, cside: [ninst*k][Kp] and [ninst*k][16], cstats reset
// and filled; cscratch: 2 x ninst*k floats of norms and packing errors, from
// which ibound[ninst] takes each instance's largest, the bound's terms for
// its points).  With acc != null the exact fixed-point sums of the points and
// the counts are added to acc[g][d] / counts[g] (g = inst*k + j; both zeroed
// by the caller), accumulated in shared memory first when an instance's
// k*d*8 bytes fit (km_tc_fuses), else added to them directly (integer
// atomics: the result does not depend on their order).  With delta != 0 the
// sums and counts already hold the assignment found in `assign` (the previous
// call's): only the points whose centroid changes are subtracted from the old
// one and added to the new one (integer sums: exactly the full sums).  Units
// of instances with active[inst] == 0 are skipped.
bool km_tc_fuses(int d, int k);
int km_tc_assign(const KmTcUnit *units, int nunits, const KmTcPoints &P, const float *v, int d,
                 const float *C, int ninst, int k, void *cpk, void *cside, float *cscratch,
                 float2 *ibound, SetStats *cstats, const unsigned char *active, int *assign,
                 float *dis, long long *acc, int *counts, const int *shift, int delta, int *err,
                 cudaStream_t st);

// After the caller's synchronisation: reports a timed trial of the grouped
// assignment's variant tuner (autotune.cuh); true once the variant choice of
// the last call is final, so that a CUDA graph may capture the assignment.
bool km_assign_tune_collect();

// L1 / chi2 k-means centroids (yael/kmeans.c:253-275): per cluster and
// coordinate the median (l1) or the minimiser of the summed chi2 distance of
// the cluster's points, which are first sorted by cluster (keys / vals:
// n-element scratch pairs, offs: k + 1, tmp: n x d, sort_tmp:
// km_alt_sort_bytes(n)).
size_t km_alt_sort_bytes(long n);
int km_alt_update(const int *assign, long n, const float *v, int d, int k, bool l1, int *keys,
                  int *keys2, int *vals, int *vals2, int *offs, float *tmp, void *sort_tmp,
                  size_t sort_bytes, float *C, cudaStream_t st);
int km_normalize_l1(float *C, long ncl, int d, cudaStream_t st);

// counts[inst*k + assign[p]]++ over points of active instances
int km_histogram(const int *assign, const int *pinst, long n, int k,
                 const unsigned char *active, int *counts, cudaStream_t st);

// exclusive scan of counts -> offs (ncl + 1 entries, offs[ncl] = total),
// cursor = offs
int km_scan(const int *counts, long ncl, long *offs, long *cursor, cudaStream_t st);

// perm[cursor[g]++] = p  (order inside a cluster is arbitrary; the sums below
// are exact integers, so the result does not depend on it)
int km_scatter(const int *assign, const int *pinst, long n, int k,
               const unsigned char *active, long *cursor, long *perm, cudaStream_t st);

// acc[g][c] = sum over the cluster's points of llrint(v * 2^shift[inst]),
// then C[g][c] = (float)((double)acc * 2^-shift * (1.0 / count)).  Clusters
// with count 0 become NaN (0 * inf), as in the reference before the split.
// perm holds the *total cluster-sorted points (km_scatter); nmax bounds it.
int km_update(const long *perm, const long *total, long nmax, const int *assign,
              const int *pinst, const int *counts, const float *v, int d, long ncl, int k,
              const int *shift, const unsigned char *active, long long *acc, float *C,
              cudaStream_t st);

// kth[p] >= the exact squared distance from point p to centroid assign[p]
// (FP32 direct differences widened by their rounding bound; +inf for -1): an
// upper bound of p's nearest distance for the next assignment
int km_prior_bound(const float *v, int d, long n, const int *assign, const float *C, float *kth,
                   cudaStream_t st);

// the readout of km_update alone, for sums accumulated elsewhere (km_tc_assign);
// with counts_out / err_out (host-mapped memory, say) it also copies the
// counts and *err there
int km_finalize(const long long *acc, const int *counts, long ncl, int d, int k,
                const int *shift, const unsigned char *active, float *C, cudaStream_t st,
                int *counts_out = nullptr, const int *err = nullptr, int *err_out = nullptr);

// rows of C scaled to unit L2 norm (yael/vector.c:2016-2025 arithmetic)
int km_normalize(float *C, long ncl, int d, int k, const unsigned char *active,
                 cudaStream_t st);

// fixed slices of one instance's points (<= kSliceLen each): the unit of the
// deterministic objective sums and of the per-instance max |v|
struct KmSlice {
  long p0;
  int n;
  int inst;
};
constexpr int kSliceLen = 4096;
int km_slice_sums(const KmSlice *sl, int nsl, const float *dis, double *out, cudaStream_t st);

// Per instance i (slices first[i] .. + count[i] - 1, listed in instance
// order, npts[i] points): mu[i] = the mean of its points (FP32 sums in a fixed
// order, deterministic), amax[i] = max |v| and cmax[i] >= max |fl(v - mu[i])|.
// part: 3 x nsl x d floats of scratch.
int km_inst_stats(const KmSlice *sl, int nsl, const float *v, int d, int ninst,
                  const int *first, const int *count, const long *npts, float *part, float *mu,
                  float *amax, float *cmax, cudaStream_t st);

// Stable grouping of n points by key[i] in [0, k): perm lists the points
// key by key, each key's in index order (start[b] .. start[b + 1] - 1, start
// has k + 1 entries); key_of[j] = key[perm[j]] when not null.  Scratch in the
// workspace slots slot_cnt / slot_tot.
int km_group_by_key(const int *key, long n, int k, long *perm, long *start, int *key_of,
                    Workspace &ws, int slot_cnt, int slot_tot, cudaStream_t st);

// C[i] = v[sel[i]] for rows of the listed instances
int km_gather(const float *v, int d, const long *rows, long nrows, float *C, cudaStream_t st);

}  // namespace yg
