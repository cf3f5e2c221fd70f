/*
 * yael_gpu.h -- C ABI of the GB300 (sm_103a) implementation of yael's
 * distance-GEMM path: exact k-NN, cross distances, k-means, hierarchical
 * k-means; and of the path's callers and data formats: VLAD /
 * bag-of-features, Gaussian mixtures and Fisher vectors, k-means LSH, the
 * vector files.
 *
 * The first group of functions are drop-in replacements: same symbol names,
 * argument order, meaning, ownership and error convention as the reference
 * declarations cited beside each one (paths relative to the reference
 * project).  Arrays are host memory in yael's layout: vector j of a set of n
 * d-dimensional vectors is at x + j*d ("column-major d x n", yael/nn.h:11-24).
 * Outputs are caller-allocated unless stated.  Failures print a message and
 * abort(), as the reference does with assert()/abort(); no result is ever
 * computed on the CPU.
 *
 * The yael_gpu_* group is new: explicit precision choice, device-pointer
 * inputs, status codes instead of abort(), and batched (grouped) calls.
 */
#ifndef YAEL_GPU_H
#define YAEL_GPU_H

#include <stdio.h>

#ifdef __cplusplus
extern "C" {
#endif

#define YAEL_GPU_ABI_VERSION 1

/* ------------------------------------------------------------------ */
/* drop-in: exact k-NN (yael/nn.h)                                     */

/* yael/nn.h:41-45 (yael/nn.c:451-525).  distance_type 2 or 12 = squared L2,
 * 16 = dot product (k smallest, like the reference's min-heap); 1, 3, 4, 5, 6
 * = the per-coordinate types of compute_cross_distances_alt, computed in the
 * reference's arithmetic and searched exhaustively.  k <= nb.  Neighbours are
 * ordered by increasing distance, ties by increasing base index.  b_weights
 * (may be NULL) multiplies each base vector's distance. */
void knn_full(int distance_type, int nq, int nb, int d, int k, const float *b,
              const float *q, const float *b_weights, int *assign, float *dis);

/* yael/nn.h:49-54 (yael/nn.c:679-699).  n_thread is accepted and ignored. */
void knn_full_thread(int distance_type, int nq, int nb, int d, int k,
                     const float *b, const float *q, const float *b_weights,
                     int *assign, float *dis, int n_thread);

/* yael/nn.h:63-65 (yael/nn.c:608-621): 1-NN, returns the sum of distances. */
double nn(int n, int nb, int d, const float *b, const float *v, int *assign);

/* yael/nn.h:68-71 (yael/nn.c:715-726) */
double nn_thread(int n, int nb, int d, const float *b, const float *v,
                 int *assign, int n_thread);

/* yael/nn.h:75-77 (yael/nn.c:624-632): returns malloc'd distances (free()). */
float *knn(int n, int nb, int d, int k, const float *b, const float *v, int *assign);

/* yael/nn.h:80-83 (yael/nn.c:704-711) */
float *knn_thread(int nq, int nb, int d, int k, const float *b, const float *v,
                  int *assign, int n_thread);

/* yael/nn.h:103-105 (yael/nn.c:528-580): re-order each query's short list
 * (stops at the first negative id) by exact distance, ties by list position. */
void knn_reorder_shortlist(int n, int nb, int d, int k, const float *b,
                           const float *v, int *idx, float *dis);

/* yael/nn.h:128-131 (yael/nn.c:583-600) */
void knn_recompute_exact_dists(int n, int nb, int d, int k, const float *b,
                               const float *v, int label0, int *kp,
                               const int *idx, float *dis);

/* yael/nn.h:141-143 (yael/nn.c:92-97): dist2[i + na*j] = ||a_i - b_j||^2 */
void compute_cross_distances(int d, int na, int nb, const float *a,
                             const float *b, float *dist2);

/* yael/nn.h:151-154 (yael/nn.c:100-129) */
void compute_cross_distances_nonpacked(int d, int na, int nb, const float *a,
                                       int lda, const float *b, int ldb,
                                       float *dist2, int ldd);

/* yael/nn.h:156-159 (yael/nn.c:777-792) */
void compute_cross_distances_thread(int d, int na, int nb, const float *a,
                                    const float *b, float *dist2, int nt);

/* yael/nn.h:174-176 (yael/nn.c:352-356).  Every type runs on the GPU: 12
 * (expanded-form L2) and 16 (dot product) as GEMMs; 1 (L1), 2 (L2), 3 / 4
 * (chi2 forms), 5 (histogram intersection), 6 (dot) as the reference's
 * per-coordinate sums (float lanes for 1 / 3 when d % 4 == 0, else double
 * sums of float terms), bit-identical to its x86 build; other types abort
 * with a message. */
void compute_cross_distances_alt(int distance_type, int d, int na, int nb,
                                 const float *a, const float *b, float *dist2);

/* yael/nn.h:180-183 (yael/nn.c:280-350) */
void compute_cross_distances_alt_nonpacked(int distance_type, int d, int na,
                                           int nb, const float *a, int lda,
                                           const float *b, int ldb,
                                           float *dist2, int ldd);

/* yael/nn.h:188-191 (yael/nn.c:795-810) */
void compute_cross_distances_alt_thread(int distance_type, int d, int na, int nb,
                                        const float *a, const float *b,
                                        float *dist2, int nt);

/* yael/nn.h:195-198 (yael/nn.c:156-162) */
void compute_distances_1(int d, int nb, const float *a, const float *b, float *dist2);

/* yael/nn.h:200-203 (yael/nn.c:132-154) */
void compute_distances_1_nonpacked(int d, int nb, const float *a, const float *b,
                                   int ldb, float *dist2);

/* yael/nn.h:205-209 (yael/nn.c:830-837) */
void compute_distances_1_thread(int d, int nb, const float *a, const float *b,
                                float *dist2, int n_thread);

/* yael/nn.h:211-215 (yael/nn.c:840-860) */
void compute_distances_1_nonpacked_thread(int d, int nb, const float *a,
                                          const float *b, int ldb, float *dist2,
                                          int n_thread);

/* ------------------------------------------------------------------ */
/* drop-in: k-means (yael/kmeans.h)                                    */

/* flag bits, same values as yael/kmeans.h:11-18 */
#define YAEL_KMEANS_QUIET 0x10000
#define YAEL_KMEANS_INIT_BERKELEY 0x20000
#define YAEL_KMEANS_NORMALIZE_CENTS 0x40000
#define YAEL_KMEANS_INIT_RANDOM 0x80000
#define YAEL_KMEANS_INIT_USER 0x100000
#define YAEL_KMEANS_L1 0x200000
#define YAEL_KMEANS_CHI2 0x400000

/* yael/kmeans.h:41-44 (yael/kmeans.c:332-447).  Same flags, seed (0 draws
 * lrand48()), redo, outputs (each may be NULL) and return value (qerr / n, or
 * -1 when too many empty clusters were split).  Assignments are exact:
 * nearest centroid by FP64 distance, ties to the lowest index.  Centroids are
 * exact integer sums (2^-S fixed point, S chosen from the data so nothing
 * overflows) divided by the count.  flags & 0xffff (threads) is ignored;
 * KMEANS_L1 / KMEANS_CHI2: assignment by the L1 / chi2 distance (type 1 / 3),
 * centroids the per-coordinate medians / chi2 minimisers, as the reference. */
float kmeans(int d, int n, int k, int niter, const float *v, int flags, long seed,
             int redo, float *centroids, float *dis, int *assign, int *nassign);

/* yael/kmeans.h:51-53 (yael/kmeans.c:492-504): malloc'd k x d centroids */
float *clustering_kmeans(int n, int d, const float *points, int k, int nb_iter_max,
                         double normalize);

/* yael/kmeans.h:58-61 (yael/kmeans.c:484-490) */
float *clustering_kmeans_assign(int n, int d, const float *points, int k,
                                int nb_iter_max, double normalize,
                                int **clust_assign_out);

/* yael/kmeans.h:65-68 (yael/kmeans.c:452-482): nb_iter_max / 100000 = redo */
float *clustering_kmeans_assign_with_score(int n, int d, const float *points, int k,
                                           int nb_iter_max, double normalize,
                                           int n_thread, double *score_out,
                                           int **clust_assign_out);

/* ------------------------------------------------------------------ */
/* drop-in: hierarchical k-means (yael/hkm.h)                          */

/* same layout as yael/hkm.h:10-16 */
typedef struct hkm_s {
  int nlevel;        /* number of levels */
  int bf;            /* branching factor */
  int k;             /* number of leaves, bf^nlevel */
  int d;             /* dimension */
  float **centroids; /* level l: bf^(l+1) x d centroids */
} hkm_t;

/* yael/hkm.h:21-23 (yael/hkm.c:36-116).  Every child clustering of a level
 * runs in one grouped GPU pass; seeds are drawn with lrand48() in (level,
 * parent) order as the reference does.  An empty node exits(1) like the
 * reference. */
hkm_t *hkm_learn(int n, int d, int nlevel, int bf, const float *v, int nb_iter_max,
                 int nt, int verbose, int **clust_assign_out);

/* yael/hkm.h:25 (yael/hkm.c:119-126) */
void hkm_delete(hkm_t *hkm);

/* yael/hkm.h:28 (yael/hkm.c:131-150): greedy descent, exact nearest child */
void hkm_quantize(const hkm_t *hkm, int n, const float *v, int *idx);

/* yael/hkm.h:31-32 (yael/hkm.c:181-232): same binary format */
void hkm_write(const char *filename, const hkm_t *hkm);
hkm_t *hkm_read(const char *filename);

/* yael/hkm.h:35 (yael/hkm.c:154-157) */
float *hkm_get_centroids(const hkm_t *hkm, int l, int no);

/* Image descriptors on the exact nearest-centroid assignment
 * (yael/vlad.h:17-76, yael/vlad.c:10-139): VLAD sums are the reference's own
 * float additions in point (or list) order; bag-of-features counts exact.
 * Points without a nearest centroid (all-NaN rows) are left out. */
void vlad_compute(int k, int d, const float *centroids, int n, const float *v, float *desc);
void vlad_compute_weighted(int k, int d, const float *centroids, int n, const float *v,
                           const float *weights, float *desc);
void vlad_compute_subsets(int k, int d, const float *centroids, int n, const float *v,
                          int n_subset, const int *subset_indexes, const int *subset_ends,
                          float *desc);
void bof_compute(int k, int d, const float *centroids, int n, const float *v, int *desc);
void bof_compute_ma(int k, int d, const float *centroids, int n, const float *v, int *desc,
                    int ma, float alpha, int nt);
void bof_compute_subsets(int k, int d, const float *centroids, int n, const float *v,
                         int n_subset, const int *subset_indexes, const int *subset_ends,
                         float *desc);

/* ------------------------------------------------------------------ */
/* drop-in: Gaussian mixtures and Fisher vectors (yael/gmm.h)          */

/* same layout as yael/gmm.h:19-25 */
typedef struct gmm_s {
  int d;        /* dimension */
  int k;        /* components */
  float *w;     /* k weights */
  float *mu;    /* k x d means */
  float *sigma; /* k x d diagonal variances */
} gmm_t;

/* flag bits, same values as yael/gmm.h:28-41 */
#define YAEL_GMM_FLAGS_W 1
#define YAEL_GMM_FLAGS_NO_NORM 2
#define YAEL_GMM_FLAGS_1SIGMA 4
#define YAEL_GMM_FLAGS_SIGMA 8
#define YAEL_GMM_FLAGS_MU 16
#define YAEL_GMM_FLAGS_PURE_KMEANS 32

/* yael/gmm.h:57-59 (yael/gmm.c:436-502): the drop-in kmeans, then EM on the
 * GPU (posteriors and posterior-weighted moments per iteration, parameters on
 * the host) until the sum of the means repeats or niter iterations.  Returns
 * a malloc'd mixture (gmm_delete). */
gmm_t *gmm_learn(int d, int n, int k, int niter, const float *v, int nt, int seed, int nredo,
                 int flags);
/* yael/gmm.h:63-66 (yael/gmm.c:794-807, 43-49) */
void gmm_print(const gmm_t *g);
void gmm_delete(gmm_t *g);
/* yael/gmm.h:74-77, 135-140 (yael/gmm.c:305-362, 862-870): p (n x k) =
 * p(component | vector); squared Mahalanobis distances in direct form;
 * n_thread is ignored */
void gmm_compute_p(int n, const float *v, const gmm_t *g, float *p, int flags);
void gmm_compute_p_thread(int n, const float *v, const gmm_t *g, float *p, int flags,
                          int n_thread);
/* yael/gmm.h:95-107 (yael/gmm.c:505-725): Fisher vectors from the
 * posterior-weighted moments (FP64 sums on the GPU) */
void gmm_fisher(int n, const float *v, const gmm_t *g, int flags, float *fisher_vector_out);
void gmm_fisher_from_posteriors(int n, const float *v, const gmm_t *g, int flags,
                                const float *p, float *fisher_vector_out);
size_t gmm_fisher_sizeof(const gmm_t *g, int flags);
/* yael/gmm.h:121-124 (yael/gmm.c:728-791): Q (K x N posteriors), sgmm (mean
 * then variance, D each), ll (D x N: coordinate d of vector i at ll[d*N+i]);
 * sdesc = D x K mean terms then D x K variance terms */
void gmm_fisher_spatial(int N, int K, int D, const float *Q, const float *sgmm,
                        const float *ll, float *sdesc);
/* yael/gmm.h:128-131 (yael/gmm.c:810-850): d, k, w, mu, sigma as raw int32 /
 * float32; an I/O error prints and aborts */
void gmm_write(const gmm_t *g, FILE *f);
gmm_t *gmm_read(FILE *f);

/* ------------------------------------------------------------------ */
/* drop-in: k-means LSH (yael/kmlsh.h)                                 */

/* same layouts as yael/kmlsh.h:24-29, 62-67, 74-80 */
typedef struct nnlist_s {
  long n;     /* number of lists */
  long k;     /* entries per list */
  int *idx;   /* n x k ids (-1: empty) */
  float *dis; /* n x k distances (1e30: empty) */
} nnlist_t;

typedef struct kmlsh_s {
  int nhash;         /* number of partitions (hash functions) */
  int d;             /* dimension */
  int nclust;        /* cells per partition */
  float **centroids; /* nhash arrays of nclust x d */
} kmlsh_t;

typedef struct kmlsh_idx_s {
  int nhash;
  int n;           /* vectors indexed */
  int nclust;
  int *perm;       /* per partition: the n ids ordered by cell */
  int *boundaries; /* per partition: the nclust + 1 cell starts in perm */
} kmlsh_idx_t;

/* flag bits and constants, same values as yael/kmlsh.h:49-58 */
#define YAEL_KMLSH_NT 0x000000ff
#define YAEL_KMLSH_QUIET 0x00010000
#define YAEL_KMLSH_WRITE_INTER_NHASH 0x00020000
#define YAEL_KMLSH_BLOCK_SIZE 256
#define YAEL_KMLSH_NB_ITER_MAX 8
#define YAEL_KMLSH_VECTYPE_FVEC 0
#define YAEL_KMLSH_VECTYPE_BVEC 1

/* yael/kmlsh.h:31-44 (yael/kmlsh.c:31-92): n lists of k (id, distance);
 * nnlist_addn keeps each list's k smallest distinct ids, the largest in
 * slot 0, in the reference's slot order.  _noalloc leaves idx / dis NULL. */
nnlist_t *nnlist_new(int n, int k);
nnlist_t *nnlist_new_noalloc(int n, int k);
void nnlist_delete(nnlist_t *l);
void nnlist_addn(nnlist_t *l, int lno, int n, int *idx, float *dis);

/* yael/kmlsh.h:86-104 (yael/kmlsh.c:99-206): each partition is the drop-in
 * kmeans (8 iterations, random init, seed drawn by lrand48()) of nlearn
 * vectors sampled with ivec_new_random_idx, as the reference */
kmlsh_t *kmlsh_new(int nhash, int nclust, int d);
void kmlsh_delete(kmlsh_t *lsh);
void kmlsh_learn_xvec(kmlsh_t *lsh, int n, int nlearn, const void *v, int flags,
                      int vec_type);
kmlsh_t *kmlsh_new_learn_bvec(int nhash, int nclust, int d, int n, int nlearn,
                              const unsigned char *v, int flags);
kmlsh_t *kmlsh_new_learn_fvec(int nhash, int nclust, int d, int n, int nlearn,
                              const float *v, int flags);

/* yael/kmlsh.h:106-119 (yael/kmlsh.c:376-476): per partition, the exact
 * k-NN of every cell's queries among the cell's base vectors (one batched
 * GPU call over the occupied cells), merged into one list of k per query
 * in the reference's order.  nt is ignored. */
nnlist_t *kmlsh_match_xvec(const kmlsh_t *lsh, const kmlsh_idx_t *lshidx_b, const void *vb,
                           int nb, const kmlsh_idx_t *lshidx_q, const void *vq, int nq, int k,
                           int nt, int vec_type);
nnlist_t *kmlsh_match_bvec(const kmlsh_t *lsh, const kmlsh_idx_t *lshidx_b,
                           const unsigned char *vb, int nb, const kmlsh_idx_t *lshidx_q,
                           const unsigned char *vq, int nq, int k, int nt);
nnlist_t *kmlsh_match_fvec(const kmlsh_t *lsh, const kmlsh_idx_t *lshidx_b, const float *vb,
                           int nb, const kmlsh_idx_t *lshidx_q, const float *vq, int nq, int k,
                           int nt);

/* yael/kmlsh.h:124-135 (yael/kmlsh.c:479-520): nclust = sqrt(nb), 100 *
 * nclust learning vectors, then learn, index and match as above */
nnlist_t *kmlsh_ann_xvec(const void *vb, int nb, const void *vq, int nq, int d, int k,
                         int nhash, int flags, int vec_type);
nnlist_t *kmlsh_ann_bvec(const unsigned char *vb, int nb, const unsigned char *vq, int nq,
                         int d, int k, int nhash, int flags);
nnlist_t *kmlsh_ann_fvec(const float *vb, int nb, const float *vq, int nq, int d, int k,
                         int nhash, int flags);

/* yael/kmlsh.h:138-169 (yael/kmlsh.c:210-372): per partition the
 * nearest centroid of each vector (one k = 1 GPU search), then the ids
 * ordered by cell (stable) and the cell starts */
kmlsh_idx_t *kmlsh_idx_new(const kmlsh_t *lsh, int n);
void kmlsh_idx_delete(kmlsh_idx_t *lshidx);
kmlsh_idx_t *kmlsh_idx_new_compile_xvec(const kmlsh_t *lsh, const void *v, int n, int flags,
                                        int vec_type);
kmlsh_idx_t *kmlsh_idx_new_compile_bvec(const kmlsh_t *lsh, const unsigned char *v, int n,
                                        int flags);
kmlsh_idx_t *kmlsh_idx_new_compile_fvec(const kmlsh_t *lsh, const float *v, int n, int flags);
int kmlsh_idx_get_nvec(const kmlsh_idx_t *lshidx, int h, int c);
int kmlsh_idx_get_maxincell(const kmlsh_idx_t *lshidx, int h);
int *kmlsh_idx_get_vecids(const kmlsh_idx_t *lshidx, int h, int c);
void kmeans_cohash_xvec(const kmlsh_t *lsh, int h, const void *v, int n, int *perm,
                        int *boundaries, int flags, int vec_type);
void kmeans_cohash_bvec(const kmlsh_t *lsh, int h, const unsigned char *v, int n, int *perm,
                        int *boundaries, int flags);
void kmeans_cohash_fvec(const kmlsh_t *lsh, int h, const float *v, int n, int *perm,
                        int *boundaries, int flags);

/* yael/kmlsh.h:175-184 (yael/kmlsh.c:526-611): same files; an I/O error
 * prints and exits(1).  kmlsh_idx_write checks each record's write status
 * (the reference compares the second one with nclust + 1 and so exits). */
void kmlsh_write(const char *filename, const kmlsh_t *lsh);
void kmlsh_read(const char *filename, const kmlsh_t *lsh);
void kmlsh_idx_write(const char *filename, const kmlsh_idx_t *lshidx);
void kmlsh_idx_read(const char *filename, kmlsh_idx_t *lshidx);

/* Vector files (host code, doc/file_format.rst): records of an int32
 * dimension d followed by d floats (.fvecs), int32 (.ivecs) or uint8
 * (.bvecs).  Same return values as the reference; where it asserts on a
 * dimension / count mismatch (b2fvecs_read) these print and return -1.
 * Arrays from the *_new_* readers are malloc'd. */
/* yael/vector.h:190-212 (yael/vector.c:1369-1580; bvec_fwrite and
 * bvecs_fwrite are defined at yael/vector.c:1540, 1559): 0 / count written */
int fvec_fwrite(FILE *f, const float *v, int d);
int ivec_fwrite(FILE *f, const int *v, int d);
int bvec_fwrite(FILE *f, const unsigned char *v, int d);
int fvecs_fwrite(FILE *f, int d, int n, const float *v);
int ivecs_fwrite(FILE *f, int d, int n, const int *v);
int bvecs_fwrite(FILE *f, int d, int n, const unsigned char *v);
int fvecs_write(const char *fname, int d, int n, const float *v);
int ivecs_write(const char *fname, int d, int n, const int *v);
int bvecs_write(const char *fname, int d, int n, const unsigned char *v);
/* yael/vector.h:183-185 (yael/vector.c:593-640): file bytes, *d_out, *n_out */
long fvecs_fsize(const char *fname, int *d_out, int *n_out);
long ivecs_fsize(const char *fname, int *d_out, int *n_out);
long bvecs_fsize(const char *fname, int *d_out, int *n_out);
/* yael/vector.h:217-248, 325-328 (yael/vector.c:651-720, 1121-1150,
 * 1298-1320): number of vectors read, -1 on error */
int fvecs_new_read(const char *fname, int *d_out, float **vf);
int fvecs_new_fread_max(FILE *f, int *d_out, float **vf, long nmax);
int ivecs_new_read(const char *fname, int *d_out, int **vi);
int ivecs_new_fread_max(FILE *f, int *d_out, int **vi, long nmax);
int bvecs_new_read(const char *fname, int *d_out, unsigned char **v_out);
int b2fvecs_new_read(const char *fname, int *d_out, float **v_out);
/* yael/vector.h:263-266 (yael/vector.c:882-935): the first n vectors */
int fvecs_read(const char *fname, int d, int n, float *v);
int b2fvecs_read(const char *fname, int d, int n, float *v);
/* yael/vector.h:280-317 (yael/vector.c:966-1090): one record (its d, 0 at
 * end of file, -1 on error); n records (the count, 0 on error) */
int fvec_fread(FILE *f, float *v, int d_alloc);
int ivec_fread(FILE *f, int *v, int d_alloc);
int bvec_fread(FILE *f, unsigned char *v, int d_alloc);
long fvecs_fread(FILE *f, float *v, long n, int d_alloc);
long ivecs_fread(FILE *f, int *v, long n, int d_alloc);
long bvecs_fread(FILE *f, unsigned char *v, long n, int d_alloc);
/* yael/vector.h:193-200 (yael/vector.c:1386-1445): d elements without the
 * dimension header; 0, -1 on error */
int fvec_fwrite_raw(FILE *f, const float *v, long d);
int ivec_fwrite_raw(FILE *f, const int *v, long d);
int bvec_fwrite_raw(FILE *f, const unsigned char *v, long d);
int fvec_write_raw(const char *fname, const float *v, long d);
int ivec_write_raw(const char *fname, const int *v, long d);
int bvec_write_raw(const char *fname, const unsigned char *v, long d);
/* yael/vector.h:282-295 (yael/vector.c:1149-1250): n headerless elements
 * (n, -1 on a short read: the caller's buffer is left allocated, where the
 * reference frees it); the *_new_* forms return a malloc'd array or NULL */
int fvec_fread_raw(FILE *f, float *v, long n);
int ivec_fread_raw(FILE *f, int *v, long n);
int bvec_fread_raw(FILE *f, unsigned char *v, long n);
float *fvec_new_fread_raw(FILE *f, long d);
int *ivec_new_fread_raw(FILE *f, long d);
unsigned char *bvec_new_fread_raw(FILE *f, long d);
float *fvec_new_read_raw(const char *fname, long d);
int *ivec_new_read_raw(const char *fname, long d);
unsigned char *bvec_new_read_raw(const char *fname, long d);
/* yael/vector.h:207-210, 270 (yael/vector.c:939-964, 1279-1294, 1475-1491):
 * one text line per vector, "%d " / "%f " per element; the writers return n
 * (-1 if the file cannot be opened), the reader the whole vectors read */
int ivecs_write_txt(const char *fname, int d, int n, const int *v);
int fvecs_write_txt(const char *fname, int d, int n, const float *v);
int fvecs_read_txt(const char *fname, int d, int n, float *v);

/* ------------------------------------------------------------------ */
/* extension API                                                       */

#define YAEL_GPU_PREC_ENV (-1) /* take YAEL_GPU_PRECISION (fp32 | bf16 | bf16x3 | fp16), default fp32 */
#define YAEL_GPU_PREC_FP32 0   /* FP32 CUDA-core distances (the plain drop-in path) */
#define YAEL_GPU_PREC_BF16 1   /* BF16 tensor-core distances + exact FP32 re-rank */
#define YAEL_GPU_PREC_BF16X3 2 /* tensor cores on a 3xBF16 split (x = hi + lo) + re-rank */
#define YAEL_GPU_PREC_FP16 3   /* FP16 tensor-core distances + exact FP32 re-rank: the bf16
                                  rate with 2^-11 rounding, for data fp16 holds (|x| < 16384,
                                  base ||x||^2 < 2^15; other rows are settled by later passes) */

/* status codes of the yael_gpu_* functions */
#define YAEL_GPU_OK 0
#define YAEL_GPU_ECUDA 1
#define YAEL_GPU_EARG 2
#define YAEL_GPU_EUNSUPPORTED 3
#define YAEL_GPU_ENOMEM 4
#define YAEL_GPU_ETIMEOUT 5

typedef struct {
  int precision;   /* YAEL_GPU_PREC_* */
  int metric;      /* yael distance_type: 2 (or 12) = squared L2, 16 = dot product */
  int device_ptrs; /* 1: b, q, assign, dis are device pointers on the current device */
  void *stream;    /* cudaStream_t for device_ptrs calls; NULL = the library's stream */
  /* filled on return */
  int n_fallback;   /* queries whose certificate failed and were recomputed exhaustively */
  int n_candidates; /* total candidates re-ranked */
  int exact_class;  /* 1 if every distance was computed exactly (integer-valued data) */
  int timing;       /* 1: time the passes with CUDA events on the launching stream */
  float ms_scan;    /* main fused distance + selection pass (sum over query batches) */
  float ms_sample;  /* threshold-estimation pass over the base sample */
  float ms_rerank;  /* re-rank + certificate */
  int scan_launches; /* launches of the main pass included in ms_scan */
  int n_second;     /* queries re-run through the 3xBF16 split pass */
  int n_band;       /* rejected queries re-run through a band pass (thresholds from the
                       k-th exact distance the first re-rank found) */
  float ms_second;  /* band, split and exhaustive passes together */
  int wait_limit_us; /* every wait inside the tensor-core passes gives up after this many
                        microseconds (0: 2 s), and the call then returns YAEL_GPU_ETIMEOUT */
} yael_gpu_knn_opts;

/* k-NN with explicit options.  Same result contract as knn_full. */
int yael_gpu_knn_ex(int nq, int nb, int d, int k, const float *b, const float *q,
                    int *assign, float *dis, yael_gpu_knn_opts *opts);

/* One (queries, base) pair of a batched k-NN call. */
typedef struct {
  int nq, nb;          /* query rows and base rows of this pair (k <= nb) */
  const float *q;      /* nq x d, row-major (yael layout) */
  const float *b;      /* nb x d */
  int *assign;         /* out: nq x k ids into this pair's base */
  float *dis;          /* out: nq x k distances */
} yael_gpu_knn_pair;

/* knn_full over npairs independent pairs of uneven sizes, all with the same d,
 * k, metric and precision (opts may be NULL: L2, YAEL_GPU_PRECISION).  No
 * counterpart in the reference, whose callers loop over knn_full (per-cell
 * searches, hkm / kmlsh children); results are those of that loop.  With
 * device arrays, the BF16 pass and k >= 9 every pass is one persistent launch
 * over all the pairs (YAEL_GPU_BATCH_GROUPED=0: off); otherwise pairs run
 * concurrently, largest first, on a persistent pool of host workers each with
 * its own stream and workspace (YAEL_GPU_BATCH_WORKERS, default 8).  With
 * opts->device_ptrs every array is device memory and opts->stream (a
 * cudaStream_t, NULL = default stream) is synchronised before the pairs start.
 * Returns when every pair is done; opts' counters are summed over the pairs.
 * Returns a status code (first error met; later pairs are skipped). */
int yael_gpu_knn_batch(int npairs, const yael_gpu_knn_pair *pairs, int d, int k,
                       yael_gpu_knn_opts *opts);

typedef struct {
  int precision;   /* YAEL_GPU_PREC_*: distance pass of the assignment step */
  int device_ptrs; /* 1: v and the outputs are device pointers */
  void *stream;    /* cudaStream_t for device_ptrs calls; NULL = the library's stream */
  /* filled on return */
  int status;      /* YAEL_GPU_OK or an error code (then the return value is -2) */
  long iterations; /* total Lloyd iterations over all runs */
  long n_fallback; /* points recomputed by the exhaustive FP64 path */
  long n_second;   /* points re-run through the 3xBF16 split pass */
  float ms_assign; /* GPU time of the assignment steps */
  float ms_update; /* GPU time of counts, sums, splits' uploads and objective */
  long n_band;     /* points re-run through a band pass */
  int prec_used;   /* filled: the distance pass of the last assignment (YAEL_GPU_PREC_*;
                      the chosen form runs fp16 operands where the data range allows) */
  /* Optional record of every iteration, for checkers of the assignment step
   * (host memory; n_probe = 0 turns it off).  Iteration t (0-based, over all
   * runs, t < probe_iters) stores the assignment of the n_probe points
   * probe_rows, the centroids that assignment was made against (when
   * probe_centroids is not NULL) and the iteration's objective (sum of the
   * points' distances).  Recording synchronises the stream every iteration. */
  int n_probe;
  const long *probe_rows;
  int probe_iters;
  int *probe_assign;      /* probe_iters x n_probe */
  float *probe_centroids; /* probe_iters x k x d, or NULL */
  double *probe_qerr;     /* probe_iters, or NULL */
  int wait_limit_us;      /* as in yael_gpu_knn_opts */
} yael_gpu_kmeans_opts;

/* kmeans() with options; returns -2 on error (message: yael_gpu_last_error). */
float yael_gpu_kmeans_ex(int d, int n, int k, int niter, const float *v, int flags,
                         long seed, int redo, float *centroids, float *dis, int *assign,
                         int *nassign, yael_gpu_kmeans_opts *opts);

/* hkm_learn() with flat outputs: centroids = all levels concatenated
 * (sum_l bf^(l+1) * d floats), assign (n ints, may be NULL).  Returns a status
 * code; iterations and ms (GPU time) may be NULL.
 * small_nodes = 0: a node with fewer points than bf is an error, as in the
 * reference (its kmeans asserts k <= n).  small_nodes = 1: such a node gets one
 * child per point (children past the last point repeat it) without k-means;
 * its lrand48() draw is still made so later seeds stay in step. */
int yael_gpu_hkm_learn_ex(int n, int d, int nlevel, int bf, const float *v,
                          int nb_iter_max, int small_nodes, float *centroids, int *assign,
                          long *iterations, float *ms);

/* Work counters of the calling thread's last kmeans / hkm call (the drop-in
 * symbols and the _ex functions).  No counterpart in the reference. */
typedef struct {
  long instance_iterations; /* Lloyd iterations summed over the clusterings run */
  long point_iterations;    /* points assigned, summed over iterations: the rows the
                               assignment passes had to read */
  long level_iterations;    /* iterations of the batched loop (hkm: over all levels) */
  float ms_assign;          /* GPU time of the assignment steps */
  float ms_update;          /* GPU time of the updates */
  int prec_used;            /* distance pass of the last assignment (YAEL_GPU_PREC_*) */
} yael_gpu_call_stats;
int yael_gpu_last_stats(yael_gpu_call_stats *out);

/* Exact k-NN that allocates no GPU memory.  No counterpart in the reference:
 * it exists for callers that cannot let a library call cudaMalloc -- a
 * process whose device memory is all handed to its own pool allocator, or a
 * latency-critical path where cudaMalloc / cudaFree would synchronise the
 * device.  Same results as yael_gpu_knn_ex with the FP32 pass (L2, ids ordered
 * by distance then index).  b (nb x d), q (nq x d), assign and dis (nq x k)
 * are device pointers; the work is ordered on stream (a cudaStream_t, NULL =
 * the default stream) and the call returns when it is complete.
 * Scratch comes from one 32 MiB __device__ array that the library holds on
 * every GPU that loads it.  Limits: k <= 16, and the scratch must fit (about
 * 12 bytes per base row plus 8 C + 24 bytes per query, C the smallest power
 * of two >= 2k; e.g. nb = 1M with nq = 20k at k = 10); larger requests
 * return YAEL_GPU_EARG with the size in yael_gpu_last_error() -- use
 * yael_gpu_knn_ex for them.  Each call looks up the array's device address
 * (a lookup, no allocation) and synchronises the stream before it returns,
 * error returns included: never call it on a stream that is being captured
 * into a CUDA graph.  All calls share the array: calls whose GPU work
 * overlaps race and must be serialised by the caller. */
int yael_gpu_knn_noalloc(int nq, int nb, int d, int k, const float *b, const float *q,
                         int *assign, float *dis, void *stream);

/* message of the last failure on the calling thread ("" if none) */
const char *yael_gpu_last_error(void);

/* YAEL_GPU_ABI_VERSION of the loaded library */
int yael_gpu_version(void);

/* number of kernels this library has launched in this process */
long yael_gpu_launch_count(void);

#ifdef __cplusplus
}
#endif
#endif
