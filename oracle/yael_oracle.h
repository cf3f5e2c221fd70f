/*
 * yael_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * A CPU restatement of yael's distance-GEMM path (exact k-NN, k-means Lloyd loop,
 * hierarchical k-means) and of two of its callers (k-means LSH, Gaussian
 * mixtures), used as the checker for the GPU library and as the timed CPU
 * baseline.  Nothing in the product library links, loads or calls this code;
 * only tests/, __graft_entry__.smoke() and bench.py's CPU legs do.
 *
 * Two arithmetic modes:
 *   ORC_PORT  -- the reference's own arithmetic, step for step: blocked 256x256
 *                expanded-form FP32 distances through BLAS sgemm (yael/nn.c:100-129,
 *                451-525), the bounded max-heap with yael's tie behaviour
 *                (yael/binheap.c:139-156, 201-211), float centroid accumulation
 *                (yael/kmeans.c:277-288).  Bit-exact with the compiled reference
 *                when linked to the same BLAS.
 *   ORC_EXACT -- the semantics the GPU library implements: FP64 distances
 *                (yael/vector.c:2348-2358 form), canonical (distance, index) order,
 *                argmin ties to the lowest index (the k=1 rule of yael/nn.c:431-435),
 *                exact fixed-point centroid sums read out through FP64.  The RNG
 *                stream (seeds, init, empty-cluster splits) is identical in both
 *                modes and identical to the reference's.
 */
#ifndef YAEL_ORACLE_H
#define YAEL_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_PORT 0
#define ORC_EXACT 1

/* kmeans flag bits, same values as yael/kmeans.h:11-18 */
#define ORC_KMEANS_QUIET 0x10000
#define ORC_KMEANS_INIT_BERKELEY 0x20000
#define ORC_KMEANS_NORMALIZE_CENTS 0x40000
#define ORC_KMEANS_INIT_RANDOM 0x80000
#define ORC_KMEANS_INIT_USER 0x100000
#define ORC_KMEANS_L1 0x200000
#define ORC_KMEANS_CHI2 0x400000

const char *oracle_blas_name(void);

/* FP64 brute force: for each query the k smallest FP64 squared L2 distances,
 * ordered by (distance, base index).  dis receives the FP64 value rounded to
 * float; dis64 (may be NULL) the FP64 value.  Follows yael/nn.c:451-525 for
 * the interface (b(d,nb), q(d,nq), outputs (k,nq)). */
void orc_knn_exact(int nq, int nb, int d, int k, const float *b, const float *q,
                   int *assign, float *dis, double *dis64, int nt);

/* Restatement of knn_full_thread (yael/nn.c:679-699 -> 451-525): distance_type
 * 2/12 (expanded form via sgemm) or 16 (sgemm dot product). */
void orc_knn_port(int distance_type, int nq, int nb, int d, int k, const float *b,
                  const float *q, const float *b_weights, int *assign, float *dis,
                  int nt);

/* Restatement of compute_cross_distances_alt_nonpacked (yael/nn.c:164-350):
 * every distance type, with the SSE2 lane form for L1 / chi2 when d % 4 == 0
 * in builds with SSE2 (as the reference's x86 build), double sums otherwise.
 * orc_knn_port takes these types as well (knn_full's _alt dispatch). */
void orc_cross_distances_alt(int dt, int d, int na, int nb, const float *a, int lda,
                             const float *b, int ldb, float *dist2, int ldd);

/* vlad_compute (yael/vlad.c:10-27) with the nearest centroids of the port */
void orc_vlad_compute(int k, int d, const float *centroids, int n, const float *v, float *desc,
                      int nt);

/* Restatement of compute_cross_distances_nonpacked (yael/nn.c:100-129). */
void orc_cross_distances_port(int d, int na, int nb, const float *a, int lda,
                              const float *b, int ldb, float *dist2, int ldd);

/* FP64 reference of the full cross-distance matrix dist2[i + ldd*j]. */
void orc_cross_distances_exact(int d, int na, int nb, const float *a,
                               const float *b, double *dist2);

/* Restatement of kmeans() (yael/kmeans.c:332-447) in the given mode.
 * Returns qerr/n, or -1 on abandon (yael/kmeans.c:302-306, 443-444).
 * *iters_out (may be NULL) receives the total number of Lloyd iterations. */
float orc_kmeans(int d, int n, int k, int niter, const float *v, int flags,
                 long seed, int redo, float *centroids, float *dis, int *assign,
                 int *nassign, int mode, long *iters_out);

/* One Lloyd step of ORC_EXACT mode on given centroids (no RNG): assignment,
 * counts, fixed-point centroid update.  Used to check a single GPU iteration. */
void orc_kmeans_step_exact(int d, int n, int k, const float *v, const float *c_in,
                           int *assign, float *dis, int *nassign, float *c_out,
                           int fixed_shift);

/* Checker of one assignment step at any size: the number of the n points
 * whose assign[i] is not the ORC_EXACT nearest of the k centroids c (FP64
 * distances in the dist64 form, ties to the lowest index; a point with no
 * finite distance must have -1).  The k distances of a point are screened in
 * FP32 through BLAS sgemm; every centroid whose FP32 value can be within the
 * screen's rounding bound of the smallest, (d + 4) 2^-24 (||x|| + ||c||)^2
 * each, is then recomputed in FP64, so the answer is the FP64 argmin's.
 * first_bad (may be NULL) receives the first disagreeing point or -1.
 * Not part of the reference: a test utility for sizes where the FP64 brute
 * force of assign_exact would take minutes. */
long orc_assign_check(int d, int n, int k, const float *v, const float *c, const int *assign,
                      int nt, long *first_bad);

/* Checker of k-NN results at any size: the number of the nq queries whose
 * row of idx (k ids) is not the ORC_EXACT result (the k smallest dist64
 * distances in (distance, id) order).  Distances are screened in FP32 through
 * BLAS sgemm; every base row whose FP32 value can be within the screen's
 * rounding bound ((d + 4) 2^-24 (||q|| + ||b||)^2) of the k-th smallest is
 * recomputed in FP64.  Queries or rows with non-finite values are compared
 * with orc_knn_exact's answer directly.  first_bad (may be NULL) receives the
 * first disagreeing query or -1.  Test utility, not part of the reference. */
long orc_knn_check(int d, int nq, int nb, int k, const float *b, const float *q, const int *idx,
                   int nt, long *first_bad);

/* The FP64 objective of an assignment: the sum over the n points of the
 * dist64 distance to centroid assign[i] (points with assign -1 add nothing),
 * summed per thread slice then across slices in FP64.  Test utility. */
double orc_objective64(int d, int n, const float *v, const float *c, const int *assign, int nt);

/* The fixed-point shift used by ORC_EXACT centroid sums for this data. */
int orc_fixed_shift(long n, long d, const float *v);

/* The empty-cluster split of k-means (yael/kmeans.c:166-209) on the k x d
 * centroids C, with the counts nassign and the seed its caller draws;
 * returns the number of clusters split.  Test utility: the restatement the
 * k-means loop already uses, exported to check the GPU library's host split. */
int orc_reassign_empty(int d, int k, float *C, const int *nassign, unsigned int seed);

/* hierarchical k-means (yael/hkm.c:36-116).  centroids_out receives the
 * levels concatenated (level l holds bf^(l+1) rows of d floats).  assign_out
 * (n ints, may be NULL).  Returns 0, or -1 when a node is empty (where the
 * reference exits, yael/hkm.c:77-80) or too small for bf clusters.  With
 * ORC_HKM_SMALL_NODES or'ed into mode, a node with 0 < n < bf points gets one
 * child per point instead (the GPU library's small_nodes = 1 rule, not the
 * reference's). */
#define ORC_HKM_SMALL_NODES 0x100
int orc_hkm_learn(int n, int d, int nlevel, int bf, const float *points,
                  int nb_iter_max, float *centroids_out, int *assign_out, int mode);

/* greedy descent (yael/hkm.c:131-150) */
void orc_hkm_quantize(int nlevel, int bf, int d, const float *centroids, int npt,
                      const float *v, int *idx, int mode);

/* k-means LSH search (yael/kmlsh.c:479-500: learn 133-185, cell assignment
 * 210-279, per-cell search and merge 376-456) with nt threads, split as the
 * reference splits them.  vec_type 0: float rows, 1: byte rows.  idx_out /
 * dis_out (nq x k) receive the merged lists in the reference's slot order.
 * The RNG stream (lrand48 per partition, then the kmeans seed) is the
 * reference's. */
void orc_kmlsh_ann(const void *vb, int nb, const void *vq, int nq, int d, int k, int nhash,
                   int vec_type, int mode, int nt, int *idx_out, float *dis_out);

/* Gaussian mixtures in the reference's arithmetic (yael/gmm.c): expanded
 * sgemm forms, its float / double roundings and its slice order for nt > 1.
 * orc_gmm_compute_p follows gmm_compute_p_thread (854-870); orc_gmm_learn
 * follows gmm_learn (436-502) with the port-mode k-means; returns -1 where
 * the reference would assert or loop for ever in gmm_handle_empty. */
void orc_gmm_compute_p(int n, const float *v, int d, int k, const float *w, const float *mu,
                       const float *sigma, float *p, int flags, int nt);
int orc_gmm_learn(int d, int n, int k, int niter, const float *v, int nt, int seed, int nredo,
                  int flags, float *w, float *mu, float *sigma, int *iters_out);
/* one EM iteration of orc_gmm_learn on the given mixture, in place */
int orc_gmm_em_step(int n, const float *v, int d, int k, float *w, float *mu, float *sigma,
                    int flags, int nt);

/* RNG pieces, exposed so the tests can compare them with the GPU library's. */
double orc_gaussrand_r(unsigned int *seed);
void orc_random_init(int n, int k, unsigned int seed, int *sel);

#ifdef __cplusplus
}
#endif
#endif
