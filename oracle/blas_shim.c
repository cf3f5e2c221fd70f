/*
 * blas_shim.c -- test infrastructure (oracle), never part of the product path.
 *
 * yael calls the Fortran BLAS entry points sgemm_ / sgemv_ with 32-bit
 * integer arguments (compiled with -DFINTEGER=int; see yael/nn.c:30-38 and
 * configure.sh:53).  No system BLAS is installed on these machines, but the
 * numpy / scipy wheels bundle OpenBLAS with prefixed symbol names:
 *   scipy.libs/libscipy_openblas-*.so   -> scipy_sgemm_   (32-bit ints)
 *   numpy.libs/libscipy_openblas64_-*.so -> scipy_sgemm_64_ (64-bit ints)
 * This shim defines sgemm_ / sgemv_ and forwards to whichever of the two it
 * can dlopen (path from $YAEL_ORACLE_BLAS, else the path the Makefile found at
 * build time).  If neither loads it falls back to a plain triple loop and says
 * so once on stderr (correct results, slow; only the CPU timing changes).
 */
#include <dlfcn.h>
#include <stdio.h>
#include <stdlib.h>
#include <pthread.h>

#ifndef ORACLE_BLAS_PATH
#define ORACLE_BLAS_PATH ""
#endif

typedef int (*sgemm32_t)(const char *, const char *, const int *, const int *,
                         const int *, const float *, const float *, const int *,
                         const float *, const int *, const float *, float *,
                         const int *);
typedef int (*sgemv32_t)(const char *, const int *, const int *, const float *,
                         const float *, const int *, const float *, const int *,
                         const float *, float *, const int *);
typedef int (*sgemm64_t)(const char *, const char *, const long *, const long *,
                         const long *, const float *, const float *, const long *,
                         const float *, const long *, const float *, float *,
                         const long *);
typedef int (*sgemv64_t)(const char *, const long *, const long *, const float *,
                         const float *, const long *, const float *, const long *,
                         const float *, float *, const long *);

static sgemm32_t g_sgemm32;
static sgemv32_t g_sgemv32;
static sgemm64_t g_sgemm64;
static sgemv64_t g_sgemv64;
static const char *g_blas_name = "naive-c-loops";
static pthread_once_t g_once = PTHREAD_ONCE_INIT;

static void shim_load(void)
{
  const char *path = getenv("YAEL_ORACLE_BLAS");
  if (!path || !*path) path = ORACLE_BLAS_PATH;
  if (path && *path) {
    void *h = dlopen(path, RTLD_NOW | RTLD_LOCAL);
    if (h) {
      g_sgemm32 = (sgemm32_t)dlsym(h, "scipy_sgemm_");
      g_sgemv32 = (sgemv32_t)dlsym(h, "scipy_sgemv_");
      if (!g_sgemm32 || !g_sgemv32) {
        g_sgemm32 = NULL; g_sgemv32 = NULL;
        g_sgemm64 = (sgemm64_t)dlsym(h, "scipy_sgemm_64_");
        g_sgemv64 = (sgemv64_t)dlsym(h, "scipy_sgemv_64_");
        if (!g_sgemm64 || !g_sgemv64) { g_sgemm64 = NULL; g_sgemv64 = NULL; }
      }
      if (g_sgemm32 || g_sgemm64) g_blas_name = path;
    }
  }
  if (!g_sgemm32 && !g_sgemm64)
    fprintf(stderr, "[oracle blas shim] no OpenBLAS found, using plain C loops\n");
}

const char *oracle_blas_name(void)
{
  pthread_once(&g_once, shim_load);
  return g_blas_name;
}

static int is_t(const char *c) { return *c == 'T' || *c == 't' || *c == 'C' || *c == 'c'; }

/* column-major C(m,n) = alpha op(A)(m,kk) op(B)(kk,n) + beta C */
static void naive_sgemm(const char *ta, const char *tb, long m, long n, long kk,
                        float alpha, const float *a, long lda, const float *b,
                        long ldb, float beta, float *c, long ldc)
{
  long i, j, l;
  for (j = 0; j < n; j++)
    for (i = 0; i < m; i++) {
      float s = 0;
      for (l = 0; l < kk; l++) {
        float av = is_t(ta) ? a[l + i * lda] : a[i + l * lda];
        float bv = is_t(tb) ? b[j + l * ldb] : b[l + j * ldb];
        s += av * bv;
      }
      c[i + j * ldc] = alpha * s + (beta == 0 ? 0 : beta * c[i + j * ldc]);
    }
}

int sgemm_(const char *ta, const char *tb, const int *m, const int *n,
           const int *k, const float *alpha, const float *a, const int *lda,
           const float *b, const int *ldb, const float *beta, float *c,
           const int *ldc)
{
  pthread_once(&g_once, shim_load);
  if (g_sgemm32)
    return g_sgemm32(ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc);
  if (g_sgemm64) {
    long M = *m, N = *n, K = *k, LA = *lda, LB = *ldb, LC = *ldc;
    return g_sgemm64(ta, tb, &M, &N, &K, alpha, a, &LA, b, &LB, beta, c, &LC);
  }
  naive_sgemm(ta, tb, *m, *n, *k, *alpha, a, *lda, b, *ldb, *beta, c, *ldc);
  return 0;
}

int sgemv_(const char *trans, const int *m, const int *n, const float *alpha,
           const float *a, const int *lda, const float *x, const int *incx,
           const float *beta, float *y, const int *incy)
{
  pthread_once(&g_once, shim_load);
  if (g_sgemv32)
    return g_sgemv32(trans, m, n, alpha, a, lda, x, incx, beta, y, incy);
  if (g_sgemv64) {
    long M = *m, N = *n, LA = *lda, IX = *incx, IY = *incy;
    return g_sgemv64(trans, &M, &N, alpha, a, &LA, x, &IX, beta, y, &IY);
  }
  {
    /* y = alpha op(A) x + beta y, A column-major m x n */
    long M = *m, N = *n, i, j, rows = is_t(trans) ? N : M, cols = is_t(trans) ? M : N;
    for (i = 0; i < rows; i++) {
      float s = 0;
      for (j = 0; j < cols; j++) {
        float av = is_t(trans) ? a[j + i * (long)*lda] : a[i + j * (long)*lda];
        s += av * x[j * (long)*incx];
      }
      y[i * (long)*incy] = *alpha * s + (*beta == 0 ? 0 : *beta * y[i * (long)*incy]);
    }
  }
  return 0;
}
