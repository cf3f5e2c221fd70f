// yael_knn: exact k-NN between two vector files, the command-line program of
// yael's progs/knn.c (same options, defaults, formats and outputs) on the GPU
// library: knn_full_thread, then knn_reorder_shortlist, as there.  The
// distance pass is chosen with YAEL_GPU_PRECISION (default fp32; bf16 gives
// the same ids).
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/yael_gpu.h"

namespace {

enum Fmt { FVEC, IVEC, BVEC, TEXT };

void usage(const char *cmd) {
  printf("Usage: %s [options]\n", cmd);
  printf(
      "  Input\n"
      "    -b filename    database to be searched (fvec file format)\n"
      "    -bb filename   database to be searched (bvec format)\n"
      "    -bt filename   database to be searched (text format)\n"
      "    -q filename    query vectors (file in fvec format)\n"
      "    -qb filename   query vectors (file in bvec format)\n"
      "    -qt filename   query vectors (text format)\n"
      "    -nb #          use the first n database vectors (default: all)\n"
      "    -nq #          use the first n query vectors (default: all)\n"
      "    -d #           dimension of the vector (used with the text format only)\n"
      "  Search parameters\n"
      "    -k #           number of nearest neighbors to retrieve (default: 10)\n"
      "    -nt #          number of threads (accepted, the search runs on the GPU)\n"
      "  Output\n"
      "    -onn idxfile   file (fmt=ivec) of k-NN indexes, 1 vec/query (default: nn.out)\n"
      "    -onnt idxfile  same as onn but in text format\n"
      "    -odis disfile  square distances to k-NN, 1 vec/query (default: dis.out)\n"
      "    -odist disfile same as dis but output in text format\n"
      "  Others:\n"
      "    -verbose       more messages\n"
      "    -silence       fewer messages\n\n"
      "Remark: in text format, all the parameters nb, nq and d must be defined\n");
  exit(0);
}

[[noreturn]] void die(const char *msg, const char *arg) {
  fprintf(stderr, "yael_knn: %s%s%s\n", msg, arg ? " " : "", arg ? arg : "");
  exit(1);
}

// n x d floats from a file (fvec, bvec or whitespace-separated text); n = 0 or
// d = 0 on entry: the file's own count / dimension.  NaN values become 2, as
// the reference program does (progs/knn.c: fvec_purge_nans).
float *read_vectors(const char *fname, Fmt fmt, int verbose, int *nptr, int *dptr) {
  int n = *nptr, d = *dptr, ret = -1;
  float *v = nullptr;
  if (fmt == FVEC || fmt == BVEC) {
    int fd, fn;
    const long bytes = fmt == FVEC ? fvecs_fsize(fname, &fd, &fn) : bvecs_fsize(fname, &fd, &fn);
    if (bytes < 0) die("cannot read", fname);
    if (d == 0 || n == 0) {
      fprintf(stderr, "File %s contains (%ld bytes) %d vectors of dimension %d\n", fname, bytes,
              fn, fd);
      if (d == 0) d = fd;
      if (n == 0) n = fn;
    }
    if (fd != d) die("vectors of another dimension in", fname);
    if (n > fn) die("fewer vectors than asked in", fname);
    v = (float *)malloc(sizeof(float) * ((size_t)n * d + 1));
    ret = fmt == FVEC ? fvecs_read(fname, d, n, v) : b2fvecs_read(fname, d, n, v);
  } else {
    if (n == 0 || d == 0) die("text input needs -nb / -nq and -d:", fname);
    FILE *f = fopen(fname, "r");
    if (!f) die("cannot open", fname);
    v = (float *)malloc(sizeof(float) * ((size_t)n * d + 1));
    long i;
    for (i = 0; i < (long)n * d; i++)
      if (fscanf(f, "%f", v + i) != 1) break;
    fclose(f);
    ret = (int)(i / d);
  }
  if (ret < n) die("could not read all the vectors of", fname);
  long nnan = 0;
  for (long i = 0; i < (long)n * d; i++)
    if (isnan(v[i])) {
      v[i] = 2.f;
      nnan++;
    }
  if (nnan > 0 && verbose >= 1)
    fprintf(stderr, "found %ld NaN values in what read from %s\n", nnan, fname);
  *nptr = n;
  *dptr = d;
  return v;
}

}  // namespace

int main(int argc, char **argv) {
  int k = 10, d = 0, nb = 0, nq = 0, nt = 1, verbose = 1;
  Fmt fmt_b = FVEC, fmt_q = FVEC, fmt_nn = IVEC, fmt_dis = FVEC;
  const char *fb = nullptr, *fq = nullptr, *fnn = "nn.out", *fdis = "dis.out";
  if (argc == 1) usage(argv[0]);
  for (int i = 1; i < argc; i++) {
    const char *a = argv[i];
    const bool more = i + 1 < argc;
    auto num = [&](int *dst) {
      if (sscanf(argv[++i], "%d", dst) != 1) die("not a number:", argv[i]);
    };
    if (!strcmp(a, "-h") || !strcmp(a, "--help")) usage(argv[0]);
    else if (!strcmp(a, "-silence")) verbose = 0;
    else if (!strcmp(a, "-verbose")) verbose = 2;
    else if (!strcmp(a, "-k") && more) num(&k);
    else if (!strcmp(a, "-d") && more) num(&d);
    else if (!strcmp(a, "-nt") && more) num(&nt);
    else if (!strcmp(a, "-nb") && more) num(&nb);
    else if (!strcmp(a, "-nq") && more) num(&nq);
    else if (!strcmp(a, "-b") && more) { fb = argv[++i]; fmt_b = FVEC; }
    else if (!strcmp(a, "-bb") && more) { fb = argv[++i]; fmt_b = BVEC; }
    else if (!strcmp(a, "-bt") && more) { fb = argv[++i]; fmt_b = TEXT; }
    else if (!strcmp(a, "-q") && more) { fq = argv[++i]; fmt_q = FVEC; }
    else if (!strcmp(a, "-qb") && more) { fq = argv[++i]; fmt_q = BVEC; }
    else if (!strcmp(a, "-qt") && more) { fq = argv[++i]; fmt_q = TEXT; }
    else if (!strcmp(a, "-onn") && more) { fnn = argv[++i]; fmt_nn = IVEC; }
    else if (!strcmp(a, "-onnt") && more) { fnn = argv[++i]; fmt_nn = TEXT; }
    else if (!strcmp(a, "-odis") && more) { fdis = argv[++i]; fmt_dis = FVEC; }
    else if (!strcmp(a, "-odist") && more) { fdis = argv[++i]; fmt_dis = TEXT; }
  }
  if (!fb || !fq) die("a database (-b / -bb / -bt) and queries (-q / -qb / -qt) are needed", nullptr);
  fprintf(stderr, "k = %d\nd = %d\nnt = %d\n", k, d, nt);
  const char *names[] = {"fvec", "ivec", "bvec", "txt"};
  if (verbose) {
    fprintf(stderr, "fb = %s  (fmt = %s)\n", fb, names[fmt_b]);
    fprintf(stderr, "fq = %s  (fmt = %s)\n", fq, names[fmt_q]);
    fprintf(stderr, "fnn = %s  (fmt = %s)\n", fnn, names[fmt_nn]);
    fprintf(stderr, "fdis = %s  (fmt = %s)\n", fdis, names[fmt_dis]);
  }
  float *vb = read_vectors(fb, fmt_b, verbose, &nb, &d);
  float *vq = read_vectors(fq, fmt_q, verbose, &nq, &d);
  if (k > nb) die("k is larger than the database", nullptr);
  int *idx = (int *)malloc(sizeof(int) * ((size_t)k * nq + 1));
  float *dis = (float *)malloc(sizeof(float) * ((size_t)k * nq + 1));
  knn_full_thread(2, nq, nb, d, k, vb, vq, nullptr, idx, dis, nt);
  knn_reorder_shortlist(nq, nb, d, k, vb, vq, idx, dis);
  int ret;
  if (fmt_dis == FVEC) {
    ret = fvecs_write(fdis, k, nq, dis);
  } else {
    FILE *f = fopen(fdis, "w");
    if (!f) die("cannot write", fdis);
    for (int i = 0; i < nq; i++) {
      for (int j = 0; j < k; j++) fprintf(f, "%f ", dis[(long)i * k + j]);
      fprintf(f, "\n");
    }
    fclose(f);
    ret = nq;
  }
  if (ret != nq) die("could not write", fdis);
  if (fmt_nn == IVEC) {
    ret = ivecs_write(fnn, k, nq, idx);
  } else {
    FILE *f = fopen(fnn, "w");
    if (!f) die("cannot write", fnn);
    for (int i = 0; i < nq; i++) {
      for (int j = 0; j < k; j++) fprintf(f, "%d ", idx[(long)i * k + j]);
      fprintf(f, "\n");
    }
    fclose(f);
    ret = nq;
  }
  if (ret != nq) die("could not write", fnn);
  free(idx);
  free(dis);
  free(vb);
  free(vq);
  return 0;
}
