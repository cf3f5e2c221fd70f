// yael_kmeans: k-means of a vector file, the command-line program of yael's
// progs/kmeans.c (same options, defaults, formats and outputs) on the GPU
// library: the file readers and writers of include/yael_gpu.h and the drop-in
// kmeans().  The assignment pass is chosen with YAEL_GPU_PRECISION (default
// fp32; bf16 gives the same assignments).
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include "../../include/yael_gpu.h"

namespace {

const int kDefaultNiter = 40;
const int kDefaultNredo = 1;

void usage(const char *cmd) {
  printf("Usage: %s [options]\n", cmd);
  printf(
      "  Input\n"
      "    -i filename     input set of vectors to cluster (fvec file format)\n"
      "    -itxt filename  the same but for an input text file\n"
      "    -n #            use n points from the file. Default: all the vectors\n"
      "    -d #            dimension of the vector (used with -itxt only)\n"
      "  Clustering parameters\n"
      "    -k #            number of centroids to produce\n"
      "    -niter #        maximum number of iterations. Default: %d\n"
      "    -nredo #        number of runs to perform. Default: %d\n"
      "    -seed #         initialize the random generate with a number\n"
      "    -nt #           number of threads (accepted, the clustering runs on the GPU)\n"
      "  Ouput\n"
      "    -o clustfile    output cluster file (fvec format)\n"
      "    -otxt clustfile output cluster file (text format)\n",
      kDefaultNiter, kDefaultNredo);
  exit(0);
}

[[noreturn]] void die(const char *msg, const char *arg) {
  fprintf(stderr, "yael_kmeans: %s%s%s\n", msg, arg ? " " : "", arg ? arg : "");
  exit(1);
}

}  // namespace

int main(int argc, char **argv) {
  int k = 10, d = 0, n = 0, niter = kDefaultNiter, nredo = kDefaultNredo, seed = 0;
  long ncpu = sysconf(_SC_NPROCESSORS_ONLN);
  int nt = ncpu > 0 ? (int)ncpu : 1;
  bool txt_in = false, txt_out = false;
  const char *fi = nullptr, *fo = nullptr;
  if (argc == 1) usage(argv[0]);
  for (int i = 1; i < argc; i++) {
    const char *a = argv[i];
    const bool more = i + 1 < argc;
    auto num = [&](int *dst) {
      if (sscanf(argv[++i], "%d", dst) != 1) die("not a number:", argv[i]);
    };
    if (!strcmp(a, "-h") || !strcmp(a, "--help")) usage(argv[0]);
    else if (!strcmp(a, "-k") && more) num(&k);
    else if (!strcmp(a, "-d") && more) num(&d);
    else if (!strcmp(a, "-n") && more) num(&n);
    else if (!strcmp(a, "-niter") && more) num(&niter);
    else if (!strcmp(a, "-nt") && more) num(&nt);
    else if (!strcmp(a, "-nredo") && more) num(&nredo);
    else if (!strcmp(a, "-seed") && more) num(&seed);
    else if (!strcmp(a, "-i") && more) { fi = argv[++i]; txt_in = false; }
    else if (!strcmp(a, "-itxt") && more) { fi = argv[++i]; txt_in = true; }
    else if (!strcmp(a, "-o") && more) { fo = argv[++i]; txt_out = false; }
    else if (!strcmp(a, "-otxt") && more) { fo = argv[++i]; txt_out = true; }
  }
  if (!fi || !fo) die("an input (-i / -itxt) and an output (-o / -otxt) are needed", nullptr);
  fprintf(stderr, "k = %d\nd = %d\nn = %d\nniter = %d\nnredo = %d\n", k, d, n, niter, nredo);
  fprintf(stderr, "nt = %d\nseed = %d\n", nt, seed);
  fprintf(stderr, "fi = %s  (fmt = %s)\n", fi, txt_in ? "txt" : "fvec");
  fprintf(stderr, "fo = %s  (fmt = %s)\n", fo, txt_out ? "txt" : "fvec");

  float *v = nullptr;
  int ret;
  if (!txt_in) {
    int fd, fn;
    const long bytes = fvecs_fsize(fi, &fd, &fn);
    if (bytes < 0) die("cannot read", fi);
    if (d == 0 || n == 0) {
      fprintf(stderr, "File %s contains (%ld bytes) %d vectors of dimension %d\n", fi, bytes, fn,
              fd);
      if (d == 0) d = fd;
      if (n == 0) n = fn;
    }
    if (fd != d) die("vectors of another dimension in", fi);
    if (n > fn) die("fewer vectors than asked in", fi);
    v = (float *)malloc(sizeof(float) * ((size_t)n * d + 1));
    ret = fvecs_read(fi, d, n, v);
  } else {
    if (n == 0 || d == 0) die("text input needs -n and -d:", fi);
    v = (float *)malloc(sizeof(float) * ((size_t)n * d + 1));
    ret = fvecs_read_txt(fi, d, n, v);
  }
  if (ret < n) die("could not read all the vectors of", fi);
  if (k > n) die("k is larger than the number of vectors", nullptr);

  long nnan = 0;  // fvec_purge_nans(v, n * d, 2) of the reference program
  for (long i = 0; i < (long)n * d; i++)
    if (isnan(v[i])) {
      v[i] = 2.f;
      nnan++;
    }
  if (nnan > 0) fprintf(stderr, "found %ld NaN values\n", nnan);

  float *centroids = (float *)malloc(sizeof(float) * ((size_t)k * d + 1));
  int *nassign = (int *)malloc(sizeof(int) * ((size_t)k + 1));
  kmeans(d, n, k, niter, v, nt, seed, nredo, centroids, nullptr, nullptr, nassign);

  ret = txt_out ? fvecs_write_txt(fo, d, k, centroids) : fvecs_write(fo, d, k, centroids);
  if (ret != k) die("could not write", fo);
  free(centroids);
  free(nassign);
  free(v);
  return 0;
}
