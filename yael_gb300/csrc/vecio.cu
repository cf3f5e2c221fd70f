// Vector file formats of yael (yael/vector.c:591-1590, doc/file_format.rst):
// a file is a sequence of records, each an int32 dimension d followed by d
// elements (float for .fvecs, int32 for .ivecs, uint8 for .bvecs).  Host code:
// the same readers and writers, return values and error behaviour as the
// reference's, so that its command-line programs and callers can use them
// unchanged.  Arrays returned by the *_new_* readers are malloc'd (free()).
#include <errno.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/yael_gpu.h"

namespace {

// one record: d, then d elements of `unit` bytes; 0 ok, -1 / -2 write errors
int rec_write(FILE *f, const void *v, int d, size_t unit, const char *who) {
  if (fwrite(&d, sizeof(int), 1, f) != 1) {
    perror(who);
    return -1;
  }
  if (fwrite(v, unit, (size_t)d, f) != (size_t)d) {
    perror(who);
    return -2;
  }
  return 0;
}

// the number of records (all of the first record's dimension) of a file
long file_shape(size_t unit, const char *fname, int *d_out, int *n_out) {
  *d_out = -1;
  *n_out = -1;
  FILE *f = fopen(fname, "r");
  if (!f) {
    fprintf(stderr, "vecs_fsize %s: %s\n", fname, strerror(errno));
    return -1;
  }
  int d;
  if (fread(&d, sizeof(int), 1, f) != 1) {  // empty file
    fclose(f);
    *n_out = 0;
    return 0;
  }
  fseek(f, 0, SEEK_END);
  const long bytes = ftell(f);
  fclose(f);
  const long rec = (long)unit * d + 4;
  if (d < 0 || rec <= 0 || bytes % rec != 0) {
    fprintf(stderr, "vecs_fsize %s: file size %ld does not fit records of dimension %d\n",
            fname, bytes, d);
    return -1;
  }
  *d_out = d;
  *n_out = (int)(bytes / rec);
  return bytes;
}

// one record into v (at most d_alloc elements): its dimension, 0 at end of
// file, -1 on error
int rec_read(FILE *f, void *v, int d_alloc, size_t unit) {
  int d;
  const size_t got = fread(&d, sizeof(int), 1, f);
  if (feof(f)) return 0;
  if (got != 1) {
    perror("vec_fread");
    return -1;
  }
  if (d < 0 || d > d_alloc) {
    fprintf(stderr, "vec_fread: vector of dimension %d, room for %d\n", d, d_alloc);
    return -1;
  }
  if (fread(v, unit, (size_t)d, f) != (size_t)d) {
    perror("vec_fread");
    return -1;
  }
  return d;
}

// up to n records of dimension d_alloc into v: the number read (0 on error)
long recs_read(FILE *f, void *v, long n, int d_alloc, size_t unit) {
  long i;
  int d = -1;
  for (i = 0; i < n; i++) {
    const int r = rec_read(f, (char *)v + unit * (size_t)i * d_alloc, d_alloc, unit);
    if (r == 0) break;
    if (r < 0) return 0;
    if (i == 0) {
      d = r;
      if (d != d_alloc)
        fprintf(stderr, "vecs_fread: room for dimension %d, found %d\n", d_alloc, d);
    }
    if (r != d) {
      fprintf(stderr, "vecs_fread: vectors of different dimensions\n");
      return 0;
    }
  }
  return i;
}

// records of one dimension (4-byte elements) into a growing malloc'd array:
// at most nmax (< 0: all); the count, -1 on error (then *out = NULL, *d_out = -1)
int recs4_new_read(FILE *f, int *d_out, void **out, long nmax) {
  long n, cap = 0;
  int d = -1;
  char *buf = nullptr;
  for (n = 0; nmax < 0 || n < nmax; n++) {
    int dn;
    if (fread(&dn, sizeof(int), 1, f) != 1) {
      if (feof(f)) break;
      perror("vecs_new_read");
      goto fail;
    }
    if (n == 0) {
      d = dn;
    } else if (dn != d) {
      fprintf(stderr, "vecs_new_read: vectors of dimensions %d and %d\n", d, dn);
      goto fail;
    }
    if (d < 0) {
      fprintf(stderr, "vecs_new_read: negative dimension %d\n", d);
      goto fail;
    }
    if ((n + 1) * d > cap) {
      long nc = cap ? cap : 1024;
      while ((n + 1) * d > nc) nc *= 2;
      char *nb = (char *)realloc(buf, (size_t)nc * 4);
      if (!nb) {
        fprintf(stderr, "vecs_new_read: out of memory\n");
        goto fail;
      }
      buf = nb;
      cap = nc;
    }
    if (fread(buf + (size_t)n * d * 4, 4, (size_t)d, f) != (size_t)d) {
      fprintf(stderr, "vecs_new_read: truncated record\n");
      goto fail;
    }
  }
  if (buf && n * d > 0) {
    char *shrunk = (char *)realloc(buf, (size_t)n * d * 4);
    if (shrunk) buf = shrunk;
  }
  *out = buf;
  *d_out = d;
  return (int)n;
fail:
  free(buf);
  *out = nullptr;
  *d_out = -1;
  return -1;
}

}  // namespace

extern "C" {

int fvec_fwrite(FILE *f, const float *v, int d) { return rec_write(f, v, d, 4, "fvec_fwrite"); }
int ivec_fwrite(FILE *f, const int *v, int d) { return rec_write(f, v, d, 4, "ivec_fwrite"); }
int bvec_fwrite(FILE *f, const unsigned char *v, int d) {
  return rec_write(f, v, d, 1, "bvec_fwrite");
}

int fvecs_fwrite(FILE *f, int d, int n, const float *v) {
  for (int i = 0; i < n; i++)
    if (fvec_fwrite(f, v + (long)i * d, d) < 0) return i;
  return n;
}

int ivecs_fwrite(FILE *f, int d, int n, const int *v) {
  for (int i = 0; i < n; i++) ivec_fwrite(f, v + (long)i * d, d);
  return n;
}

int bvecs_fwrite(FILE *f, int d, int n, const unsigned char *v) {
  for (int i = 0; i < n; i++) bvec_fwrite(f, v + (long)i * d, d);
  return n;
}

int fvecs_write(const char *fname, int d, int n, const float *v) {
  FILE *f = fopen(fname, "w");
  if (!f) {
    fprintf(stderr, "fvecs_write: cannot open %s: %s\n", fname, strerror(errno));
    return -1;
  }
  const int r = fvecs_fwrite(f, d, n, v);
  fclose(f);
  return r;
}

int ivecs_write(const char *fname, int d, int n, const int *v) {
  FILE *f = fopen(fname, "w");
  if (!f) {
    perror("ivecs_write");
    return -1;
  }
  const int r = ivecs_fwrite(f, d, n, v);
  fclose(f);
  return r;
}

int bvecs_write(const char *fname, int d, int n, const unsigned char *v) {
  FILE *f = fopen(fname, "w");
  if (!f) {
    perror("bvecs_write");
    return -1;
  }
  const int r = bvecs_fwrite(f, d, n, v);
  fclose(f);
  return r;
}

long fvecs_fsize(const char *fname, int *d_out, int *n_out) {
  return file_shape(4, fname, d_out, n_out);
}
long ivecs_fsize(const char *fname, int *d_out, int *n_out) {
  return file_shape(4, fname, d_out, n_out);
}
long bvecs_fsize(const char *fname, int *d_out, int *n_out) {
  return file_shape(1, fname, d_out, n_out);
}

int fvec_fread(FILE *f, float *v, int d_alloc) { return rec_read(f, v, d_alloc, 4); }
int ivec_fread(FILE *f, int *v, int d_alloc) { return rec_read(f, v, d_alloc, 4); }
int bvec_fread(FILE *f, unsigned char *v, int d_alloc) { return rec_read(f, v, d_alloc, 1); }

long fvecs_fread(FILE *f, float *v, long n, int d_alloc) { return recs_read(f, v, n, d_alloc, 4); }
long ivecs_fread(FILE *f, int *v, long n, int d_alloc) { return recs_read(f, v, n, d_alloc, 4); }
long bvecs_fread(FILE *f, unsigned char *v, long n, int d_alloc) {
  return recs_read(f, v, n, d_alloc, 1);
}

int fvecs_new_fread_max(FILE *f, int *d_out, float **vf_out, long nmax) {
  return recs4_new_read(f, d_out, (void **)vf_out, nmax);
}
int ivecs_new_fread_max(FILE *f, int *d_out, int **vi_out, long nmax) {
  return recs4_new_read(f, d_out, (void **)vi_out, nmax);
}

int fvecs_new_read(const char *fname, int *d_out, float **vf_out) {
  FILE *f = fopen(fname, "r");
  if (!f) {
    fprintf(stderr, "fvecs_new_read: could not open %s: %s\n", fname, strerror(errno));
    *d_out = -1;
    return -1;
  }
  const int n = fvecs_new_fread_max(f, d_out, vf_out, -1);
  fclose(f);
  return n;
}

int ivecs_new_read(const char *fname, int *d_out, int **vi_out) {
  FILE *f = fopen(fname, "r");
  if (!f) {
    fprintf(stderr, "ivecs_new_read: could not open %s: %s\n", fname, strerror(errno));
    *d_out = -1;
    *vi_out = nullptr;
    return -1;
  }
  const int n = ivecs_new_fread_max(f, d_out, vi_out, -1);
  fclose(f);
  return n;
}

int fvecs_read(const char *fname, int d, int n, float *v) {
  FILE *f = fopen(fname, "r");
  if (!f) {
    fprintf(stderr, "fvecs_read: could not open %s: %s\n", fname, strerror(errno));
    return -1;
  }
  long i;
  for (i = 0; i < n; i++) {
    int dn;
    if (fread(&dn, sizeof(int), 1, f) != 1) {
      if (feof(f)) break;
      perror("fvecs_read");
      fclose(f);
      return -1;
    }
    if (dn != d) {
      fprintf(stderr, "fvecs_read: vector of dimension %d, expected %d\n", dn, d);
      fclose(f);
      return -1;
    }
    if (fread(v + (long)d * i, sizeof(float), (size_t)d, f) != (size_t)d) {
      fprintf(stderr, "fvecs_read: truncated record\n");
      fclose(f);
      return -1;
    }
  }
  fclose(f);
  return (int)i;
}

int bvecs_new_read(const char *fname, int *d_out, unsigned char **v_out) {
  int n, d;
  if (file_shape(1, fname, &d, &n) < 0) {
    *d_out = -1;
    *v_out = nullptr;
    return -1;
  }
  FILE *f = fopen(fname, "r");
  if (!f) {
    fprintf(stderr, "bvecs_new_read: cannot open %s: %s\n", fname, strerror(errno));
    *d_out = -1;
    *v_out = nullptr;
    return -1;
  }
  unsigned char *v = (unsigned char *)malloc((size_t)n * (d > 0 ? d : 0) + 1);
  recs_read(f, v, n, d, 1);
  fclose(f);
  *d_out = d;
  *v_out = v;
  return n;
}

// n records of a .bvecs file, converted to float
static long b2f_read(FILE *f, float *v, long n, int d) {
  unsigned char *row = (unsigned char *)malloc(d > 0 ? (size_t)d : 1);
  long i;
  for (i = 0; i < n; i++) {
    const int r = rec_read(f, row, d, 1);
    if (r != d) break;
    for (int c = 0; c < d; c++) v[i * d + c] = (float)row[c];
  }
  free(row);
  return i;
}

int b2fvecs_read(const char *fname, int d, int n, float *v) {
  int dn, nn;
  if (bvecs_fsize(fname, &dn, &nn) < 0 || dn != d || n > nn) {
    fprintf(stderr, "b2fvecs_read: %s holds %d vectors of dimension %d, asked %d of %d\n",
            fname, nn, dn, n, d);
    return -1;
  }
  FILE *f = fopen(fname, "r");
  if (!f) return -1;
  b2f_read(f, v, n, d);
  fclose(f);
  return n;
}

int b2fvecs_new_read(const char *fname, int *d_out, float **v_out) {
  int n, d;
  if (bvecs_fsize(fname, &d, &n) < 0) {
    *d_out = -1;
    *v_out = nullptr;
    return -1;
  }
  float *v = (float *)malloc(sizeof(float) * ((size_t)n * (d > 0 ? d : 0) + 1));
  FILE *f = fopen(fname, "r");
  if (!f) {
    free(v);
    *d_out = -1;
    *v_out = nullptr;
    return -1;
  }
  b2f_read(f, v, n, d);
  fclose(f);
  *v_out = v;
  *d_out = d;
  return n;
}

// Raw vectors (yael/vector.c:1149-1250, 1386-1445): d elements with no
// dimension header.  Where the reference frees the caller's buffer on a short
// read (fvec_fread_raw & co.) these leave it alone; where it asserts or hands a
// null FILE to fread on an unopenable file these print and return -1 / NULL.
static int raw_fwrite(FILE *f, const void *v, long d, size_t unit, const char *who) {
  if (fwrite(v, unit, (size_t)d, f) != (size_t)d) {
    perror(who);
    return -1;
  }
  return 0;
}

static int raw_fread(FILE *f, void *v, long n, size_t unit, const char *who) {
  if (fread(v, unit, (size_t)n, f) != (size_t)n) {
    perror(who);
    return -1;
  }
  return (int)n;
}

static void *raw_new_fread(FILE *f, long d, size_t unit, const char *who) {
  void *v = malloc(unit * (size_t)(d > 0 ? d : 0) + 1);
  if (raw_fread(f, v, d, unit, who) < 0) {
    free(v);
    return nullptr;
  }
  return v;
}

static void *raw_new_read(const char *fname, long d, size_t unit, const char *who) {
  FILE *f = fopen(fname, "r");
  if (!f) {
    fprintf(stderr, "%s: cannot open %s: %s\n", who, fname, strerror(errno));
    return nullptr;
  }
  void *v = raw_new_fread(f, d, unit, who);
  fclose(f);
  return v;
}

static int raw_write(const char *fname, const void *v, long d, size_t unit, const char *who) {
  FILE *f = fopen(fname, "w");
  if (!f) {
    fprintf(stderr, "%s: cannot open %s: %s\n", who, fname, strerror(errno));
    return -1;
  }
  const int r = raw_fwrite(f, v, d, unit, who);
  fclose(f);
  return r;
}

int fvec_fwrite_raw(FILE *f, const float *v, long d) {
  return raw_fwrite(f, v, d, 4, "fvec_fwrite_raw");
}
int ivec_fwrite_raw(FILE *f, const int *v, long d) {
  return raw_fwrite(f, v, d, 4, "ivec_fwrite_raw");
}
int bvec_fwrite_raw(FILE *f, const unsigned char *v, long d) {
  return raw_fwrite(f, v, d, 1, "bvec_fwrite_raw");
}
int fvec_write_raw(const char *fname, const float *v, long d) {
  return raw_write(fname, v, d, 4, "fvec_write_raw");
}
int ivec_write_raw(const char *fname, const int *v, long d) {
  return raw_write(fname, v, d, 4, "ivec_write_raw");
}
int bvec_write_raw(const char *fname, const unsigned char *v, long d) {
  return raw_write(fname, v, d, 1, "bvec_write_raw");
}
int fvec_fread_raw(FILE *f, float *v, long n) { return raw_fread(f, v, n, 4, "fvec_fread_raw"); }
int ivec_fread_raw(FILE *f, int *v, long n) { return raw_fread(f, v, n, 4, "ivec_fread_raw"); }
int bvec_fread_raw(FILE *f, unsigned char *v, long n) {
  return raw_fread(f, v, n, 1, "bvec_fread_raw");
}
float *fvec_new_fread_raw(FILE *f, long d) {
  return (float *)raw_new_fread(f, d, 4, "fvec_new_fread_raw");
}
int *ivec_new_fread_raw(FILE *f, long d) {
  return (int *)raw_new_fread(f, d, 4, "ivec_new_fread_raw");
}
unsigned char *bvec_new_fread_raw(FILE *f, long d) {
  return (unsigned char *)raw_new_fread(f, d, 1, "bvec_new_fread_raw");
}
float *fvec_new_read_raw(const char *fname, long d) {
  return (float *)raw_new_read(fname, d, 4, "fvec_new_read_raw");
}
int *ivec_new_read_raw(const char *fname, long d) {
  return (int *)raw_new_read(fname, d, 4, "ivec_new_read_raw");
}
unsigned char *bvec_new_read_raw(const char *fname, long d) {
  return (unsigned char *)raw_new_read(fname, d, 1, "bvec_new_read_raw");
}

// Text vectors (yael/vector.c:939-964, 1279-1294, 1475-1491): one line per
// vector, each element followed by a space ("%d " / "%f "); the writers return
// the characters of the line ends written (n), the reader the number of whole
// vectors read (elements read / d).  The writers close their file (the
// reference leaves it open until exit).
int ivecs_write_txt(const char *fname, int d, int n, const int *v) {
  FILE *f = fopen(fname, "w");
  if (!f) {
    perror("ivecs_write_txt: cannot open file");
    return -1;
  }
  int ret = 0;
  for (long i = 0; i < n; i++) {
    for (long j = 0; j < d; j++) fprintf(f, "%d ", v[i * d + j]);
    ret += fprintf(f, "\n");
  }
  fclose(f);
  return ret;
}

int fvecs_write_txt(const char *fname, int d, int n, const float *v) {
  FILE *f = fopen(fname, "w");
  if (!f) {
    perror("fvecs_write_txt: cannot open file");
    return -1;
  }
  int ret = 0;
  for (long i = 0; i < n; i++) {
    for (long j = 0; j < d; j++) fprintf(f, "%f ", (double)v[i * d + j]);
    ret += fprintf(f, "\n");
  }
  fclose(f);
  return ret;
}

int fvecs_read_txt(const char *fname, int d, int n, float *v) {
  FILE *f = fopen(fname, "r");
  if (!f) {
    fprintf(stderr, "fvecs_read_txt: could not open %s: %s\n", fname, strerror(errno));
    return -1;
  }
  if (d <= 0) {
    fclose(f);
    return 0;
  }
  long i;
  const long total = (long)n * d;
  for (i = 0; i < total; i++) {
    if (fscanf(f, "%f", v + i) != 1) {
      if (feof(f)) break;
      perror("fvecs_read_txt");
      fclose(f);
      return -1;
    }
  }
  fclose(f);
  return (int)(i / d);
}

}  // extern "C"
