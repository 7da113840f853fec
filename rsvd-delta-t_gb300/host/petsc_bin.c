/* PETSc binary Mat/Vec files (the reference's file interface, MatLoad /
 * MatView / VecLoad / VecView through PetscViewerBinary, e.g.
 * SourceCode/LNSStructure.c:23-26, SourceCode/SaveResults.c:32-85).
 *
 * Throughput: every region of a file (row lengths, column indices, values)
 * is read with large fread calls straight into its destination array and
 * byte-swapped there by all host threads (OpenMP), so a file is read once
 * with no staging copy of its whole contents; the writers convert blocks of
 * entries in parallel into a 32 MB buffer and write each block with one
 * fwrite. Big-endian on disk; PetscInt is int32 or int64 (detected from the
 * class id); scalars are complex128. */
#include "petsc_bin.h"

#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define MAT_CLASSID 1211216
#define VEC_CLASSID 1211214
#define IO_CHUNK ((size_t)1 << 28) /* bytes per fread call */
#define WBUF ((size_t)32 << 20)    /* bytes per write block */

static int fail(char *err, int errlen, const char *fmt, ...) {
  if (err && errlen > 0) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(err, (size_t)errlen, fmt, ap);
    va_end(ap);
  }
  return -1;
}

static uint64_t be64(const unsigned char *p) {
  uint64_t v = 0;
  for (int i = 0; i < 8; ++i) v = (v << 8) | p[i];
  return v;
}

static uint32_t be32(const unsigned char *p) {
  return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | (uint32_t)p[3];
}

static void put64(unsigned char *p, uint64_t v) {
  for (int i = 7; i >= 0; --i) {
    p[i] = (unsigned char)(v & 0xff);
    v >>= 8;
  }
}

/* Big-endian 64-bit words in place <-> host order (the host is
 * little-endian on both machines this builds for; the swap is its own
 * inverse). */
static void swap64_inplace(uint64_t *a, int64_t n) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) a[i] = __builtin_bswap64(a[i]);
}

static int read_all(FILE *f, void *dst, size_t bytes) {
  unsigned char *p = (unsigned char *)dst;
  while (bytes > 0) {
    const size_t n = bytes < IO_CHUNK ? bytes : IO_CHUNK;
    if (fread(p, 1, n, f) != n) return -1;
    p += n;
    bytes -= n;
  }
  return 0;
}

static long file_size(FILE *f) {
  if (fseek(f, 0, SEEK_END) != 0) return -1;
  const long n = ftell(f);
  fseek(f, 0, SEEK_SET);
  return n;
}

/* Header: class id and `count` PetscInts after it, in the width the class
 * id reveals (4 or 8); returns the width, or 0. */
static int read_header(FILE *f, long len, uint32_t classid, int64_t *vals, int count) {
  unsigned char h[40];
  const size_t need4 = (size_t)4 * (count + 1), need8 = (size_t)8 * (count + 1);
  if (len < (long)need4 || fread(h, 1, need4, f) != need4) return 0;
  int w = 0;
  if (be32(h) == classid) {
    w = 4;
  } else if (len >= (long)need8 && fread(h + need4, 1, need8 - need4, f) == need8 - need4 && be64(h) == classid) {
    w = 8;
  }
  if (!w) return 0;
  for (int i = 0; i < count; ++i)
    vals[i] = w == 4 ? (int64_t)(int32_t)be32(h + 4 * (i + 1)) : (int64_t)be64(h + 8 * (i + 1));
  if (fseek(f, (long)(w * (count + 1)), SEEK_SET) != 0) return 0;
  return w;
}

/* n PetscInts of width w from f into out (int64). */
static int read_ints(FILE *f, int w, int64_t n, int64_t *out) {
  if (n <= 0) return 0;
  if (w == 8) {
    if (read_all(f, out, sizeof(int64_t) * (size_t)n)) return -1;
    swap64_inplace((uint64_t *)out, n);
    return 0;
  }
  uint32_t *tmp = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)n);
  if (!tmp) return -1;
  if (read_all(f, tmp, sizeof(uint32_t) * (size_t)n)) {
    free(tmp);
    return -1;
  }
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) out[i] = (int64_t)(int32_t)__builtin_bswap32(tmp[i]);
  free(tmp);
  return 0;
}

int pb_read_mat(const char *path, pb_csr *m, char *err, int errlen) {
  memset(m, 0, sizeof *m);
  FILE *f = fopen(path, "rb");
  if (!f) return fail(err, errlen, "cannot open %s", path);
  const long len = file_size(f);
  int64_t hv[3];
  const int w = read_header(f, len, MAT_CLASSID, hv, 3);
  if (!w) {
    fclose(f);
    return fail(err, errlen, "%s is not a PETSc binary matrix", path);
  }
  int64_t M = hv[0], N = hv[1], nz = hv[2];
  if (M < 0 || N < 0) {
    fclose(f);
    return fail(err, errlen, "%s: negative matrix size", path);
  }
  const int dense = nz == -1;
  if (dense) nz = M * N;
  const size_t need = (size_t)w * 4 + (dense ? 0 : (size_t)w * (size_t)(M + nz)) + (size_t)16 * nz;
  if (nz < 0 || (long)need > len) {
    fclose(f);
    return fail(err, errlen, "%s: file truncated", path);
  }
  m->rows = M;
  m->cols = N;
  m->nnz = nz;
  m->rowptr = (int64_t *)calloc((size_t)M + 1, sizeof(int64_t));
  m->col = (int64_t *)malloc(sizeof(int64_t) * (nz > 0 ? (size_t)nz : 1));
  m->val = (double *)malloc(sizeof(double) * 2 * (nz > 0 ? (size_t)nz : 1));
  if (!m->rowptr || !m->col || !m->val) {
    fclose(f);
    pb_free(m);
    return fail(err, errlen, "out of memory reading %s", path);
  }
  if (dense) {
    for (int64_t i = 0; i <= M; ++i) m->rowptr[i] = i * N;
#pragma omp parallel for schedule(static)
    for (int64_t j = 0; j < nz; ++j) m->col[j] = j % (N > 0 ? N : 1);
  } else {
    /* Row lengths land in rowptr[1..M], then a prefix sum. */
    if (read_ints(f, w, M, m->rowptr + 1)) {
      fclose(f);
      pb_free(m);
      return fail(err, errlen, "%s: file truncated", path);
    }
    int64_t s = 0;
    for (int64_t i = 1; i <= M; ++i) {
      if (m->rowptr[i] < 0) {
        fclose(f);
        pb_free(m);
        return fail(err, errlen, "%s: negative row length", path);
      }
      s += m->rowptr[i];
      m->rowptr[i] = s;
    }
    if (s != nz) {
      fclose(f);
      pb_free(m);
      return fail(err, errlen, "%s: row lengths sum to %lld, header says %lld", path, (long long)s, (long long)nz);
    }
    if (read_ints(f, w, nz, m->col)) {
      fclose(f);
      pb_free(m);
      return fail(err, errlen, "%s: file truncated", path);
    }
    int64_t bad = 0;
#pragma omp parallel for schedule(static) reduction(+ : bad)
    for (int64_t j = 0; j < nz; ++j) bad += (m->col[j] < 0 || m->col[j] >= N);
    if (bad) {
      fclose(f);
      pb_free(m);
      return fail(err, errlen, "%s: column index out of range", path);
    }
  }
  if (read_all(f, m->val, sizeof(double) * 2 * (size_t)nz)) {
    fclose(f);
    pb_free(m);
    return fail(err, errlen, "%s: file truncated", path);
  }
  fclose(f);
  swap64_inplace((uint64_t *)m->val, 2 * nz);
  return 0;
}

void pb_free(pb_csr *m) {
  free(m->rowptr);
  free(m->col);
  free(m->val);
  memset(m, 0, sizeof *m);
}

int pb_read_vec(const char *path, double **v, int64_t *n, char *err, int errlen) {
  FILE *f = fopen(path, "rb");
  if (!f) return fail(err, errlen, "cannot open %s", path);
  const long len = file_size(f);
  int64_t cnt = 0;
  const int w = read_header(f, len, VEC_CLASSID, &cnt, 1);
  if (!w) {
    fclose(f);
    return fail(err, errlen, "%s is not a PETSc binary vector", path);
  }
  if (cnt < 0 || (long)((size_t)2 * w + (size_t)16 * cnt) > len) {
    fclose(f);
    return fail(err, errlen, "%s: file truncated", path);
  }
  *v = (double *)malloc(sizeof(double) * 2 * (cnt > 0 ? (size_t)cnt : 1));
  if (!*v || read_all(f, *v, sizeof(double) * 2 * (size_t)cnt)) {
    fclose(f);
    free(*v);
    *v = NULL;
    return fail(err, errlen, "%s: cannot read the values", path);
  }
  fclose(f);
  swap64_inplace((uint64_t *)*v, 2 * cnt);
  *n = cnt;
  return 0;
}

/* Writes n 64-bit words produced by get(i) big-endian, in WBUF blocks
 * filled by all threads. */
typedef uint64_t (*word_fn)(const void *ctx, int64_t i);

static int write_words(FILE *f, int64_t n, word_fn get, const void *ctx) {
  const int64_t per = (int64_t)(WBUF / 8);
  uint64_t *buf = (uint64_t *)malloc(WBUF);
  if (!buf) return -1;
  int ok = 1;
  for (int64_t i0 = 0; i0 < n && ok; i0 += per) {
    const int64_t m = n - i0 < per ? n - i0 : per;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < m; ++i) buf[i] = __builtin_bswap64(get(ctx, i0 + i));
    ok = fwrite(buf, 8, (size_t)m, f) == (size_t)m;
  }
  free(buf);
  return ok ? 0 : -1;
}

typedef struct {
  const double *a;
  int64_t rows, cols, ld;
  int is_complex;
} dense_src;

static uint64_t w_rowlen(const void *c, int64_t i) {
  (void)i;
  return (uint64_t)((const dense_src *)c)->cols;
}

static uint64_t w_colidx(const void *c, int64_t i) { return (uint64_t)(i % ((const dense_src *)c)->cols); }

/* Word i of the values: entry (r, c) in row-major order, real then
 * imaginary part. */
static uint64_t w_value(const void *c, int64_t i) {
  const dense_src *d = (const dense_src *)c;
  const int64_t e = i >> 1, r = e / d->cols, col = e % d->cols;
  double x;
  if (d->is_complex)
    x = d->a[2 * (col * d->ld + r) + (i & 1)];
  else
    x = (i & 1) ? 0.0 : d->a[col * d->ld + r];
  uint64_t u;
  memcpy(&u, &x, 8);
  return u;
}

static int write_dense_impl(const char *path, const double *a, int64_t rows, int64_t cols, int64_t ld,
                            int is_complex, char *err, int errlen) {
  FILE *f = fopen(path, "wb");
  if (!f) return fail(err, errlen, "cannot create %s", path);
  unsigned char h[32];
  put64(h, MAT_CLASSID);
  put64(h + 8, (uint64_t)rows);
  put64(h + 16, (uint64_t)cols);
  put64(h + 24, (uint64_t)(rows * cols));
  int ok = fwrite(h, 1, 32, f) == 32;
  dense_src d = {a, rows, cols, ld, is_complex};
  if (ok && cols > 0) {
    ok = write_words(f, rows, w_rowlen, &d) == 0 && write_words(f, rows * cols, w_colidx, &d) == 0 &&
         write_words(f, 2 * rows * cols, w_value, &d) == 0;
  } else if (ok) {
    ok = write_words(f, rows, w_rowlen, &d) == 0;
  }
  if (fclose(f) != 0) ok = 0;
  return ok ? 0 : fail(err, errlen, "write error on %s", path);
}

int pb_write_dense(const char *path, const double *a, int64_t rows, int64_t cols, int64_t ld, char *err,
                   int errlen) {
  return write_dense_impl(path, a, rows, cols, ld, 1, err, errlen);
}

int pb_write_dense_real(const char *path, const double *a, int64_t rows, int64_t cols, int64_t ld, char *err,
                        int errlen) {
  return write_dense_impl(path, a, rows, cols, ld, 0, err, errlen);
}

typedef struct {
  const double *v;
  int is_complex;
} vec_src;

static uint64_t w_vec(const void *c, int64_t i) {
  const vec_src *s = (const vec_src *)c;
  const double x = s->is_complex ? s->v[i] : ((i & 1) ? 0.0 : s->v[i >> 1]);
  uint64_t u;
  memcpy(&u, &x, 8);
  return u;
}

int pb_write_vec(const char *path, const double *v, int64_t n, int is_complex, char *err, int errlen) {
  FILE *f = fopen(path, "wb");
  if (!f) return fail(err, errlen, "cannot create %s", path);
  unsigned char h[16];
  put64(h, VEC_CLASSID);
  put64(h + 8, (uint64_t)n);
  int ok = fwrite(h, 1, 16, f) == 16;
  vec_src s = {v, is_complex};
  if (ok) ok = write_words(f, 2 * n, w_vec, &s) == 0;
  if (fclose(f) != 0) ok = 0;
  return ok ? 0 : fail(err, errlen, "write error on %s", path);
}
