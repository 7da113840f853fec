#include "petsc_bin.h"

#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define MAT_CLASSID 1211216
#define VEC_CLASSID 1211214

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

static double bedouble(const unsigned char *p) {
  uint64_t u = be64(p);
  double d;
  memcpy(&d, &u, sizeof d);
  return d;
}

static unsigned char *slurp(const char *path, size_t *len, char *err, int errlen) {
  FILE *f = fopen(path, "rb");
  if (!f) {
    fail(err, errlen, "cannot open %s", path);
    return NULL;
  }
  fseek(f, 0, SEEK_END);
  long n = ftell(f);
  fseek(f, 0, SEEK_SET);
  unsigned char *buf = (unsigned char *)malloc(n > 0 ? (size_t)n : 1);
  if (!buf || (n > 0 && fread(buf, 1, (size_t)n, f) != (size_t)n)) {
    fclose(f);
    free(buf);
    fail(err, errlen, "cannot read %s", path);
    return NULL;
  }
  fclose(f);
  *len = (size_t)n;
  return buf;
}

/* Index width (4 or 8) from the class id, or 0. */
static int width(const unsigned char *b, size_t len, uint32_t classid) {
  if (len >= 4 && be32(b) == classid) return 4;
  if (len >= 8 && be64(b) == classid) return 8;
  return 0;
}

static int64_t geti(const unsigned char *p, int w) {
  return w == 4 ? (int64_t)(int32_t)be32(p) : (int64_t)be64(p);
}

int pb_read_mat(const char *path, pb_csr *m, char *err, int errlen) {
  memset(m, 0, sizeof *m);
  size_t len = 0;
  unsigned char *b = slurp(path, &len, err, errlen);
  if (!b) return -1;
  int w = width(b, len, MAT_CLASSID);
  if (!w || len < (size_t)(4 * w)) {
    free(b);
    return fail(err, errlen, "%s is not a PETSc binary matrix", path);
  }
  int64_t M = geti(b + w, w), N = geti(b + 2 * w, w), nz = geti(b + 3 * w, w);
  size_t off = (size_t)4 * w;
  if (M < 0 || N < 0) {
    free(b);
    return fail(err, errlen, "%s: negative matrix size", path);
  }
  int dense = nz == -1;
  if (dense) nz = M * N;
  m->rows = M;
  m->cols = N;
  m->nnz = nz;
  m->rowptr = (int64_t *)calloc((size_t)M + 1, sizeof(int64_t));
  m->col = (int64_t *)malloc(sizeof(int64_t) * (nz > 0 ? (size_t)nz : 1));
  m->val = (double *)malloc(sizeof(double) * 2 * (nz > 0 ? (size_t)nz : 1));
  if (!m->rowptr || !m->col || !m->val) {
    free(b);
    pb_free(m);
    return fail(err, errlen, "out of memory reading %s", path);
  }
  if (dense) {
    for (int64_t i = 0; i <= M; ++i) m->rowptr[i] = i * N;
    for (int64_t j = 0; j < nz; ++j) m->col[j] = j % (N > 0 ? N : 1);
  } else {
    if (off + (size_t)w * (size_t)(M + nz) > len) {
      free(b);
      pb_free(m);
      return fail(err, errlen, "%s: file truncated", path);
    }
    int64_t s = 0;
    for (int64_t i = 0; i < M; ++i) {
      int64_t rl = geti(b + off + (size_t)i * w, w);
      if (rl < 0) {
        free(b);
        pb_free(m);
        return fail(err, errlen, "%s: negative row length", path);
      }
      s += rl;
      m->rowptr[i + 1] = s;
    }
    if (s != nz) {
      free(b);
      pb_free(m);
      return fail(err, errlen, "%s: row lengths sum to %lld, header says %lld", path, (long long)s,
                  (long long)nz);
    }
    off += (size_t)w * M;
    for (int64_t j = 0; j < nz; ++j) {
      m->col[j] = geti(b + off + (size_t)j * w, w);
      if (m->col[j] < 0 || m->col[j] >= N) {
        free(b);
        pb_free(m);
        return fail(err, errlen, "%s: column index out of range", path);
      }
    }
    off += (size_t)w * nz;
  }
  if (off + (size_t)16 * nz > len) {
    free(b);
    pb_free(m);
    return fail(err, errlen, "%s: file truncated", path);
  }
  for (int64_t j = 0; j < 2 * nz; ++j) m->val[j] = bedouble(b + off + (size_t)8 * j);
  free(b);
  return 0;
}

void pb_free(pb_csr *m) {
  free(m->rowptr);
  free(m->col);
  free(m->val);
  memset(m, 0, sizeof *m);
}

int pb_read_vec(const char *path, double **v, int64_t *n, char *err, int errlen) {
  size_t len = 0;
  unsigned char *b = slurp(path, &len, err, errlen);
  if (!b) return -1;
  int w = width(b, len, VEC_CLASSID);
  if (!w) {
    free(b);
    return fail(err, errlen, "%s is not a PETSc binary vector", path);
  }
  int64_t cnt = geti(b + w, w);
  size_t off = (size_t)2 * w;
  if (cnt < 0 || off + (size_t)16 * cnt > len) {
    free(b);
    return fail(err, errlen, "%s: file truncated", path);
  }
  *v = (double *)malloc(sizeof(double) * 2 * (cnt > 0 ? (size_t)cnt : 1));
  for (int64_t j = 0; j < 2 * cnt; ++j) (*v)[j] = bedouble(b + off + (size_t)8 * j);
  *n = cnt;
  free(b);
  return 0;
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
  unsigned char e[16];
  for (int64_t i = 0; i < rows && ok; ++i) {
    put64(e, (uint64_t)cols);
    ok = fwrite(e, 1, 8, f) == 8;
  }
  for (int64_t i = 0; i < rows && ok; ++i)
    for (int64_t j = 0; j < cols && ok; ++j) {
      put64(e, (uint64_t)j);
      ok = fwrite(e, 1, 8, f) == 8;
    }
  for (int64_t i = 0; i < rows && ok; ++i)
    for (int64_t j = 0; j < cols && ok; ++j) {
      double re, im;
      if (is_complex) {
        re = a[2 * (j * ld + i)];
        im = a[2 * (j * ld + i) + 1];
      } else {
        re = a[j * ld + i];
        im = 0.0;
      }
      uint64_t u;
      memcpy(&u, &re, 8);
      put64(e, u);
      memcpy(&u, &im, 8);
      put64(e + 8, u);
      ok = fwrite(e, 1, 16, f) == 16;
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

int pb_write_vec(const char *path, const double *v, int64_t n, int is_complex, char *err, int errlen) {
  FILE *f = fopen(path, "wb");
  if (!f) return fail(err, errlen, "cannot create %s", path);
  unsigned char h[16];
  put64(h, VEC_CLASSID);
  put64(h + 8, (uint64_t)n);
  int ok = fwrite(h, 1, 16, f) == 16;
  unsigned char e[16];
  for (int64_t i = 0; i < n && ok; ++i) {
    double re = is_complex ? v[2 * i] : v[i], im = is_complex ? v[2 * i + 1] : 0.0;
    uint64_t u;
    memcpy(&u, &re, 8);
    put64(e, u);
    memcpy(&u, &im, 8);
    put64(e + 8, u);
    ok = fwrite(e, 1, 16, f) == 16;
  }
  if (fclose(f) != 0) ok = 0;
  return ok ? 0 : fail(err, errlen, "write error on %s", path);
}
