/* Test helper (built by tests/test_host_io.py): reads a PETSc-binary
 * matrix with host/petsc_bin.c and writes it back as a dense matrix (or a
 * vector), so that the test can compare both directions with the Python
 * reader/writer, and prints the read and write times.
 *   petsc_bin_check mat <in> <out-dense>
 *   petsc_bin_check vec <in> <out-vec> */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "petsc_bin.h"

static double now(void) {
  struct timespec t;
  clock_gettime(CLOCK_MONOTONIC, &t);
  return t.tv_sec + 1e-9 * t.tv_nsec;
}

int main(int argc, char **argv) {
  if (argc != 4) return 2;
  char err[512];
  if (!strcmp(argv[1], "mat")) {
    pb_csr m;
    double t0 = now();
    if (pb_read_mat(argv[2], &m, err, sizeof err)) {
      fprintf(stderr, "%s\n", err);
      return 1;
    }
    double t1 = now();
    /* CSR -> dense column-major (the test matrices are small). */
    double *d = (double *)calloc((size_t)(2 * m.rows * m.cols), sizeof(double));
    for (int64_t r = 0; r < m.rows; ++r)
      for (int64_t j = m.rowptr[r]; j < m.rowptr[r + 1]; ++j) {
        d[2 * (m.col[j] * m.rows + r)] = m.val[2 * j];
        d[2 * (m.col[j] * m.rows + r) + 1] = m.val[2 * j + 1];
      }
    double t2 = now();
    if (pb_write_dense(argv[3], d, m.rows, m.cols, m.rows, err, sizeof err)) {
      fprintf(stderr, "%s\n", err);
      return 1;
    }
    double t3 = now();
    printf("%lld %lld %lld %.6f %.6f\n", (long long)m.rows, (long long)m.cols, (long long)m.nnz, t1 - t0, t3 - t2);
    free(d);
    pb_free(&m);
    return 0;
  }
  if (!strcmp(argv[1], "vec")) {
    double *v = NULL;
    int64_t n = 0;
    if (pb_read_vec(argv[2], &v, &n, err, sizeof err)) {
      fprintf(stderr, "%s\n", err);
      return 1;
    }
    if (pb_write_vec(argv[3], v, n, 1, err, sizeof err)) {
      fprintf(stderr, "%s\n", err);
      return 1;
    }
    printf("%lld\n", (long long)n);
    free(v);
    return 0;
  }
  return 2;
}
