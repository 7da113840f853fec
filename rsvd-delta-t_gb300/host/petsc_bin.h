/* PETSc binary Mat/Vec files in C (the reference's file interface:
 * MatLoad/MatView/VecLoad through PetscViewerBinary, e.g.
 * SourceCode/LNSStructure.c:23-26, SourceCode/SaveResults.c:32-85).
 * Big-endian; PetscInt is int32 or int64 (detected from the class id);
 * scalars are complex128. Only the first object of a file is read. */
#ifndef RSVDT_PETSC_BIN_H
#define RSVDT_PETSC_BIN_H
#include <stdint.h>

typedef struct {
  int64_t rows, cols, nnz;
  int64_t *rowptr; /* rows + 1 */
  int64_t *col;    /* nnz */
  double *val;     /* 2 * nnz, interleaved complex */
} pb_csr;

/* Returns 0 on success; on failure a message is written to err. */
int pb_read_mat(const char *path, pb_csr *m, char *err, int errlen);
void pb_free(pb_csr *m);
/* Reads a Vec (2*n doubles allocated into *v). */
int pb_read_vec(const char *path, double **v, int64_t *n, char *err, int errlen);
/* Writes a dense column-major rows x cols complex matrix (leading dimension
 * ld) in AIJ layout with every entry present, as MatView of a dense matrix
 * does, with 64-bit indices. */
int pb_write_dense(const char *path, const double *a, int64_t rows, int64_t cols, int64_t ld,
                   char *err, int errlen);
/* Same for a real matrix stored as doubles (written as complex with zero
 * imaginary parts, the layout of the reference's complex build). */
int pb_write_dense_real(const char *path, const double *a, int64_t rows, int64_t cols, int64_t ld,
                        char *err, int errlen);
/* Writes a Vec of n complex values (is_complex = 1, 2n doubles) or of n
 * real values stored as complex with zero imaginary parts, with a 64-bit
 * length, as VecView does (SourceCode/TransientRunRK4.c:117-119). */
int pb_write_vec(const char *path, const double *v, int64_t n, int is_complex, char *err, int errlen);

#endif
