/*
 * CPU oracle for the RSVD-Delta-t time-stepping path.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the checker that the CUDA path is
 * compared against (tests, the smoke check and the CPU baseline of the
 * benchmark). The product library never links, loads or calls it.
 *
 * It restates, operation for operation, the reference's algorithm
 * (AliFarghadan/RSVD-Delta-t, SourceCode/*.c) in plain C99 complex double,
 * without PETSc/SLEPc. Each function names the reference lines it follows.
 * Matrices that the reference keeps as PETSc dense matrices are stored
 * column-major here, with the reference's column ordering: the spectral
 * block Y_hat is rows x (k*Nw_eff) with column iw*k+ik ("frequency-major",
 * SourceCode/CreateRandomMat.c:34, SourceCode/PermuteMat.c:24-34).
 *
 * Complex arrays cross the interface as interleaved (re, im) doubles.
 */
#ifndef RSVDT_ORACLE_H
#define RSVDT_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* SourceCode/SetupTimeFreqGrid.c:16-21. out_dt[0] = dt;
 * out_ints = {Ns, Nt, ResRatio}. Returns 0. */
int orc_setup_grid(double w, int64_t Nw, double dt_in, double transient_length,
                   double *out_dt, int64_t *out_ints);

/* SourceCode/CreateDFTiDFTMats.c:42-59,93: idft is Nw_eff x 2Ns, stored
 * row-major idft[iw*2Ns + jt]. */
int orc_build_idft(int64_t Nw_eff, int64_t Ns, int real_op, double *idft);
/* SourceCode/CreateDFTiDFTMats.c:61-85: dft is Nw x Nw_eff, stored
 * column-major dft[iw*Nw + j]. */
int orc_build_dft(int64_t Nw, int64_t Nw_eff, int real_op, double *dft);

/* Problem handle: operator A (square CSR, int64 indices, complex values) and
 * the time grid. The CSR arrays are copied. */
void *orc_create(int64_t N, const int64_t *rowptr, const int64_t *col, const double *val,
                 int64_t Nw, double w, double dt, int64_t Ns, int64_t Nt, int64_t R,
                 int transient_removal, int real_op);
void orc_destroy(void *h);
/* Number of OpenMP threads used by the time-stepping loops (<=0: all). */
void orc_set_threads(void *h, int nthreads);
/* Threads for the row loops of one RK4 step (1: serial). */
void orc_set_row_threads(void *h, int nthreads);

/* Weight / input / output matrices (SourceCode/ReadWeightMats.c:26-99):
 * which = 0 W_f^{-1/2} (Nb x Nb), 1 B (N x Nb), 2 C (Nc x N),
 *         3 W_q^{1/2} (Nc x Nc), 4 W_q^{-1/2} (Nc x Nc). */
int orc_set_weight(void *h, int which, int64_t rows, int64_t cols, const int64_t *rowptr,
                   const int64_t *col, const double *val);

/* TSActionRK4 (SourceCode/TSActionRK4.c:15-164) without the weights: F is
 * N x (k*Nw_eff) frequency-major, Y receives N x (k*Nw_eff) frequency-major.
 * dir = 1 direct, 0 adjoint. */
int orc_ts_action(void *h, int dir, int64_t k, const double *F, double *Y);

/* DirectActionRK4 / AdjointActionRK4 with ApplyWeightMats
 * (SourceCode/DirectActionRK4.c:24-28, SourceCode/AdjointActionRK4.c:24-28,
 * SourceCode/ApplyWeightMats.c:16-80). Yin has rows_in rows, Yout rows_out
 * rows; both k*Nw_eff columns. */
int orc_action(void *h, int dir, int64_t k, const double *Yin, double *Yout);

/* rk4 steps i0..i0+nsteps-1 of SourceCode/TSRK4.c:6-51 for ONE test vector,
 * starting from state y (N) and previous full-step forcing F3 (N); Fk is the
 * N x Nw_eff coefficient block of that test vector (column-major). y and F3
 * are updated in place. */
int orc_rk4_steps(void *h, int dir, const double *Fk, int64_t i0, int64_t nsteps, double *y,
                  double *F3);

/* QRAllFreqs (SourceCode/QRAllFreqs.c:22-32), in place on rows x (k*nw). */
int orc_qr_all_freqs(int64_t rows, int64_t k, int64_t nw, double *Y);
/* Per-frequency thin SVD of the rows x k blocks (SourceCode/SVDAllFreqs.c:34-56,
 * SourceCode/SVDAllFreqsBeforeAdjoint.c:31-49): U (rows x k*nw) left vectors,
 * S (k x nw, column-major) singular values in descending order. */
int orc_svd_all_freqs(int64_t rows, int64_t k, int64_t nw, const double *Y, double *U,
                      double *S);

/* The main.c sequence (SourceCode/main.c:134-144): direct action, q power
 * iterations, SVD, store U, adjoint action, SVD, inverse weights.
 * F is Nb x (k*Nw_eff); U is Nc x (k*Nw_eff); V is Nb x (k*Nw_eff); S k x Nw_eff. */
int orc_run(void *h, int64_t k, int64_t q, const double *F, double *U, double *V, double *S);

#ifdef __cplusplus
}
#endif
#endif
