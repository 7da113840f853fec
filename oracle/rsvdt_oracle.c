/*
 * CPU oracle for the RSVD-Delta-t time-stepping path (TEST INFRASTRUCTURE).
 *
 * Only the tests, the smoke check and the benchmark's CPU-baseline leg load
 * this library; the product path never does. It restates the reference
 * (AliFarghadan/RSVD-Delta-t, SourceCode/) in C99 complex double, following
 * its operation order so that it agrees with a single-rank PETSc run to
 * rounding:
 *   - MatMultAdd / MatMultHermitianTransposeAdd on a SeqAIJ matrix start
 *     from the added vector and add the products in ascending index order;
 *     the explicit conjugate transpose built here keeps that order.
 *   - Dense MatMult / MatMatMult sum over the inner index in ascending order.
 * QR follows SLEPc's default classical Gram-Schmidt with a second pass
 * (R has a real positive diagonal). SVD is one-sided Jacobi; singular
 * vectors agree with SLEPc's up to a unit-modulus factor per column. The
 * PGMRES solve of the transient-removal step (tolerance 1e-15) is an LU
 * solve with partial pivoting here.
 *
 * Build with -ffp-contract=off so that x86 and Arm hosts round alike.
 */
#include "rsvdt_oracle.h"

#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef double complex zc;

typedef struct {
  int present;
  int64_t rows, cols;
  int64_t *rowptr;
  int64_t *col;
  zc *val;
} csr_t;

typedef struct {
  int64_t N, Nw, Nw_eff, Ns, Nt, R;
  double w, dt;
  int tr, real_op, nthreads;
  int row_threads; /* > 1: the RK4 step's row loops run on that many threads */
  csr_t A, AH;
  zc *idft; /* Nw_eff x 2Ns, row-major */
  zc *dft;  /* Nw x Nw_eff, column-major */
  csr_t W[5], WH[5];
} orc_t;

static const double ORC_PI = 3.14159265358979323846;

/* ------------------------------------------------------------------ CSR -- */

static void csr_free(csr_t *m) {
  free(m->rowptr);
  free(m->col);
  free(m->val);
  memset(m, 0, sizeof(*m));
}

static int csr_copy_in(csr_t *m, int64_t rows, int64_t cols, const int64_t *rowptr,
                       const int64_t *col, const double *val) {
  int64_t nnz = rowptr[rows] - rowptr[0];
  m->rows = rows;
  m->cols = cols;
  m->rowptr = (int64_t *)malloc(sizeof(int64_t) * (rows + 1));
  m->col = (int64_t *)malloc(sizeof(int64_t) * (nnz > 0 ? nnz : 1));
  m->val = (zc *)malloc(sizeof(zc) * (nnz > 0 ? nnz : 1));
  if (!m->rowptr || !m->col || !m->val) return -1;
  for (int64_t i = 0; i <= rows; ++i) m->rowptr[i] = rowptr[i] - rowptr[0];
  for (int64_t j = 0; j < nnz; ++j) {
    m->col[j] = col[rowptr[0] + j];
    if (m->col[j] < 0 || m->col[j] >= cols) return -2;
    m->val[j] = val[2 * (rowptr[0] + j)] + I * val[2 * (rowptr[0] + j) + 1];
  }
  m->present = 1;
  return 0;
}

/* Conjugate transpose with ascending column (original row) order per row,
 * i.e. the summation order of SeqAIJ MatMultHermitianTransposeAdd. */
static int csr_conj_transpose(const csr_t *a, csr_t *t) {
  int64_t nnz = a->rowptr[a->rows];
  t->rows = a->cols;
  t->cols = a->rows;
  t->rowptr = (int64_t *)calloc((size_t)t->rows + 1, sizeof(int64_t));
  t->col = (int64_t *)malloc(sizeof(int64_t) * (nnz > 0 ? nnz : 1));
  t->val = (zc *)malloc(sizeof(zc) * (nnz > 0 ? nnz : 1));
  if (!t->rowptr || !t->col || !t->val) return -1;
  for (int64_t j = 0; j < nnz; ++j) t->rowptr[a->col[j] + 1]++;
  for (int64_t i = 0; i < t->rows; ++i) t->rowptr[i + 1] += t->rowptr[i];
  int64_t *fill = (int64_t *)malloc(sizeof(int64_t) * (t->rows > 0 ? t->rows : 1));
  memcpy(fill, t->rowptr, sizeof(int64_t) * t->rows);
  for (int64_t i = 0; i < a->rows; ++i)
    for (int64_t j = a->rowptr[i]; j < a->rowptr[i + 1]; ++j) {
      int64_t c = a->col[j];
      t->col[fill[c]] = i;
      t->val[fill[c]] = conj(a->val[j]);
      fill[c]++;
    }
  free(fill);
  t->present = 1;
  return 0;
}

/* out = A x + f (MatMultAdd, SourceCode/TSRK4.c:18,31,33,35); f may be NULL. */
static void spmv_add_rows(const csr_t *a, const zc *x, const zc *f, zc *out, int nth) {
  /* Rows are independent: the same sums in the same order on any number of
   * threads. */
#pragma omp parallel for schedule(static) num_threads(nth > 1 ? nth : 1) if (nth > 1)
  for (int64_t i = 0; i < a->rows; ++i) {
    zc s = f ? f[i] : 0.0;
    for (int64_t j = a->rowptr[i]; j < a->rowptr[i + 1]; ++j) s += a->val[j] * x[a->col[j]];
    out[i] = s;
  }
}

static void spmv_add(const csr_t *a, const zc *x, const zc *f, zc *out) {
  for (int64_t i = 0; i < a->rows; ++i) {
    zc s = f ? f[i] : 0.0;
    for (int64_t j = a->rowptr[i]; j < a->rowptr[i + 1]; ++j) s += a->val[j] * x[a->col[j]];
    out[i] = s;
  }
}

/* Y_out (a.rows x ncols) = A * Y_in (a.cols x ncols), column-major
 * (MatMatMult, SourceCode/ApplyWeightMats.c:18-76). */
static void csr_matmat(const csr_t *a, int64_t ncols, const zc *Yin, zc *Yout) {
  for (int64_t c = 0; c < ncols; ++c) spmv_add(a, Yin + c * a->cols, NULL, Yout + c * a->rows);
}

/* ------------------------------------------------------------ grid, DFT -- */

int orc_setup_grid(double w, int64_t Nw, double dt_in, double transient_length, double *out_dt,
                   int64_t *out_ints) {
  /* SourceCode/SetupTimeFreqGrid.c:16-21 */
  double T_ss = 2 * ORC_PI / w;
  double dt_w = T_ss / (double)Nw;
  double dt = dt_w / ceil(dt_w / dt_in);
  int64_t Ns = (int64_t)round(T_ss / dt);
  int64_t Nt = (int64_t)round(transient_length / dt);
  out_dt[0] = dt;
  out_ints[0] = Ns;
  out_ints[1] = Nt;
  out_ints[2] = Ns / Nw;
  return 0;
}

static void build_idft(int64_t Nw_eff, int64_t Ns, int real_op, zc *idft) {
  /* SourceCode/CreateDFTiDFTMats.c:23-59 and :93 (transpose). The column of
   * frequency iw holds conj(exp(alpha*f*it)) * 2/Nt with alpha = -2*pi*i/Nt,
   * Nt = 2*Ns half-step samples; f = iw for the first half of the
   * frequencies and (iw - Nw) + Nt for the negative ones. */
  int64_t Nt = 2 * Ns;
  double alpha_im = -2 * ORC_PI / (double)Nt;
  for (int64_t iw = 0; iw < Nw_eff; ++iw) {
    int64_t f;
    if (real_op)
      f = iw;
    else if (Nw_eff % 2 == 0)
      f = (iw <= Nw_eff / 2 - 1) ? iw : (iw - Nw_eff) + Nt;
    else
      f = (iw <= (Nw_eff - 1) / 2) ? iw : (iw - Nw_eff) + Nt;
    double v_im = alpha_im * (double)f;
    for (int64_t it = 0; it < Nt; ++it) {
      double y = v_im * (double)it;
      zc e = cos(y) + I * sin(y);
      idft[iw * Nt + it] = conj(e) * (2. / (double)Nt);
    }
  }
}

static void build_dft(int64_t Nw, int64_t Nw_eff, int real_op, zc *dft) {
  /* SourceCode/CreateDFTiDFTMats.c:61-85: dft[j, iw] = exp(alpha*iw*j),
   * alpha = -2*pi*i/Nw_eff (-2*pi*i/(2 Nw_eff) for a real operator): the
   * `Nw` of that formula is the column count of idft (line 26). */
  double alpha_im = real_op ? -2 * ORC_PI / (double)(2 * Nw_eff) : -2 * ORC_PI / (double)Nw_eff;
  for (int64_t iw = 0; iw < Nw_eff; ++iw) {
    double v_im = alpha_im * (double)iw;
    for (int64_t j = 0; j < Nw; ++j) {
      double y = v_im * (double)j;
      dft[iw * Nw + j] = cos(y) + I * sin(y);
    }
  }
}

int orc_build_idft(int64_t Nw_eff, int64_t Ns, int real_op, double *idft) {
  build_idft(Nw_eff, Ns, real_op, (zc *)idft);
  return 0;
}

int orc_build_dft(int64_t Nw, int64_t Nw_eff, int real_op, double *dft) {
  build_dft(Nw, Nw_eff, real_op, (zc *)dft);
  return 0;
}

/* --------------------------------------------------------------- handle -- */

void *orc_create(int64_t N, const int64_t *rowptr, const int64_t *col, const double *val,
                 int64_t Nw, double w, double dt, int64_t Ns, int64_t Nt, int64_t R,
                 int transient_removal, int real_op) {
  orc_t *h = (orc_t *)calloc(1, sizeof(orc_t));
  if (!h) return NULL;
  h->N = N;
  h->Nw = Nw;
  h->Nw_eff = real_op ? Nw / 2 : Nw; /* SourceCode/LNSStructure.c:44 */
  h->Ns = Ns;
  h->Nt = Nt;
  h->R = R;
  h->w = w;
  h->dt = dt;
  h->tr = transient_removal;
  h->real_op = real_op;
  h->nthreads = 0;
  if (csr_copy_in(&h->A, N, N, rowptr, col, val) || csr_conj_transpose(&h->A, &h->AH)) {
    orc_destroy(h);
    return NULL;
  }
  h->idft = (zc *)malloc(sizeof(zc) * h->Nw_eff * 2 * Ns);
  h->dft = (zc *)malloc(sizeof(zc) * Nw * h->Nw_eff);
  build_idft(h->Nw_eff, Ns, real_op, h->idft);
  build_dft(Nw, h->Nw_eff, real_op, h->dft);
  return h;
}

void orc_destroy(void *vh) {
  orc_t *h = (orc_t *)vh;
  if (!h) return;
  csr_free(&h->A);
  csr_free(&h->AH);
  for (int i = 0; i < 5; ++i) {
    csr_free(&h->W[i]);
    csr_free(&h->WH[i]);
  }
  free(h->idft);
  free(h->dft);
  free(h);
}

void orc_set_threads(void *vh, int nthreads) { ((orc_t *)vh)->nthreads = nthreads; }

void orc_set_row_threads(void *vh, int nthreads) { ((orc_t *)vh)->row_threads = nthreads; }

int orc_set_weight(void *vh, int which, int64_t rows, int64_t cols, const int64_t *rowptr,
                   const int64_t *col, const double *val) {
  orc_t *h = (orc_t *)vh;
  if (which < 0 || which > 4) return -1;
  csr_free(&h->W[which]);
  csr_free(&h->WH[which]);
  if (csr_copy_in(&h->W[which], rows, cols, rowptr, col, val)) return -2;
  if (csr_conj_transpose(&h->W[which], &h->WH[which])) return -3;
  return 0;
}

/* ------------------------------------------------------------ RK4 step -- */

typedef struct {
  zc *F2, *k1, *k2, *k3, *k4, *yt;
} work_t;

static int work_alloc(work_t *w, int64_t N) {
  zc *p = (zc *)malloc(sizeof(zc) * 6 * (N > 0 ? N : 1));
  if (!p) return -1;
  w->F2 = p;
  w->k1 = p + N;
  w->k2 = p + 2 * N;
  w->k3 = p + 3 * N;
  w->k4 = p + 4 * N;
  w->yt = p + 5 * N;
  return 0;
}

/* F = Fk * idft[:, jt] (SourceCode/CreateForcingOnFly.c:17-19). Fk is
 * N x Nw_eff column-major. Each F[n] sums over the frequencies in order. */
static void forcing(const orc_t *h, const zc *Fk, int64_t jt, zc *F) {
  int64_t N = h->N, Nt2 = 2 * h->Ns;
  const int nth = h->row_threads;
#pragma omp parallel for schedule(static) num_threads(nth > 1 ? nth : 1) if (nth > 1)
  for (int64_t n = 0; n < N; ++n) {
    zc s = 0;
    for (int64_t iw = 0; iw < h->Nw_eff; ++iw) s += Fk[iw * N + n] * h->idft[iw * Nt2 + jt];
    F[n] = s;
  }
}

/* y_out[n] = a * x[n] + y[n] over all rows (VecWAXPY / VecAXPY). */
static void waxpy_rows(int64_t N, double a, const zc *x, const zc *y, zc *out, int nth) {
#pragma omp parallel for schedule(static) num_threads(nth > 1 ? nth : 1) if (nth > 1)
  for (int64_t n = 0; n < N; ++n) out[n] = a * x[n] + y[n];
}

/* Half-step forcing indices of step i (SourceCode/TSRK4.c:21-26). */
static void step_indices(const orc_t *h, int dir, int64_t i, int64_t *j2, int64_t *j3) {
  double two_ns = 2.0 * (double)h->Ns;
  if (dir) {
    *j2 = (int64_t)fmod((double)(2 * (i - 1) + 1), two_ns);
    *j3 = (int64_t)fmod((double)(2 * (i - 1) + 2), two_ns);
  } else {
    *j2 = (int64_t)fmod(1e6 * (double)h->Ns - 1 - (double)(2 * (i - 1)), two_ns);
    *j3 = (int64_t)fmod(1e6 * (double)h->Ns - 1 - (double)(2 * (i - 1) + 1), two_ns);
  }
}

/* One forced RK4 step (SourceCode/TSRK4.c:18-47). F3 holds the forcing of
 * the step's start on entry and of its end on exit. */
static void rk4_step(const orc_t *h, int dir, const zc *Fk, int64_t i, zc *y, zc *F3,
                     work_t *w) {
  const csr_t *A = dir ? &h->A : &h->AH;
  int64_t N = h->N;
  double dt = h->dt;
  const int nth = h->row_threads;
  int64_t j2, j3;
  spmv_add_rows(A, y, F3, w->k1, nth);
  step_indices(h, dir, i, &j2, &j3);
  forcing(h, Fk, j2, w->F2);
  forcing(h, Fk, j3, F3);
  waxpy_rows(N, dt / 2, w->k1, y, w->yt, nth);
  spmv_add_rows(A, w->yt, w->F2, w->k2, nth);
  waxpy_rows(N, dt / 2, w->k2, y, w->yt, nth);
  spmv_add_rows(A, w->yt, w->F2, w->k3, nth);
  waxpy_rows(N, dt, w->k3, y, w->yt, nth);
  spmv_add_rows(A, w->yt, F3, w->k4, nth);
  waxpy_rows(N, dt / 6, w->k1, y, y, nth);
  waxpy_rows(N, dt / 6 * 2, w->k2, y, y, nth);
  waxpy_rows(N, dt / 6 * 2, w->k3, y, y, nth);
  waxpy_rows(N, dt / 6, w->k4, y, y, nth);
}

/* Unforced RK4 step (SourceCode/TSTransRK4.c:15-36). */
static void rk4_step_unforced(const orc_t *h, int dir, zc *y, work_t *w) {
  const csr_t *A = dir ? &h->A : &h->AH;
  int64_t N = h->N;
  double dt = h->dt;
  spmv_add(A, y, NULL, w->k1);
  for (int64_t n = 0; n < N; ++n) w->yt[n] = dt / 2 * w->k1[n] + y[n];
  spmv_add(A, w->yt, NULL, w->k2);
  for (int64_t n = 0; n < N; ++n) w->yt[n] = dt / 2 * w->k2[n] + y[n];
  spmv_add(A, w->yt, NULL, w->k3);
  for (int64_t n = 0; n < N; ++n) w->yt[n] = dt * w->k3[n] + y[n];
  spmv_add(A, w->yt, NULL, w->k4);
  for (int64_t n = 0; n < N; ++n) y[n] += dt / 6 * w->k1[n];
  for (int64_t n = 0; n < N; ++n) y[n] += dt / 6 * 2 * w->k2[n];
  for (int64_t n = 0; n < N; ++n) y[n] += dt / 6 * 2 * w->k3[n];
  for (int64_t n = 0; n < N; ++n) y[n] += dt / 6 * w->k4[n];
}

int orc_rk4_steps(void *vh, int dir, const double *Fk, int64_t i0, int64_t nsteps, double *y,
                  double *F3) {
  orc_t *h = (orc_t *)vh;
  work_t w;
  if (work_alloc(&w, h->N)) return -1;
  for (int64_t i = i0; i < i0 + nsteps; ++i)
    rk4_step(h, dir, (const zc *)Fk, i, (zc *)y, (zc *)F3, &w);
  free(w.F2);
  return 0;
}

/* ------------------------------------------------------- dense helpers -- */

/* In-place thin QR of a rows x cols column-major block: classical
 * Gram-Schmidt with a second pass, R with a real positive diagonal
 * (SLEPc BVOrthogonalize defaults, SourceCode/QRAllFreqs.c:26,
 * SourceCode/QRDecomposition.c:18). */
static void qr_cgs2(int64_t rows, int64_t cols, zc *Q) {
  zc *h = (zc *)malloc(sizeof(zc) * (cols > 0 ? cols : 1));
  for (int64_t j = 0; j < cols; ++j) {
    zc *v = Q + j * rows;
    for (int pass = 0; pass < 2; ++pass) {
      for (int64_t i = 0; i < j; ++i) {
        const zc *q = Q + i * rows;
        zc s = 0;
        for (int64_t n = 0; n < rows; ++n) s += conj(q[n]) * v[n];
        h[i] = s;
      }
      for (int64_t i = 0; i < j; ++i) {
        const zc *q = Q + i * rows;
        for (int64_t n = 0; n < rows; ++n) v[n] -= h[i] * q[n];
      }
    }
    double nrm = 0;
    for (int64_t n = 0; n < rows; ++n) nrm += creal(v[n]) * creal(v[n]) + cimag(v[n]) * cimag(v[n]);
    nrm = sqrt(nrm);
    for (int64_t n = 0; n < rows; ++n) v[n] = nrm > 0 ? v[n] / nrm : 0;
  }
  free(h);
}

/* One-sided Jacobi SVD of a rows x cols column-major block A (overwritten
 * with U * diag(s)). Outputs U (rows x cols) and s (cols), descending. */
static void svd_jacobi(int64_t rows, int64_t cols, zc *A, zc *U, double *s) {
  for (int sweep = 0; sweep < 80; ++sweep) {
    double off = 0;
    for (int64_t p = 0; p < cols - 1; ++p)
      for (int64_t q = p + 1; q < cols; ++q) {
        zc *ap = A + p * rows, *aq = A + q * rows;
        double app = 0, aqq = 0;
        zc apq = 0;
        for (int64_t n = 0; n < rows; ++n) {
          app += creal(ap[n]) * creal(ap[n]) + cimag(ap[n]) * cimag(ap[n]);
          aqq += creal(aq[n]) * creal(aq[n]) + cimag(aq[n]) * cimag(aq[n]);
          apq += conj(ap[n]) * aq[n];
        }
        double mag = cabs(apq);
        if (mag == 0 || mag <= 1e-15 * sqrt(app * aqq)) continue;
        double rel = mag / sqrt(app * aqq);
        if (rel > off) off = rel;
        /* Rotation that diagonalises the 2x2 Gram [[app, apq],[conj(apq), aqq]]. */
        zc ph = apq / mag;
        double tau = (aqq - app) / (2 * mag);
        double t = (tau >= 0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1 + tau * tau));
        double c = 1 / sqrt(1 + t * t), sn = c * t;
        for (int64_t n = 0; n < rows; ++n) {
          zc x = ap[n], y = aq[n];
          ap[n] = c * x - sn * conj(ph) * y;
          aq[n] = sn * ph * x + c * y;
        }
      }
    if (off <= 1e-15) break;
  }
  /* Norms, order, normalise. */
  int64_t *idx = (int64_t *)malloc(sizeof(int64_t) * cols);
  double *nr = (double *)malloc(sizeof(double) * cols);
  for (int64_t j = 0; j < cols; ++j) {
    double acc = 0;
    const zc *a = A + j * rows;
    for (int64_t n = 0; n < rows; ++n) acc += creal(a[n]) * creal(a[n]) + cimag(a[n]) * cimag(a[n]);
    nr[j] = sqrt(acc);
    idx[j] = j;
  }
  for (int64_t i = 1; i < cols; ++i) {
    int64_t t = idx[i], j = i;
    while (j > 0 && nr[idx[j - 1]] < nr[t]) {
      idx[j] = idx[j - 1];
      --j;
    }
    idx[j] = t;
  }
  for (int64_t j = 0; j < cols; ++j) {
    int64_t src = idx[j];
    s[j] = nr[src];
    for (int64_t n = 0; n < rows; ++n) U[j * rows + n] = nr[src] > 0 ? A[src * rows + n] / nr[src] : 0;
  }
  free(idx);
  free(nr);
}

/* Dense LU solve with partial pivoting of an m x m column-major system. */
static int lu_solve(int64_t m, zc *M, zc *b) {
  for (int64_t c = 0; c < m; ++c) {
    int64_t piv = c;
    double best = cabs(M[c * m + c]);
    for (int64_t r = c + 1; r < m; ++r)
      if (cabs(M[c * m + r]) > best) {
        best = cabs(M[c * m + r]);
        piv = r;
      }
    if (best == 0) return -1;
    if (piv != c) {
      for (int64_t cc = 0; cc < m; ++cc) {
        zc t = M[cc * m + c];
        M[cc * m + c] = M[cc * m + piv];
        M[cc * m + piv] = t;
      }
      zc t = b[c];
      b[c] = b[piv];
      b[piv] = t;
    }
    for (int64_t r = c + 1; r < m; ++r) {
      zc l = M[c * m + r] / M[c * m + c];
      M[c * m + r] = l;
      for (int64_t cc = c + 1; cc < m; ++cc) M[cc * m + r] -= l * M[cc * m + c];
      b[r] -= l * b[c];
    }
  }
  for (int64_t r = m - 1; r >= 0; --r) {
    zc s = b[r];
    for (int64_t cc = r + 1; cc < m; ++cc) s -= M[cc * m + r] * b[cc];
    b[r] = s / M[r * m + r];
  }
  return 0;
}

/* --------------------------------------------------------- TS action -- */

/* Transient removal for one test vector (SourceCode/CreateMtilde.c:41-54,
 * SourceCode/TSExpADeltaT.c:25-34, SourceCode/GalerkinProj.c:26-74).
 * Yk: N x (Nw+1) snapshots; Yhat_k: N x Nw_eff output. */
static int transient_removal_one(const orc_t *h, int dir, const zc *Yk, zc *Yhat_k, work_t *w) {
  int64_t N = h->N, Nw = h->Nw, Ns1 = Nw + 1, R = h->R;
  double deltaT = h->dt * (double)R;
  zc *V = (zc *)malloc(sizeof(zc) * N * Ns1);
  zc *MV = (zc *)malloc(sizeof(zc) * N * Ns1);
  zc *Mt = (zc *)malloc(sizeof(zc) * Ns1 * Ns1);
  zc *Mtmp = (zc *)malloc(sizeof(zc) * Ns1 * Ns1);
  zc *y1 = (zc *)malloc(sizeof(zc) * N);
  zc *y2 = (zc *)malloc(sizeof(zc) * N);
  zc *b = (zc *)malloc(sizeof(zc) * Ns1);
  if (!V || !MV || !Mt || !Mtmp || !y1 || !y2 || !b) return -1;
  memcpy(V, Yk, sizeof(zc) * N * Ns1);
  qr_cgs2(N, Ns1, V);
  memcpy(MV, V, sizeof(zc) * N * Ns1);
  for (int64_t s = 0; s < Ns1; ++s)
    for (int64_t it = 0; it < R; ++it) rk4_step_unforced(h, dir, MV + s * N, w);
  /* M_tilde = V^H MV (SourceCode/CreateMtilde.c:49-51). */
  for (int64_t c = 0; c < Ns1; ++c)
    for (int64_t r = 0; r < Ns1; ++r) {
      zc s = 0;
      for (int64_t n = 0; n < N; ++n) s += conj(V[r * N + n]) * MV[c * N + n];
      Mt[c * Ns1 + r] = s;
    }
  int rc = 0;
  for (int64_t iw = 0; iw < h->Nw_eff; ++iw) {
    const zc *d = h->dft + iw * Nw;
    const zc *Ya = dir ? Yk : Yk + N;      /* y1 columns */
    const zc *Yb = dir ? Yk + N : Yk;      /* y2 columns */
    for (int64_t n = 0; n < N; ++n) {
      zc s1 = 0, s2 = 0;
      for (int64_t j = 0; j < Nw; ++j) {
        s1 += Ya[j * N + n] * d[j];
        s2 += Yb[j * N + n] * d[j];
      }
      y1[n] = s1 * (double)R;
      y2[n] = s2 * (double)R;
    }
    zc e = dir ? cexp(I * h->w * (double)iw * deltaT) : cexp(-I * h->w * (double)iw * deltaT);
    for (int64_t i = 0; i < Ns1 * Ns1; ++i) Mtmp[i] = -Mt[i];
    for (int64_t i = 0; i < Ns1; ++i) Mtmp[i * Ns1 + i] += e;
    /* yt = e*y1 - y2; b = V^H yt (SourceCode/GalerkinProj.c:51-55). */
    for (int64_t r = 0; r < Ns1; ++r) {
      zc s = 0;
      for (int64_t n = 0; n < N; ++n) s += conj(V[r * N + n]) * (e * y1[n] - y2[n]);
      b[r] = s;
    }
    if (lu_solve(Ns1, Mtmp, b)) rc = -2;
    /* y1 -= V b (SourceCode/GalerkinProj.c:65-66). */
    for (int64_t n = 0; n < N; ++n) {
      zc s = 0;
      for (int64_t r = 0; r < Ns1; ++r) s += V[r * N + n] * b[r];
      Yhat_k[iw * N + n] = y1[n] - s;
    }
  }
  free(V);
  free(MV);
  free(Mt);
  free(Mtmp);
  free(y1);
  free(y2);
  free(b);
  return rc;
}

int orc_ts_action(void *vh, int dir, int64_t k, const double *Fd, double *Yd) {
  orc_t *h = (orc_t *)vh;
  const zc *F = (const zc *)Fd;
  zc *Y = (zc *)Yd;
  int64_t N = h->N, Nw = h->Nw, Nwe = h->Nw_eff, R = h->R;
  int64_t rend = h->Nt + h->Ns + (h->tr ? R : 0); /* SourceCode/TSActionRK4.c:41-42 */
  int64_t Nstore = h->tr ? Nw + 1 : Nw;           /* SourceCode/TSActionRK4.c:43 */
  int err = 0;
  int nth = h->nthreads;
#ifdef _OPENMP
  if (nth <= 0) nth = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nth) reduction(| : err)
#endif
  for (int64_t ik = 0; ik < k; ++ik) {
    work_t w;
    zc *Fk = (zc *)malloc(sizeof(zc) * N * Nwe);
    zc *Yk = (zc *)calloc((size_t)(N * Nstore), sizeof(zc));
    zc *Yh = (zc *)malloc(sizeof(zc) * N * Nwe);
    zc *y = (zc *)calloc((size_t)N, sizeof(zc));
    zc *F3 = (zc *)malloc(sizeof(zc) * N);
    if (!Fk || !Yk || !Yh || !y || !F3 || work_alloc(&w, N)) {
      err |= 1;
      continue;
    }
    /* PermuteMat + submatrix (SourceCode/TSActionRK4.c:76,93-97). */
    for (int64_t iw = 0; iw < Nwe; ++iw) memcpy(Fk + iw * N, F + (iw * k + ik) * N, sizeof(zc) * N);
    forcing(h, Fk, 0, F3); /* SourceCode/TSActionRK4.c:103 */
    for (int64_t i = 1; i <= rend; ++i) {
      rk4_step(h, dir, Fk, i, y, F3, &w);
      /* SaveSnapshots (SourceCode/SaveSnapshots.c:19-29). */
      if (i > h->Nt) {
        int64_t pos = i - h->Nt;
        if (pos % R == 0) {
          pos = pos / R - 1;
          pos = pos % Nstore;
          pos = dir ? pos : Nstore - 1 - pos;
          pos = pos % Nstore;
          memcpy(Yk + pos * N, y, sizeof(zc) * N);
        }
      }
    }
    if (h->tr) {
      if (transient_removal_one(h, dir, Yk, Yh, &w)) err |= 2;
    } else {
      /* DFT (SourceCode/DFT.c:26-38): Y_hat_k = Y_all_k * dft * ResRatio. */
      for (int64_t iw = 0; iw < Nwe; ++iw) {
        const zc *d = h->dft + iw * Nw;
        for (int64_t n = 0; n < N; ++n) {
          zc s = 0;
          for (int64_t j = 0; j < Nw; ++j) s += Yk[j * N + n] * d[j];
          Yh[iw * N + n] = s * (double)R;
        }
      }
    }
    /* ReversePermuteMat (SourceCode/ReversePermuteMat.c:24-34). */
    for (int64_t iw = 0; iw < Nwe; ++iw) memcpy(Y + (iw * k + ik) * N, Yh + iw * N, sizeof(zc) * N);
    free(Fk);
    free(Yk);
    free(Yh);
    free(y);
    free(F3);
    free(w.F2);
  }
  return err ? -1 : 0;
}

/* -------------------------------------------------------------- weights -- */

/* Y <- M * Y with M = W[which] (herm = 0) or W[which]^H (herm = 1). *rows is
 * updated to the product's row count. Returns a freshly allocated matrix. */
static zc *apply_w(const orc_t *h, int which, int herm, int64_t ncols, zc *Y, int64_t *rows) {
  const csr_t *m = herm ? &h->WH[which] : &h->W[which];
  zc *out = (zc *)malloc(sizeof(zc) * m->rows * ncols);
  csr_matmat(m, ncols, Y, out);
  free(Y);
  *rows = m->rows;
  return out;
}

enum { W_FINV = 0, W_B = 1, W_C = 2, W_Q = 3, W_QINV = 4 };

static int64_t rows_nb(const orc_t *h) { return h->W[W_B].present ? h->W[W_B].cols : h->N; }
static int64_t rows_nc(const orc_t *h) { return h->W[W_C].present ? h->W[W_C].rows : h->N; }

int orc_action(void *vh, int dir, int64_t k, const double *Yin, double *Yout) {
  orc_t *h = (orc_t *)vh;
  int64_t ncols = k * h->Nw_eff;
  int64_t rows = dir ? rows_nb(h) : rows_nc(h);
  zc *Y = (zc *)malloc(sizeof(zc) * rows * ncols);
  memcpy(Y, Yin, sizeof(zc) * rows * ncols);
  /* SourceCode/ApplyWeightMats.c:16-80 */
  if (dir) {
    if (h->W[W_FINV].present) Y = apply_w(h, W_FINV, 0, ncols, Y, &rows);
    if (h->W[W_B].present) Y = apply_w(h, W_B, 0, ncols, Y, &rows);
  } else {
    if (h->W[W_Q].present) Y = apply_w(h, W_Q, 1, ncols, Y, &rows);
    if (h->W[W_C].present) Y = apply_w(h, W_C, 1, ncols, Y, &rows);
  }
  zc *Z = (zc *)malloc(sizeof(zc) * h->N * ncols);
  int rc = orc_ts_action(h, dir, k, (const double *)Y, (double *)Z);
  free(Y);
  rows = h->N;
  if (dir) {
    if (h->W[W_C].present) Z = apply_w(h, W_C, 0, ncols, Z, &rows);
    if (h->W[W_Q].present) Z = apply_w(h, W_Q, 0, ncols, Z, &rows);
  } else {
    if (h->W[W_B].present) Z = apply_w(h, W_B, 1, ncols, Z, &rows);
    if (h->W[W_FINV].present) Z = apply_w(h, W_FINV, 1, ncols, Z, &rows);
  }
  memcpy(Yout, Z, sizeof(zc) * rows * ncols);
  free(Z);
  return rc;
}

/* ---------------------------------------------------------- QR and SVD -- */

int orc_qr_all_freqs(int64_t rows, int64_t k, int64_t nw, double *Yd) {
  zc *Y = (zc *)Yd;
  for (int64_t iw = 0; iw < nw; ++iw) qr_cgs2(rows, k, Y + iw * k * rows);
  return 0;
}

int orc_svd_all_freqs(int64_t rows, int64_t k, int64_t nw, const double *Yd, double *Ud,
                      double *S) {
  const zc *Y = (const zc *)Yd;
  zc *U = (zc *)Ud;
  zc *A = (zc *)malloc(sizeof(zc) * rows * k);
  if (!A) return -1;
  for (int64_t iw = 0; iw < nw; ++iw) {
    memcpy(A, Y + iw * k * rows, sizeof(zc) * rows * k);
    svd_jacobi(rows, k, A, U + iw * k * rows, S + iw * k);
  }
  free(A);
  return 0;
}

int orc_run(void *vh, int64_t k, int64_t q, const double *F, double *Ud, double *Vd, double *S) {
  orc_t *h = (orc_t *)vh;
  int64_t nwe = h->Nw_eff, ncols = k * nwe;
  int64_t nb = rows_nb(h), nc = rows_nc(h);
  zc *Yb = (zc *)malloc(sizeof(zc) * nb * ncols); /* Nb-row block */
  zc *Yc = (zc *)malloc(sizeof(zc) * nc * ncols); /* Nc-row block */
  zc *U = (zc *)Ud, *V = (zc *)Vd;
  int rc = 0;
  memcpy(Yb, F, sizeof(zc) * nb * ncols);
  rc |= orc_action(h, 1, k, (double *)Yb, (double *)Yc); /* SourceCode/main.c:134 */
  for (int64_t iq = 0; iq < q; ++iq) {                    /* SourceCode/PowerIterationRK4.c:20-29 */
    orc_qr_all_freqs(nc, k, nwe, (double *)Yc);
    rc |= orc_action(h, 0, k, (double *)Yc, (double *)Yb);
    orc_qr_all_freqs(nb, k, nwe, (double *)Yb);
    rc |= orc_action(h, 1, k, (double *)Yb, (double *)Yc);
  }
  /* SVDAllFreqsBeforeAdjoint + StoreU (SourceCode/main.c:138-140). */
  double *stmp = (double *)malloc(sizeof(double) * k * nwe);
  orc_svd_all_freqs(nc, k, nwe, (double *)Yc, (double *)U, stmp);
  free(stmp);
  rc |= orc_action(h, 0, k, (double *)U, (double *)Yb); /* SourceCode/main.c:142 */
  orc_svd_all_freqs(nb, k, nwe, (double *)Yb, (double *)V, S); /* SourceCode/SVDAllFreqs.c:34-56 */
  /* Inverse weights (SourceCode/SVDAllFreqs.c:63-64). */
  if (h->W[W_QINV].present) {
    zc *T = (zc *)malloc(sizeof(zc) * nc * ncols);
    csr_matmat(&h->W[W_QINV], ncols, U, T);
    memcpy(U, T, sizeof(zc) * nc * ncols);
    free(T);
  }
  if (h->W[W_FINV].present) {
    zc *T = (zc *)malloc(sizeof(zc) * nb * ncols);
    csr_matmat(&h->W[W_FINV], ncols, V, T);
    memcpy(V, T, sizeof(zc) * nb * ncols);
    free(T);
  }
  free(Yb);
  free(Yc);
  return rc ? -1 : 0;
}
