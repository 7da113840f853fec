// C ABI of the GB300 RSVD-Delta-t library (include/rsvdt.h): context,
// operator/weight upload, the resolvent actions and the main sequence.
#include <chrono>
#include <cmath>
#include <complex>
#include <cstdarg>
#include <cstring>
#include <vector>

#include <unistd.h>

#include "common.cuh"

using namespace rsvdt;

static const double kPi = 3.14159265358979323846;

namespace rsvdt {

bool cuda_ok(rsvdt_ctx *ctx, cudaError_t e, const char *what) {
  if (e == cudaSuccess) return true;
  if (ctx) {
    char buf[512];
    snprintf(buf, sizeof buf, "CUDA error in %s: %s", what, cudaGetErrorString(e));
    ctx->err = buf;
  }
  return false;
}

rsvdt_status set_err(rsvdt_ctx *ctx, rsvdt_status s, const char *fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (ctx) ctx->err = buf;
  return s;
}

void *dalloc(rsvdt_ctx *ctx, size_t bytes) {
  void *p = nullptr;
  if (bytes == 0) bytes = 16;
  if (cudaMalloc(&p, bytes) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  ctx->allocations.push_back(p);
  return p;
}

void dfree(rsvdt_ctx *ctx, void *p) {
  if (!p) return;
  for (auto &a : ctx->allocations)
    if (a == p) {
      cudaFree(p);
      a = nullptr;
      return;
    }
}

}  // namespace rsvdt

// ------------------------------------------------------------ helpers

static void free_graphs(rsvdt_ctx *ctx) {
  for (auto *gs : {ctx->step_graph, ctx->small_graph})
    for (int d = 0; d < 2; ++d)
      if (gs[d]) {
        cudaGraphExecDestroy(gs[d]);
        gs[d] = nullptr;
      }
}

static bool upload(rsvdt_ctx *ctx, void *dst, const void *src, size_t bytes) {
  return cuda_ok(ctx, cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice), "upload");
}

// Host CSR (int32) with complex values.
struct HostCSR {
  int64_t rows = 0, cols = 0;
  std::vector<int32_t> rowptr, col;
  std::vector<std::complex<double>> val;
};

static rsvdt_status csr_from_user(rsvdt_ctx *ctx, const char *name, int64_t rows, int64_t cols,
                                  const int64_t *rowptr, const int64_t *col, const double *val,
                                  HostCSR &m) {
  if (rows <= 0 || cols <= 0 || !rowptr || (!col && rowptr[rows] > rowptr[0]))
    return set_err(ctx, RSVDT_ERR_ARG, "%s: invalid CSR arguments", name);
  const int64_t nnz = rowptr[rows] - rowptr[0];
  if (rows >= INT32_MAX || cols >= INT32_MAX || nnz >= INT32_MAX || nnz < 0)
    return set_err(ctx, RSVDT_ERR_ARG, "%s: sizes exceed the 32-bit device index range", name);
  m.rows = rows;
  m.cols = cols;
  m.rowptr.resize(rows + 1);
  m.col.resize(nnz);
  m.val.resize(nnz);
  for (int64_t i = 0; i <= rows; ++i) {
    m.rowptr[i] = (int32_t)(rowptr[i] - rowptr[0]);
    if (i > 0 && m.rowptr[i] < m.rowptr[i - 1])
      return set_err(ctx, RSVDT_ERR_ARG, "%s: row pointers decrease at row %lld", name, (long long)i);
  }
  for (int64_t j = 0; j < nnz; ++j) {
    const int64_t c = col[rowptr[0] + j];
    if (c < 0 || c >= cols)
      return set_err(ctx, RSVDT_ERR_ARG, "%s: column index %lld out of range [0, %lld)", name,
                     (long long)c, (long long)cols);
    m.col[j] = (int32_t)c;
    m.val[j] = {val[2 * (rowptr[0] + j)], val[2 * (rowptr[0] + j) + 1]};
  }
  return RSVDT_OK;
}

// Conjugate transpose; rows of the result list the original rows in
// ascending order (the accumulation order of SeqAIJ
// MatMultHermitianTransposeAdd).
static HostCSR conj_transpose(const HostCSR &a) {
  HostCSR t;
  t.rows = a.cols;
  t.cols = a.rows;
  const int64_t nnz = (int64_t)a.col.size();
  t.rowptr.assign(t.rows + 1, 0);
  t.col.resize(nnz);
  t.val.resize(nnz);
  for (int64_t j = 0; j < nnz; ++j) t.rowptr[a.col[j] + 1]++;
  for (int64_t i = 0; i < t.rows; ++i) t.rowptr[i + 1] += t.rowptr[i];
  std::vector<int32_t> fill(t.rowptr.begin(), t.rowptr.end() - 1);
  for (int64_t i = 0; i < a.rows; ++i)
    for (int32_t j = a.rowptr[i]; j < a.rowptr[i + 1]; ++j) {
      const int32_t c = a.col[j];
      t.col[fill[c]] = (int32_t)i;
      t.val[fill[c]] = std::conj(a.val[j]);
      fill[c]++;
    }
  return t;
}

static rsvdt_status upload_csr(rsvdt_ctx *ctx, const HostCSR &h, DevCSR &d, bool with32) {
  d.rows = h.rows;
  d.cols = h.cols;
  d.nnz = (int64_t)h.col.size();
  d.rowptr = (int32_t *)dalloc(ctx, sizeof(int32_t) * (h.rows + 1));
  d.col = (int32_t *)dalloc(ctx, sizeof(int32_t) * (d.nnz ? d.nnz : 1));
  d.val = (z128 *)dalloc(ctx, sizeof(z128) * (d.nnz ? d.nnz : 1));
  if (!d.rowptr || !d.col || !d.val) return set_err(ctx, RSVDT_ERR_OOM, "device allocation for a sparse matrix failed");
  if (!upload(ctx, d.rowptr, h.rowptr.data(), sizeof(int32_t) * (h.rows + 1)) ||
      (d.nnz && !upload(ctx, d.col, h.col.data(), sizeof(int32_t) * d.nnz)) ||
      (d.nnz && !upload(ctx, d.val, h.val.data(), sizeof(z128) * d.nnz)))
    return RSVDT_ERR_CUDA;
  if (with32) {
    std::vector<z64> v32(d.nnz);
    for (int64_t j = 0; j < d.nnz; ++j) v32[j] = zmake<z64>((float)h.val[j].real(), (float)h.val[j].imag());
    d.val32 = (z64 *)dalloc(ctx, sizeof(z64) * (d.nnz ? d.nnz : 1));
    if (!d.val32) return set_err(ctx, RSVDT_ERR_OOM, "device allocation for a sparse matrix failed");
    if (d.nnz && !upload(ctx, d.val32, v32.data(), sizeof(z64) * d.nnz)) return RSVDT_ERR_CUDA;
  }
  bool diag = h.rows == h.cols;
  for (int64_t i = 0; i < h.rows && diag; ++i)
    diag = (h.rowptr[i + 1] - h.rowptr[i] == 1) && h.col[h.rowptr[i]] == i;
  d.diag = diag;
  d.present = true;
  return RSVDT_OK;
}

static void free_csr(rsvdt_ctx *ctx, DevCSR &d) {
  dfree(ctx, d.rowptr);
  dfree(ctx, d.col);
  dfree(ctx, d.val);
  dfree(ctx, d.val32);
  d = DevCSR();
}

static void free_bcsr(rsvdt_ctx *ctx, DevBCSR &d) {
  dfree(ctx, d.browptr);
  dfree(ctx, d.bcol);
  dfree(ctx, d.val);
  dfree(ctx, d.val32);
  d = DevBCSR();
}

// SetupTimeFreqGrid (SourceCode/SetupTimeFreqGrid.c:16-21) and the DFT /
// iDFT tables (SourceCode/CreateDFTiDFTMats.c:18-93), computed on the host
// exactly as the reference forms them and stored for the device:
// tab[jt][iw] = idft[iw][jt], dft[iw][p].
static rsvdt_status setup_grid_and_tables(rsvdt_ctx *ctx) {
  const rsvdt_params &p = ctx->par;
  ctx->w = p.w * (p.TwoPI ? 2 * kPi : 1);  // SourceCode/ReadUserInput.c:82
  const double T = 2 * kPi / ctx->w;
  const double dt_w = T / (double)p.Nw;
  ctx->dt = dt_w / std::ceil(dt_w / p.dt);
  ctx->Ns = (int64_t)std::llround(T / ctx->dt);
  ctx->Nt = (int64_t)std::llround(p.TransientLength / ctx->dt);
  ctx->Nw = p.Nw;
  ctx->R = ctx->Ns / p.Nw;
  ctx->Nw_eff = ctx->real_op ? p.Nw / 2 : p.Nw;  // SourceCode/LNSStructure.c:44
  ctx->pair = !ctx->real_op && ctx->Nw_eff % 2 == 0;
  if (ctx->R < 1 || ctx->Nw_eff < 1)
    return set_err(ctx, RSVDT_ERR_ARG, "time grid is degenerate (Ns=%lld, Nw=%lld)", (long long)ctx->Ns,
                   (long long)p.Nw);
  const int64_t Nwe = ctx->Nw_eff, Nt2 = 2 * ctx->Ns, Nw = ctx->Nw;
  std::vector<z128> tab((size_t)Nt2 * Nwe);
  std::vector<z64> tab32((size_t)Nt2 * Nwe);
  const double alpha_im = -2 * kPi / (double)Nt2;
  for (int64_t iw = 0; iw < Nwe; ++iw) {
    int64_t f;
    if (ctx->real_op)
      f = iw;
    else if (Nwe % 2 == 0)
      f = (iw <= Nwe / 2 - 1) ? iw : (iw - Nwe) + Nt2;
    else
      f = (iw <= (Nwe - 1) / 2) ? iw : (iw - Nwe) + Nt2;
    const double v_im = alpha_im * (double)f;
    for (int64_t it = 0; it < Nt2; ++it) {
      const double y = v_im * (double)it;
      const double s = 2. / (double)Nt2;
      const z128 e = zmake<z128>(std::cos(y) * s, -std::sin(y) * s);
      tab[(size_t)(it * Nwe + iw)] = e;
      tab32[(size_t)(it * Nwe + iw)] = zmake<z64>((float)e.re, (float)e.im);
    }
  }
  // The reference's `Nw` in this formula is the column count of idft, i.e.
  // Nw_eff (SourceCode/CreateDFTiDFTMats.c:26): alpha = -2 pi i / (2 Nw_eff)
  // for a real operator, -2 pi i / Nw_eff otherwise; its sample vector J has
  // 2 Nw_eff (real) or Nw_eff entries, which must equal the Nw snapshot rows
  // (an odd Nw with a real operator is a size mismatch there, and an error
  // here).
  if (ctx->real_op && 2 * Nwe != Nw)
    return set_err(ctx, RSVDT_ERR_ARG, "a real-valued operator needs an even Nw (Nw = %lld)", (long long)Nw);
  std::vector<z128> dft((size_t)Nwe * Nw);
  const double a_dft = ctx->real_op ? -2 * kPi / (double)(2 * Nwe) : -2 * kPi / (double)Nwe;
  for (int64_t iw = 0; iw < Nwe; ++iw) {
    const double v_im = a_dft * (double)iw;
    for (int64_t j = 0; j < Nw; ++j) {
      const double y = v_im * (double)j;
      dft[(size_t)(iw * Nw + j)] = zmake<z128>(std::cos(y), std::sin(y));
    }
  }
  dfree(ctx, ctx->tab);
  dfree(ctx, ctx->tab32);
  dfree(ctx, ctx->dft);
  ctx->tab = (z128 *)dalloc(ctx, sizeof(z128) * tab.size());
  ctx->tab32 = (z64 *)dalloc(ctx, sizeof(z64) * tab32.size());
  ctx->dft = (z128 *)dalloc(ctx, sizeof(z128) * dft.size());
  if (!ctx->tab || !ctx->tab32 || !ctx->dft) return set_err(ctx, RSVDT_ERR_OOM, "table allocation failed");
  if (!upload(ctx, ctx->tab, tab.data(), sizeof(z128) * tab.size()) ||
      !upload(ctx, ctx->tab32, tab32.data(), sizeof(z64) * tab32.size()) ||
      !upload(ctx, ctx->dft, dft.data(), sizeof(z128) * dft.size()))
    return RSVDT_ERR_CUDA;
  free_graphs(ctx);
  return RSVDT_OK;
}

// Device buffers for K test vectors.
// Complex values of each of the capacity mode's two chunk buffers (the
// ring and the forcing slabs, which double as temporaries of the chunked
// weight products) for a chunk of Ks test vectors.
static size_t cap_chunk_elems(const rsvdt_ctx *ctx, int64_t Ks, int64_t rows) {
  const int64_t Nstore = ctx->Nw + 1;
  return (size_t)std::max(Nstore * ctx->N, rows * ctx->Nw_eff) * Ks;
}

// Largest chunk (a divisor of K) whose buffers fit in the free device
// memory, counting the working block if it is not allocated yet and the
// transient-removal buffers.
static int64_t cap_choose_chunk(rsvdt_ctx *ctx, int64_t K, int64_t rows) {
  size_t fr = 0, tot = 0;
  if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  // Buffers this context would free before allocating new ones.
  size_t held = 0;
  if (ctx->y) held += sizeof(z128) * 6 * (size_t)ctx->N * ctx->Ks;
  if (ctx->ring) held += sizeof(z128) * 2 * cap_chunk_elems(ctx, ctx->Ks, rows);
  size_t avail = fr + held;
  const size_t blk = sizeof(z128) * (size_t)rows * ctx->Nw_eff * K;
  if (!ctx->blk || ctx->blk_elems < (size_t)rows * ctx->Nw_eff * K) avail = avail > blk ? avail - blk : 0;
  const size_t tr = ctx->par.TransientRemoval
                        ? sizeof(z128) * (2 * (size_t)ctx->N * (ctx->Nw + 1) + 2 * (size_t)ctx->N * ctx->Nw_eff)
                        : 0;
  // Gram partials of the CholQR passes (chunks of 2048 rows x nw x K^2).
  const size_t gram = sizeof(z128) * (size_t)((rows + 2047) / 2048 + 8) * ctx->Nw_eff * K * K;
  const size_t margin = ((size_t)2 << 30) + tr + gram;
  for (int64_t kc = K; kc >= 1; --kc) {
    if (K % kc) continue;
    const size_t need = sizeof(z128) * (6 * (size_t)ctx->N * kc + 2 * cap_chunk_elems(ctx, kc, rows)) + margin;
    if (need <= avail) return kc;
  }
  return 1;
}

static rsvdt_status ensure_buffers(rsvdt_ctx *ctx, int64_t K) {
  const int64_t N = ctx->N, Nwe = ctx->Nw_eff;
  const int64_t rows = std::max(N, std::max(ctx->Nb, ctx->Nc));
  const size_t blk_elems = (size_t)rows * Nwe * K;
  const int64_t Nstore = ctx->Nw + 1;  // room for the transient-removal sample
  int64_t Ks = K;
  if (ctx->capacity) {
    Ks = ctx->cap_kc > 0 ? ctx->cap_kc : cap_choose_chunk(ctx, K, rows);
    if (K % Ks != 0)
      return set_err(ctx, RSVDT_ERR_ARG, "capacity chunk %lld does not divide k = %lld", (long long)Ks, (long long)K);
  }
  if (ctx->K == K && ctx->Ks == Ks && ctx->y && ctx->blk_elems >= blk_elems && ctx->buf_capacity == ctx->capacity)
    return RSVDT_OK;
  free_graphs(ctx);
  ++ctx->blk_version;
  void **bufs[] = {&ctx->y, &ctx->zA, &ctx->zB, &ctx->acc, &ctx->F2, &ctx->F3};
  for (auto b : bufs) {
    dfree(ctx, *b);
    *b = dalloc(ctx, sizeof(z128) * N * Ks);
    if (!*b) return set_err(ctx, RSVDT_ERR_OOM, "state allocation failed");
  }
  dfree(ctx, ctx->ring);
  dfree(ctx, ctx->Fh);
  dfree(ctx, ctx->blk2);
  ctx->blk2 = nullptr;
  if (ctx->capacity) {
    const size_t ce = cap_chunk_elems(ctx, Ks, rows);
    ctx->ring = dalloc(ctx, sizeof(z128) * ce);
    ctx->Fh = dalloc(ctx, sizeof(z128) * ce);
    ctx->Fh_bytes = ctx->Fh ? sizeof(z128) * ce : 0;
  } else {
    ctx->ring = dalloc(ctx, sizeof(z128) * Nstore * N * K);
    ctx->Fh = dalloc(ctx, sizeof(z128) * N * Nwe * K);
    ctx->Fh_bytes = ctx->Fh ? sizeof(z128) * N * Nwe * K : 0;
  }
  if (ctx->capacity) {
    // One working block, re-allocated only when it must grow (its contents
    // are then lost: set the weights before the sketch).
    if (!ctx->blk || ctx->blk_elems < blk_elems) {
      dfree(ctx, ctx->blk);
      ctx->blk = (z128 *)dalloc(ctx, sizeof(z128) * blk_elems);
      ctx->blk_elems = ctx->blk ? blk_elems : 0;
    }
  } else {
    // Keep the working block's contents when it is only re-sized upward.
    z128 *old = ctx->blk;
    size_t old_elems = ctx->blk_elems;
    z128 *nb = (z128 *)dalloc(ctx, sizeof(z128) * blk_elems);
    if (nb && old) cudaMemcpy(nb, old, sizeof(z128) * std::min(old_elems, blk_elems), cudaMemcpyDeviceToDevice);
    dfree(ctx, old);
    ctx->blk = nb;
    ctx->blk2 = (z128 *)dalloc(ctx, sizeof(z128) * blk_elems);
    ctx->blk_elems = blk_elems;
  }
  dfree(ctx, ctx->S);
  ctx->S = (double *)dalloc(ctx, sizeof(double) * Nwe * K);
  if (!ctx->ring || !ctx->Fh || !ctx->blk || (!ctx->capacity && !ctx->blk2) || !ctx->S)
    return set_err(ctx, RSVDT_ERR_OOM, "spectral block allocation failed (%zu complex values each)", blk_elems);
  ctx->K = K;
  ctx->Ks = Ks;
  ctx->k0 = 0;
  ctx->buf_capacity = ctx->capacity;
  return RSVDT_OK;
}

// Nb / Nc from the weights known so far (SourceCode/ReadWeightMats.c:50-52,
// 90, 95); no cross-checks.
static void update_dims(rsvdt_ctx *ctx) {
  ctx->Nb = ctx->W[RSVDT_B].present ? ctx->W[RSVDT_B].cols : ctx->N;
  ctx->Nc = ctx->W[RSVDT_C].present ? ctx->W[RSVDT_C].rows : ctx->N;
}

static rsvdt_status check_weights(rsvdt_ctx *ctx) {
  // SourceCode/ReadWeightMats.c:26-99 size rules.
  const int64_t N = ctx->N;
  DevCSR *W = ctx->W;
  int64_t nb = W[RSVDT_B].present ? W[RSVDT_B].cols : N;
  int64_t nc = W[RSVDT_C].present ? W[RSVDT_C].rows : N;
  if (W[RSVDT_B].present && W[RSVDT_B].rows != N)
    return set_err(ctx, RSVDT_ERR_ARG, "Input matrix (B) must have %lld rows, current size = %lld x %lld",
                   (long long)N, (long long)W[RSVDT_B].rows, (long long)W[RSVDT_B].cols);
  if (W[RSVDT_W_F_SQRT_INV].present && W[RSVDT_W_F_SQRT_INV].cols != nb)
    return set_err(ctx, RSVDT_ERR_ARG,
                   "Size mismatch between input matrix (B) and input weight matrix (W_f_sqrt_inv), %lld != %lld",
                   (long long)nb, (long long)W[RSVDT_W_F_SQRT_INV].cols);
  if (W[RSVDT_C].present && W[RSVDT_C].cols != N)
    return set_err(ctx, RSVDT_ERR_ARG, "Output matrix (C) must have %lld columns, current size = %lld x %lld",
                   (long long)N, (long long)W[RSVDT_C].rows, (long long)W[RSVDT_C].cols);
  if (W[RSVDT_W_Q_SQRT].present && W[RSVDT_W_Q_SQRT].rows != nc)
    return set_err(ctx, RSVDT_ERR_ARG,
                   "Size mismatch between output matrix (C) and output weight matrix (W_q_sqrt), %lld != %lld",
                   (long long)nc, (long long)W[RSVDT_W_Q_SQRT].rows);
  if (W[RSVDT_W_Q_SQRT_INV].present && W[RSVDT_W_Q_SQRT_INV].rows != nc)
    return set_err(ctx, RSVDT_ERR_ARG,
                   "Size mismatch between output matrix (C) and inverse output weight matrix (W_q_sqrt_inv), %lld != %lld",
                   (long long)nc, (long long)W[RSVDT_W_Q_SQRT_INV].rows);
  ctx->Nb = nb;
  ctx->Nc = nc;
  return RSVDT_OK;
}

#define RSVDT_TRY(x)                   \
  do {                                 \
    rsvdt_status _s = (x);             \
    if (_s != RSVDT_OK) return _s;     \
  } while (0)

// Y <- M Y on the working block: ping-pong between blk and blk2, or in
// capacity mode chunk by chunk through the forcing-slab and ring buffers
// (each chunk is its own columns of the block, so chunks never overlap,
// whatever the row counts).
static rsvdt_status weight_step(rsvdt_ctx *ctx, const DevCSR &M, int64_t rows_in) {
  if (!M.present) return RSVDT_OK;
  if (M.cols != rows_in)
    return set_err(ctx, RSVDT_ERR_ARG, "weight product: %lld columns but the block has %lld rows",
                   (long long)M.cols, (long long)rows_in);
  if (ctx->capacity) {
    const int64_t K = ctx->K, Ks = ctx->Ks, Nwe = ctx->Nw_eff;
    z128 *tA = (z128 *)ctx->Fh, *tB = (z128 *)ctx->ring;
    for (int64_t k0 = 0; k0 < K; k0 += Ks) {
      RSVDT_TRY(launch_chunk_copy(ctx, ctx->blk, tA, rows_in, Nwe, K, k0, Ks, true));
      RSVDT_TRY(apply_weight(ctx, M, tA, tB, Nwe * Ks));
      RSVDT_TRY(launch_chunk_copy(ctx, tB, ctx->blk, M.rows, Nwe, K, k0, Ks, false));
    }
  } else {
    RSVDT_TRY(apply_weight(ctx, M, ctx->blk, ctx->blk2, ctx->Nw_eff * ctx->K));
    std::swap(ctx->blk, ctx->blk2);
  }
  ctx->blk_rows = M.rows;
  ++ctx->blk_version;
  return RSVDT_OK;
}

// Stages the working block (N rows) as the action's forcing slabs in the
// action's precision (TSActionRK4 copies Y_hat to F_hat,
// SourceCode/TSActionRK4.c:49).
static rsvdt_status stage_forcing(rsvdt_ctx *ctx, int prec) { return stage_forcing_coeffs(ctx, prec); }

// Stages the forcing slabs unless they already hold the working block's
// current contents in this precision.
static rsvdt_status stage_forcing_cached(rsvdt_ctx *ctx, int prec) {
  if (ctx->staged_version == ctx->blk_version && ctx->staged_prec == prec && ctx->k0 == 0) return RSVDT_OK;
  RSVDT_TRY(stage_forcing(ctx, prec));
  ctx->staged_version = ctx->blk_version;
  ctx->staged_prec = prec;
  return RSVDT_OK;
}


namespace rsvdt {
static rsvdt_status cap_action(rsvdt_ctx *ctx, int d);
}

// ---------------------------------------------------- progress and timing

static double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

static void print_hms(const char *prefix, double sec, const char *suffix) {
  const int t = (int)sec, hh = t / 3600, mm = (t - 3600 * hh) / 60, ss = t - 3600 * hh - 60 * mm;
  printf("%s%02d:%02d:%02d%s", prefix, hh, mm, ss, suffix);
  fflush(stdout);  // as PetscPrintf: visible at once, also through a pipe
}

// The RK4 steps of an action (all test vectors of the chunk at once), with
// the progress lines of SourceCode/DisplayProgress.c:18-50: every 10% of
// the steps at Display = 2 (the stepping then runs in ten pieces, each
// ended by a synchronisation), the elapsed time at Display >= 1.
static rsvdt_status steps_with_progress(rsvdt_ctx *ctx, int d, int prec, int64_t rend) {
  const double t0 = now_s();
  if (ctx->par.Display >= 2 && rend >= 10) {
    int64_t done = 0;
    for (int p = 0; p < 10; ++p) {
      const int64_t upto = rend * (p + 1) / 10;
      printf("Progress percentage: %d%%\n", 10 * p);
      print_hms("Elapsed time = ", now_s() - t0, "\n");
      RSVDT_TRY(run_steps(ctx, d, prec, 1 + done, upto - done, true));
      if (!cuda_ok(ctx, cudaStreamSynchronize(ctx->stream), "sync")) return RSVDT_ERR_CUDA;
      done = upto;
    }
    printf("Progress percentage: 100%%\n");
    fflush(stdout);
  } else {
    RSVDT_TRY(run_steps(ctx, d, prec, 1, rend, true));
    if (!cuda_ok(ctx, cudaStreamSynchronize(ctx->stream), "sync")) return RSVDT_ERR_CUDA;
  }
  const double el = now_s() - t0;
  ctx->tm.stepping += el;
  ctx->tm.steps += rend;
  if (ctx->par.Display >= 1) {
    char tail[96];
    snprintf(tail, sizeof tail, " (k = %lld out of %lld)\n", (long long)(ctx->k0 + ctx->Ks), (long long)ctx->K);
    print_hms("Elapsed time = ", el, tail);
  }
  return RSVDT_OK;
}

// ---------------------------------------------------------- capacity mode

// Free host memory in bytes (what can be allocated without swapping).
static size_t host_avail_bytes() {
  const long pages = sysconf(_SC_AVPHYS_PAGES), psz = sysconf(_SC_PAGESIZE);
  return pages > 0 && psz > 0 ? (size_t)pages * (size_t)psz : 0;
}

// StoreU in capacity mode (SourceCode/StoreU.c:15): U goes to host memory
// chunk by chunk, already multiplied by W_q^{-1/2} (SourceCode/SVDAllFreqs.c:63
// applies it at the end; U does not change in between), in complex128 or
// complex64, layout [row][iw][kc] per chunk.
static rsvdt_status cap_store_u(rsvdt_ctx *ctx, int64_t rows) {
  const int64_t K = ctx->K, Ks = ctx->Ks, Nwe = ctx->Nw_eff;
  const DevCSR &Wi = ctx->W[RSVDT_W_Q_SQRT_INV];
  if (Wi.present && Wi.cols != rows)
    return set_err(ctx, RSVDT_ERR_ARG, "W_q^{-1/2} has %lld columns, U has %lld rows", (long long)Wi.cols,
                   (long long)rows);
  const int64_t urows = Wi.present ? Wi.rows : rows;
  const size_t es = ctx->cap_u_c64 ? sizeof(z64) : sizeof(z128);
  const size_t cbytes = es * (size_t)urows * Nwe * Ks;
  const int64_t nch = K / Ks;
  ctx->u_host.clear();
  const size_t need = cbytes * (size_t)nch, margin = (size_t)8 << 30;
  if (need + margin > host_avail_bytes())
    return set_err(ctx, RSVDT_ERR_OOM,
                   "U needs %.1f GB of host memory and %.1f GB are free (complex64 storage halves it)",
                   need / 1e9, host_avail_bytes() / 1e9);
  z128 *tA = (z128 *)ctx->Fh, *tB = (z128 *)ctx->ring;
  for (int64_t c = 0; c < nch; ++c) {
    std::vector<unsigned char> h;
    try {
      h.resize(cbytes);
    } catch (...) {
      ctx->u_host.clear();
      return set_err(ctx, RSVDT_ERR_OOM, "host allocation of %zu bytes for U failed", cbytes);
    }
    RSVDT_TRY(launch_chunk_copy(ctx, ctx->blk, tA, rows, Nwe, K, c * Ks, Ks, true));
    const z128 *src = tA;
    if (Wi.present) {
      RSVDT_TRY(apply_weight(ctx, Wi, tA, tB, Nwe * Ks));
      src = tB;
    }
    const void *dsrc = src;
    if (ctx->cap_u_c64) {
      z64 *d64 = (z64 *)(src == tA ? tB : tA);
      RSVDT_TRY(launch_convert_to64(ctx, src, d64, urows * Nwe * Ks));
      dsrc = d64;
    }
    if (!cuda_ok(ctx, cudaMemcpyAsync(h.data(), dsrc, cbytes, cudaMemcpyDeviceToHost, ctx->stream), "U download") ||
        !cuda_ok(ctx, cudaStreamSynchronize(ctx->stream), "sync"))
      return RSVDT_ERR_CUDA;
    ctx->u_host.push_back(std::move(h));
  }
  ctx->U_rows = urows;
  return RSVDT_OK;
}

// SVDAllFreqsBeforeAdjoint + StoreU, or SVDAllFreqs, in capacity mode: the
// SVD is in place (the block becomes U, or V), U goes to the host, and
// V <- W_f^{-1/2} V is applied chunk by chunk in the block.
static rsvdt_status cap_svd(rsvdt_ctx *ctx, bool before_adjoint) {
  const int64_t rows = ctx->blk_rows;
  if (!before_adjoint && ctx->u_host.empty())
    return set_err(ctx, RSVDT_ERR_STATE, "U has not been stored (run the SVD before the adjoint first)");
  RSVDT_TRY(svd_all(ctx, ctx->blk, rows, ctx->Nw_eff, ctx->K, nullptr, ctx->S));
  if (before_adjoint) {
    RSVDT_TRY(cap_store_u(ctx, rows));
  } else {
    RSVDT_TRY(weight_step(ctx, ctx->W[RSVDT_W_F_SQRT_INV], rows));
    ctx->have_results = true;
  }
  return cuda_ok(ctx, cudaStreamSynchronize(ctx->stream), "sync") ? RSVDT_OK : RSVDT_ERR_CUDA;
}

// Columns cols[0..ncols) (indices iw*K + k; all C columns when cols is
// null) of a device block [row][iw][k] (rows x C) into a column-major host
// array, through row batches of about 64 MB.
static rsvdt_status block_cols_to_host(rsvdt_ctx *ctx, const z128 *src, int64_t rows, int64_t C, const int64_t *cols,
                                       int64_t ncols, double *out, int64_t ld) {
  const int64_t batch = std::max<int64_t>(1, ((int64_t)64 << 20) / (int64_t)(sizeof(z128) * C));
  std::vector<z128> tmp((size_t)std::min(rows, batch) * C);
  for (int64_t r0 = 0; r0 < rows; r0 += batch) {
    const int64_t nr = std::min(batch, rows - r0);
    if (!cuda_ok(ctx, cudaMemcpyAsync(tmp.data(), src + r0 * C, sizeof(z128) * nr * C, cudaMemcpyDeviceToHost,
                                      ctx->stream),
                 "download") ||
        !cuda_ok(ctx, cudaStreamSynchronize(ctx->stream), "sync"))
      return RSVDT_ERR_CUDA;
    for (int64_t j = 0; j < ncols; ++j) {
      const int64_t c = cols ? cols[j] : j;
      double *o = out + 2 * (j * ld + r0);
      for (int64_t r = 0; r < nr; ++r) {
        const z128 v = tmp[(size_t)(r * C + c)];
        o[2 * r] = v.re;
        o[2 * r + 1] = v.im;
      }
    }
  }
  return RSVDT_OK;
}

// The same from the host copy of U (capacity mode).
static void host_u_cols(const rsvdt_ctx *ctx, const int64_t *cols, int64_t ncols, double *out, int64_t ld) {
  const int64_t K = ctx->K, Ks = ctx->Ks, Nwe = ctx->Nw_eff, rows = ctx->U_rows;
  for (int64_t j = 0; j < ncols; ++j) {
    const int64_t col = cols ? cols[j] : j;
    const int64_t iw = col / K, k = col % K, c = k / Ks, kc = k % Ks;
    double *o = out + 2 * j * ld;
    if (ctx->cap_u_c64) {
      const z64 *h = (const z64 *)ctx->u_host[(size_t)c].data();
      for (int64_t r = 0; r < rows; ++r) {
        const z64 v = h[(size_t)((r * Nwe + iw) * Ks + kc)];
        o[2 * r] = v.re;
        o[2 * r + 1] = v.im;
      }
    } else {
      const z128 *h = (const z128 *)ctx->u_host[(size_t)c].data();
      for (int64_t r = 0; r < rows; ++r) {
        const z128 v = h[(size_t)((r * Nwe + iw) * Ks + kc)];
        o[2 * r] = v.re;
        o[2 * r + 1] = v.im;
      }
    }
  }
}


static rsvdt_status require_ready(rsvdt_ctx *ctx, bool need_block) {
  if (!ctx) return RSVDT_ERR_ARG;
  if (!ctx->have_operator) return set_err(ctx, RSVDT_ERR_STATE, "the operator has not been set");
  if (need_block && !ctx->have_block) return set_err(ctx, RSVDT_ERR_STATE, "no sketch / working block");
  return RSVDT_OK;
}

// ---------------------------------------------------------------- ABI

extern "C" {

void rsvdt_default_params(rsvdt_params *p) {
  std::memset(p, 0, sizeof(*p));
  p->k = 3;  // SourceCode/ReadUserInput.c:109-113
  p->q = 0;  // :114-118
  p->Nw = 0;
  p->w = 0;
  p->TwoPI = 0;
  p->dt = 0;
  p->TransientLength = 0;
  p->TransientRemoval = 0;
  p->DiscFlg = 0;
  p->beta = 0;
  p->precision = RSVDT_PREC_C128;
  p->Display = 2;  // :126-130
}

rsvdt_status rsvdt_create(const rsvdt_params *p, rsvdt_ctx **out) {
  if (!p || !out) return RSVDT_ERR_ARG;
  *out = nullptr;
  rsvdt_ctx *ctx = new rsvdt_ctx();
  ctx->par = *p;
  ctx->act_prec = base_precision(p->precision);
  rsvdt_status st = RSVDT_OK;
  if (p->k < 1) st = set_err(ctx, RSVDT_ERR_ARG, "'k' must be positive, current value: %lld", (long long)p->k);
  else if (p->q < 0) st = set_err(ctx, RSVDT_ERR_ARG, "'q' must be non-negative, current value: %lld", (long long)p->q);
  else if (p->Nw < 1) st = set_err(ctx, RSVDT_ERR_ARG, "Must specify 'Nw'");
  else if (!(p->w > 0)) st = set_err(ctx, RSVDT_ERR_ARG, "Must specify 'w' (a positive base frequency)");
  else if (!(p->dt > 0)) st = set_err(ctx, RSVDT_ERR_ARG, "Must specify 'dt' (a positive time step)");
  else if (!(p->TransientLength >= 0)) st = set_err(ctx, RSVDT_ERR_ARG, "Must specify 'TransientLength'");
  else if (p->DiscFlg && p->beta < 0)
    st = set_err(ctx, RSVDT_ERR_ARG, "'beta' must be positive, current value: %g", p->beta);
  else if (p->precision != RSVDT_PREC_C128 && p->precision != RSVDT_PREC_C64 &&
           p->precision != RSVDT_PREC_C64_REFINE)
    st = set_err(ctx, RSVDT_ERR_ARG, "unknown precision %d", (int)p->precision);
  if (st == RSVDT_OK) {
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev < 1) {
      cudaGetLastError();
      st = set_err(ctx, RSVDT_ERR_CUDA, "no CUDA device available (%s)", cudaGetErrorString(e));
    }
  }
  if (st == RSVDT_OK) {
    cudaGetDevice(&ctx->device);
    if (!cuda_ok(ctx, cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking), "stream create"))
      st = RSVDT_ERR_CUDA;
  }
  if (st == RSVDT_OK) {
    ctx->d_step = (int64_t *)dalloc(ctx, sizeof(int64_t) * 4);
    ctx->d_flags = (int32_t *)dalloc(ctx, sizeof(int32_t) * 4);
    if (!ctx->d_step || !ctx->d_flags) st = set_err(ctx, RSVDT_ERR_OOM, "device allocation failed");
  }
  if (st != RSVDT_OK) {
    // Keep the context so that rsvdt_last_error can report; the caller
    // destroys it.
    *out = ctx;
    return st;
  }
  ctx->K = 0;
  *out = ctx;
  return RSVDT_OK;
}

void rsvdt_destroy(rsvdt_ctx *ctx) {
  if (!ctx) return;
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  free_graphs(ctx);
  for (void *p : ctx->allocations)
    if (p) cudaFree(p);
  if (ctx->stream && ctx->owns_stream) cudaStreamDestroy(ctx->stream);
  if (ctx->io_stream) {
    cudaStreamSynchronize(ctx->io_stream);
    cudaStreamDestroy(ctx->io_stream);
  }
  if (ctx->io_event) cudaEventDestroy(ctx->io_event);
  if (ctx->up_event) cudaEventDestroy(ctx->up_event);
  for (auto &e : ctx->slab_event)
    if (e) cudaEventDestroy(e);
  delete ctx;
}

const char *rsvdt_last_error(const rsvdt_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

rsvdt_status rsvdt_set_operator(rsvdt_ctx *ctx, int64_t N, const int64_t *rowptr, const int64_t *col,
                                const double *val) {
  if (!ctx) return RSVDT_ERR_ARG;
  HostCSR A;
  RSVDT_TRY(csr_from_user(ctx, "operator A", N, N, rowptr, col, val, A));
  // Real-valued check (SourceCode/LNSStructure.c:37-44).
  double im2 = 0;
  for (auto &v : A.val) im2 += v.imag() * v.imag();
  ctx->real_op = std::sqrt(im2) < 1e-12;
  // Discounting A <- A - beta I (SourceCode/LNSStructure.c:53-56); MatShift
  // inserts missing diagonal entries.
  if (ctx->par.DiscFlg) {
    HostCSR B;
    B.rows = B.cols = N;
    B.rowptr.push_back(0);
    for (int64_t i = 0; i < N; ++i) {
      bool found = false;
      for (int32_t j = A.rowptr[i]; j < A.rowptr[i + 1]; ++j) {
        if (!found && A.col[j] > i) {
          B.col.push_back((int32_t)i);
          B.val.push_back(-ctx->par.beta);
          found = true;
        }
        std::complex<double> v = A.val[j];
        if (A.col[j] == i) {
          v -= ctx->par.beta;
          found = true;
        }
        B.col.push_back(A.col[j]);
        B.val.push_back(v);
      }
      if (!found) {
        B.col.push_back((int32_t)i);
        B.val.push_back(-ctx->par.beta);
      }
      B.rowptr.push_back((int32_t)B.col.size());
    }
    A = std::move(B);
  }
  HostCSR AH = conj_transpose(A);
  free_csr(ctx, ctx->A);
  free_csr(ctx, ctx->AH);
  free_bcsr(ctx, ctx->BA);
  free_bcsr(ctx, ctx->BAH);
  RSVDT_TRY(upload_csr(ctx, A, ctx->A, true));
  RSVDT_TRY(upload_csr(ctx, AH, ctx->AH, true));
  ctx->N = N;
  ctx->have_operator = true;
  update_dims(ctx);
  RSVDT_TRY(setup_grid_and_tables(ctx));
  return ensure_buffers(ctx, ctx->K > 0 ? ctx->K : ctx->par.k);
}

rsvdt_status rsvdt_set_operator_bcsr(rsvdt_ctx *ctx, int64_t nb, int32_t bs, const int64_t *browptr,
                                     const int64_t *bcol, const double *val) {
  if (!ctx) return RSVDT_ERR_ARG;
  if (nb <= 0 || bs <= 0 || bs > 16 || !browptr)
    return set_err(ctx, RSVDT_ERR_ARG, "invalid block-CSR arguments (nb=%lld, bs=%d)", (long long)nb, bs);
  const int64_t N = nb * bs;
  const int64_t nblk = browptr[nb] - browptr[0];
  if (N >= INT32_MAX || nblk < 0 || nblk >= INT32_MAX)
    return set_err(ctx, RSVDT_ERR_ARG, "block-CSR sizes exceed the 32-bit device index range");
  const int64_t bb = (int64_t)bs * bs;
  std::vector<int32_t> rp(nb + 1), cl(nblk);
  std::vector<std::complex<double>> vl(nblk * bb);
  double im2 = 0;
  for (int64_t i = 0; i <= nb; ++i) {
    rp[i] = (int32_t)(browptr[i] - browptr[0]);
    if (i > 0 && rp[i] < rp[i - 1]) return set_err(ctx, RSVDT_ERR_ARG, "block row pointers decrease");
  }
  for (int64_t j = 0; j < nblk; ++j) {
    const int64_t c = bcol[browptr[0] + j];
    if (c < 0 || c >= nb) return set_err(ctx, RSVDT_ERR_ARG, "block column %lld out of range", (long long)c);
    cl[j] = (int32_t)c;
  }
  for (int64_t e = 0; e < nblk * bb; ++e) {
    vl[e] = {val[2 * (browptr[0] * bb + e)], val[2 * (browptr[0] * bb + e) + 1]};
    im2 += vl[e].imag() * vl[e].imag();
  }
  ctx->real_op = std::sqrt(im2) < 1e-12;
  if (ctx->par.DiscFlg) {
    for (int64_t i = 0; i < nb; ++i) {
      bool found = false;
      for (int32_t j = rp[i]; j < rp[i + 1]; ++j)
        if (cl[j] == i) {
          for (int r = 0; r < bs; ++r) vl[(int64_t)j * bb + r * bs + r] -= ctx->par.beta;
          found = true;
        }
      if (!found)
        return set_err(ctx, RSVDT_ERR_ARG, "discounting needs a stored diagonal block in block row %lld",
                       (long long)i);
    }
  }
  // Conjugate transpose: block (I,J) -> (J,I) with each block conjugate-transposed.
  std::vector<int32_t> trp(nb + 1, 0), tcl(nblk);
  std::vector<std::complex<double>> tvl(nblk * bb);
  for (int64_t j = 0; j < nblk; ++j) trp[cl[j] + 1]++;
  for (int64_t i = 0; i < nb; ++i) trp[i + 1] += trp[i];
  std::vector<int32_t> fill(trp.begin(), trp.end() - 1);
  for (int64_t i = 0; i < nb; ++i)
    for (int32_t j = rp[i]; j < rp[i + 1]; ++j) {
      const int32_t d = fill[cl[j]]++;
      tcl[d] = (int32_t)i;
      for (int r = 0; r < bs; ++r)
        for (int c = 0; c < bs; ++c) tvl[(int64_t)d * bb + c * bs + r] = std::conj(vl[(int64_t)j * bb + r * bs + c]);
    }
  free_csr(ctx, ctx->A);
  free_csr(ctx, ctx->AH);
  free_bcsr(ctx, ctx->BA);
  free_bcsr(ctx, ctx->BAH);
  auto up = [&](DevBCSR &d, const std::vector<int32_t> &r, const std::vector<int32_t> &c,
                const std::vector<std::complex<double>> &v) -> rsvdt_status {
    d.bs = bs;
    d.nb = nb;
    d.nblocks = nblk;
    d.browptr = (int32_t *)dalloc(ctx, sizeof(int32_t) * (nb + 1));
    d.bcol = (int32_t *)dalloc(ctx, sizeof(int32_t) * (nblk ? nblk : 1));
    d.val = (z128 *)dalloc(ctx, sizeof(z128) * (nblk ? nblk * bb : 1));
    const int64_t s32 = bs == 5 ? 26 : bb;
    d.stride32 = (int32_t)s32;
    d.val32 = (z64 *)dalloc(ctx, sizeof(z64) * (nblk ? nblk * s32 : 1));
    if (!d.browptr || !d.bcol || !d.val || !d.val32) return set_err(ctx, RSVDT_ERR_OOM, "block-CSR allocation failed");
    std::vector<z64> v32((size_t)(nblk * s32), zmake<z64>(0.f, 0.f));
    for (int64_t j = 0; j < nblk; ++j)
      for (int64_t e = 0; e < bb; ++e) {
        const std::complex<double> x = v[(size_t)(j * bb + e)];
        v32[(size_t)(j * s32 + e)] = zmake<z64>((float)x.real(), (float)x.imag());
      }
    if (!upload(ctx, d.browptr, r.data(), sizeof(int32_t) * (nb + 1)) ||
        (nblk && !upload(ctx, d.bcol, c.data(), sizeof(int32_t) * nblk)) ||
        (nblk && !upload(ctx, d.val, v.data(), sizeof(z128) * nblk * bb)) ||
        (nblk && !upload(ctx, d.val32, v32.data(), sizeof(z64) * nblk * s32)))
      return RSVDT_ERR_CUDA;
    d.present = true;
    return RSVDT_OK;
  };
  RSVDT_TRY(up(ctx->BA, rp, cl, vl));
  RSVDT_TRY(up(ctx->BAH, trp, tcl, tvl));
  ctx->N = N;
  ctx->have_operator = true;
  update_dims(ctx);
  RSVDT_TRY(setup_grid_and_tables(ctx));
  return ensure_buffers(ctx, ctx->K > 0 ? ctx->K : ctx->par.k);
}

rsvdt_status rsvdt_set_weight(rsvdt_ctx *ctx, rsvdt_weight which, int64_t rows, int64_t cols,
                              const int64_t *rowptr, const int64_t *col, const double *val) {
  if (!ctx) return RSVDT_ERR_ARG;
  if ((int)which < 0 || (int)which > 4) return set_err(ctx, RSVDT_ERR_ARG, "unknown weight %d", (int)which);
  static const char *names[] = {"W_f_sqrt_inv", "B", "C", "W_q_sqrt", "W_q_sqrt_inv"};
  if ((which == RSVDT_W_F_SQRT_INV || which == RSVDT_W_Q_SQRT || which == RSVDT_W_Q_SQRT_INV) && rows != cols)
    return set_err(ctx, RSVDT_ERR_ARG, "%s must be square, current size = %lld x %lld", names[which],
                   (long long)rows, (long long)cols);
  HostCSR h;
  RSVDT_TRY(csr_from_user(ctx, names[which], rows, cols, rowptr, col, val, h));
  free_csr(ctx, ctx->W[which]);
  free_csr(ctx, ctx->WH[which]);
  RSVDT_TRY(upload_csr(ctx, h, ctx->W[which], false));
  RSVDT_TRY(upload_csr(ctx, conj_transpose(h), ctx->WH[which], false));
  // Sizes are cross-checked once all matrices are known (at the sketch and
  // at every action), as ReadWeightMats checks them after reading them all.
  if (ctx->have_operator) {
    update_dims(ctx);
    RSVDT_TRY(ensure_buffers(ctx, ctx->K > 0 ? ctx->K : ctx->par.k));
  }
  return RSVDT_OK;
}

rsvdt_status rsvdt_get_grid(const rsvdt_ctx *ctx, rsvdt_grid *g) {
  if (!ctx || !g) return RSVDT_ERR_ARG;
  if (!ctx->have_operator) return RSVDT_ERR_STATE;
  g->w = ctx->w;
  g->dt = ctx->dt;
  g->Ns = ctx->Ns;
  g->Nt = ctx->Nt;
  g->ResRatio = ctx->R;
  g->Nw_eff = ctx->Nw_eff;
  g->N = ctx->N;
  g->Nb = ctx->Nb;
  g->Nc = ctx->Nc;
  return RSVDT_OK;
}

rsvdt_status rsvdt_set_sketch(rsvdt_ctx *ctx, const double *F, int64_t ld, int64_t ncols) {
  RSVDT_TRY(require_ready(ctx, false));
  RSVDT_TRY(check_weights(ctx));
  if (!F || ld < ctx->Nb) return set_err(ctx, RSVDT_ERR_ARG, "invalid sketch arguments");
  if (ncols < ctx->Nw_eff || ncols % ctx->Nw_eff != 0)
    return set_err(ctx, RSVDT_ERR_ARG, "Input forcing must have a multiple of Nw_eff = %lld columns, current size = %lld x %lld",
                   (long long)ctx->Nw_eff, (long long)ctx->Nb, (long long)ncols);
  RSVDT_TRY(ensure_buffers(ctx, ncols / ctx->Nw_eff));
  const int64_t K = ctx->K, C = ctx->Nw_eff * K, rows = ctx->Nb;
  if (ctx->capacity) {
    // Row batches transposed on the host (no block-sized staging buffer).
    const int64_t batch = std::max<int64_t>(1, ((int64_t)64 << 20) / (int64_t)(sizeof(z128) * C));
    std::vector<z128> tmp((size_t)std::min(rows, batch) * C);
    for (int64_t r0 = 0; r0 < rows; r0 += batch) {
      const int64_t nr = std::min(batch, rows - r0);
      for (int64_t c = 0; c < C; ++c) {
        const double *f = F + 2 * (c * ld + r0);
        for (int64_t r = 0; r < nr; ++r) tmp[(size_t)(r * C + c)] = zmake<z128>(f[2 * r], f[2 * r + 1]);
      }
      if (!cuda_ok(ctx, cudaMemcpyAsync(ctx->blk + r0 * C, tmp.data(), sizeof(z128) * nr * C, cudaMemcpyHostToDevice,
                                        ctx->stream),
                   "upload") ||
          !cuda_ok(ctx, cudaStreamSynchronize(ctx->stream), "sync"))
        return RSVDT_ERR_CUDA;
    }
    ctx->blk_rows = rows;
    ctx->have_block = true;
  ++ctx->blk_version;
    ctx->have_results = false;
    return RSVDT_OK;
  }
  z128 *stage = (z128 *)dalloc(ctx, sizeof(z128) * ld * C);
  if (!stage) return set_err(ctx, RSVDT_ERR_OOM, "staging allocation failed");
  rsvdt_status st = RSVDT_OK;
  if (!cuda_ok(ctx, cudaMemcpyAsync(stage, F, sizeof(z128) * ld * C, cudaMemcpyHostToDevice, ctx->stream), "upload"))
    st = RSVDT_ERR_CUDA;
  if (!st) st = launch_colmajor_to_blk(ctx, stage, rows, ld, C, ctx->blk);
  if (!st && !cuda_ok(ctx, cudaStreamSynchronize(ctx->stream), "sync")) st = RSVDT_ERR_CUDA;
  dfree(ctx, stage);
  if (st) return st;
  ctx->blk_rows = rows;
  ctx->have_block = true;
  ++ctx->blk_version;
  ctx->have_results = false;
  return RSVDT_OK;
}

rsvdt_status rsvdt_random_sketch(rsvdt_ctx *ctx, uint64_t seed) {
  RSVDT_TRY(require_ready(ctx, false));
  RSVDT_TRY(launch_random(ctx, ctx->blk, ctx->Nb * ctx->Nw_eff * ctx->K, seed));
  ctx->blk_rows = ctx->Nb;
  ctx->have_block = true;
  ++ctx->blk_version;
  ctx->have_results = false;
  return cuda_ok(ctx, cudaStreamSynchronize(ctx->stream), "sync") ? RSVDT_OK : RSVDT_ERR_CUDA;
}

rsvdt_status rsvdt_get_block(rsvdt_ctx *ctx, double *Y, int64_t ld, int64_t *rows) {
  RSVDT_TRY(require_ready(ctx, true));
  const int64_t C = ctx->Nw_eff * ctx->K, r = ctx->blk_rows;
  if (rows) *rows = r;
  if (!Y) return RSVDT_OK;
  if (ld < r) return set_err(ctx, RSVDT_ERR_ARG, "ld (%lld) < rows (%lld)", (long long)ld, (long long)r);
  if (ctx->capacity) return block_cols_to_host(ctx, ctx->blk, r, C, nullptr, C, Y, ld);
  z128 *stage = (z128 *)dalloc(ctx, sizeof(z128) * ld * C);
  if (!stage) return set_err(ctx, RSVDT_ERR_OOM, "staging allocation failed");
  rsvdt_status st = launch_blk_to_colmajor(ctx, ctx->blk, r, C, stage, ld);
  if (!st && !cuda_ok(ctx, cudaMemcpyAsync(Y, stage, sizeof(z128) * ld * C, cudaMemcpyDeviceToHost, ctx->stream),
                      "download"))
    st = RSVDT_ERR_CUDA;
  if (!st && !cuda_ok(ctx, cudaStreamSynchronize(ctx->stream), "sync")) st = RSVDT_ERR_CUDA;
  dfree(ctx, stage);
  return st;
}

rsvdt_status rsvdt_action(rsvdt_ctx *ctx, rsvdt_dir dir) {
  RSVDT_TRY(require_ready(ctx, true));
  const int d = dir == RSVDT_DIRECT ? 1 : 0;
  NvtxRange range(d ? "rsvdt direct action" : "rsvdt adjoint action");
  const double t0 = now_s();
  ctx->tm.actions[d] += 1;
  rsvdt_status st;
  if (ctx->capacity) {
    st = cap_action(ctx, d);
  } else {
    int64_t rend = 0;
    RSVDT_TRY(rsvdt::action_prepare(ctx, d, &rend));
    if (!cuda_ok(ctx, cudaStreamSynchronize(ctx->stream), "sync")) return RSVDT_ERR_CUDA;
    ctx->tm.prepare += now_s() - t0;
    RSVDT_TRY(steps_with_progress(ctx, d, ctx->act_prec, rend));
    const double t1 = now_s();
    st = rsvdt::action_finish(ctx, d);
    ctx->tm.finish += now_s() - t1;
  }
  if (st == RSVDT_OK && ctx->par.Display >= 1)
    print_hms(d ? "*** Direct action elapsed time = " : "*** Adjoint action elapsed time = ", now_s() - t0, " ***\n");
  return st;
}

}  // extern "C"

namespace rsvdt {

// First half of an action: weights before, forcing slabs, y = 0 and the
// initial forcing; returns the number of RK4 steps (SourceCode/TSActionRK4.c:41-42).
// Checks and ApplyWeightMats before the stepping
// (SourceCode/ApplyWeightMats.c:17-28, 43-60); returns the number of RK4
// steps of the action (SourceCode/TSActionRK4.c:41-42).
static rsvdt_status weights_before(rsvdt_ctx *ctx, int d, int64_t *rend_out) {
  RSVDT_TRY(check_weights(ctx));
  const int64_t rows_in = d ? ctx->Nb : ctx->Nc;
  if (ctx->blk_rows != rows_in)
    return set_err(ctx, RSVDT_ERR_STATE, "%s action needs a block of %lld rows, the working block has %lld",
                   d ? "direct" : "adjoint", (long long)rows_in, (long long)ctx->blk_rows);
  if (ctx->par.Display >= 1) {
    printf("\n*** %s action begins! ***\n", d ? "Direct" : "Adjoint");
    fflush(stdout);
  }
  if (d) {
    RSVDT_TRY(weight_step(ctx, ctx->W[RSVDT_W_F_SQRT_INV], ctx->blk_rows));
    RSVDT_TRY(weight_step(ctx, ctx->W[RSVDT_B], ctx->blk_rows));
  } else {
    RSVDT_TRY(weight_step(ctx, ctx->WH[RSVDT_W_Q_SQRT], ctx->blk_rows));
    RSVDT_TRY(weight_step(ctx, ctx->WH[RSVDT_C], ctx->blk_rows));
  }
  if (ctx->blk_rows != ctx->N) return set_err(ctx, RSVDT_ERR_ARG, "forcing block has %lld rows, expected N", (long long)ctx->blk_rows);
  const bool tr = ctx->par.TransientRemoval != 0;
  ctx->Nstore = tr ? ctx->Nw + 1 : ctx->Nw;
  *rend_out = ctx->Nt + ctx->Ns + (tr ? ctx->R : 0);
  if (!cuda_ok(ctx, cudaMemsetAsync(ctx->d_flags, 0, sizeof(int32_t) * 4, ctx->stream), "memset")) return RSVDT_ERR_CUDA;
  return RSVDT_OK;
}

// ApplyWeightMats after the stepping (SourceCode/ApplyWeightMats.c:29-41,
// 61-79) and the finiteness check of the response.
static rsvdt_status weights_after(rsvdt_ctx *ctx, int d) {
  if (d) {
    RSVDT_TRY(weight_step(ctx, ctx->W[RSVDT_C], ctx->blk_rows));
    RSVDT_TRY(weight_step(ctx, ctx->W[RSVDT_W_Q_SQRT], ctx->blk_rows));
  } else {
    RSVDT_TRY(weight_step(ctx, ctx->WH[RSVDT_B], ctx->blk_rows));
    RSVDT_TRY(weight_step(ctx, ctx->WH[RSVDT_W_F_SQRT_INV], ctx->blk_rows));
  }
  RSVDT_TRY(debug_index_status(ctx));
  bool ok = true;
  RSVDT_TRY(check_finite(ctx, ctx->blk, ctx->blk_rows * ctx->Nw_eff * ctx->K, &ok));
  if (!ok) return set_err(ctx, RSVDT_ERR_DIVERGED, "NaN or Inf in the %s action's response", d ? "direct" : "adjoint");
  if (ctx->par.Display >= 1) {
    printf("*** %s action done ***\n", d ? "Direct" : "Adjoint");
    fflush(stdout);
  }
  return RSVDT_OK;
}

// First half of an action: weights before, forcing slabs, y = 0 and the
// initial forcing (TSActionRK4, SourceCode/TSActionRK4.c:38-148).
rsvdt_status action_prepare(rsvdt_ctx *ctx, int d, int64_t *rend_out) {
  RSVDT_TRY(weights_before(ctx, d, rend_out));
  RSVDT_TRY(stage_forcing(ctx, ctx->act_prec));
  return launch_forcing_init(ctx, d, ctx->act_prec);
}

// Second half: DFT or transient removal, weights after, finiteness check.
rsvdt_status action_finish(rsvdt_ctx *ctx, int d) {
  const int prec = ctx->act_prec;
  if (ctx->par.TransientRemoval) {
    RSVDT_TRY(transient_removal(ctx, d, prec, ctx->blk2));
  } else {
    RSVDT_TRY(launch_dft(ctx, prec, ctx->blk2));
  }
  std::swap(ctx->blk, ctx->blk2);
  ctx->blk_rows = ctx->N;
  ++ctx->blk_version;
  return weights_after(ctx, d);
}

// An action in capacity mode: the test vectors go through the stepping in
// chunks of Ks, each chunk's forcing staged from and its response written
// back into its own columns of the one working block.
static rsvdt_status cap_action(rsvdt_ctx *ctx, int d) {
  const int prec = ctx->act_prec;
  int64_t rend = 0;
  RSVDT_TRY(weights_before(ctx, d, &rend));
  rsvdt_status st = RSVDT_OK;
  for (int64_t k0 = 0; k0 < ctx->K && !st; k0 += ctx->Ks) {
    ctx->k0 = k0;
    st = stage_forcing(ctx, prec);
    if (!st) st = launch_forcing_init(ctx, d, prec);
    if (!st) st = steps_with_progress(ctx, d, prec, rend);
    if (!st) st = ctx->par.TransientRemoval ? transient_removal(ctx, d, prec, ctx->blk) : launch_dft(ctx, prec, ctx->blk);
  }
  ctx->k0 = 0;
  ++ctx->blk_version;
  RSVDT_TRY(st);
  ctx->blk_rows = ctx->N;
  return weights_after(ctx, d);
}

}  // namespace rsvdt

extern "C" {

rsvdt_status rsvdt_qr_all_freqs(rsvdt_ctx *ctx) {
  RSVDT_TRY(require_ready(ctx, true));
  ++ctx->blk_version;
  NvtxRange range("rsvdt qr_all_freqs");
  const double t0 = now_s();
  RSVDT_TRY(cholqr2(ctx, ctx->blk, ctx->blk_rows, ctx->Nw_eff, ctx->K, nullptr));
  if (!cuda_ok(ctx, cudaStreamSynchronize(ctx->stream), "sync")) return RSVDT_ERR_CUDA;
  ctx->tm.qr += now_s() - t0;
  return RSVDT_OK;
}

static rsvdt_status svd_all_freqs_impl(rsvdt_ctx *ctx, int32_t before_adjoint);

rsvdt_status rsvdt_svd_all_freqs(rsvdt_ctx *ctx, int32_t before_adjoint) {
  NvtxRange range(before_adjoint ? "rsvdt svd before adjoint" : "rsvdt svd");
  const double t0 = now_s();
  const rsvdt_status st = svd_all_freqs_impl(ctx, before_adjoint);
  if (ctx) ctx->tm.svd += now_s() - t0;
  return st;
}

static rsvdt_status svd_all_freqs_impl(rsvdt_ctx *ctx, int32_t before_adjoint) {
  RSVDT_TRY(require_ready(ctx, true));
  ++ctx->blk_version;
  const int64_t rows = ctx->blk_rows, n = rows * ctx->Nw_eff * ctx->K;
  if (ctx->capacity) return cap_svd(ctx, before_adjoint != 0);
  if (before_adjoint) {
    RSVDT_TRY(svd_all(ctx, ctx->blk, rows, ctx->Nw_eff, ctx->K, nullptr, ctx->S));
    // StoreU (SourceCode/StoreU.c:15).
    dfree(ctx, ctx->Ublk);
    ctx->Ublk = (z128 *)dalloc(ctx, sizeof(z128) * n);
    if (!ctx->Ublk) return set_err(ctx, RSVDT_ERR_OOM, "U allocation failed");
    if (!cuda_ok(ctx, cudaMemcpyAsync(ctx->Ublk, ctx->blk, sizeof(z128) * n, cudaMemcpyDeviceToDevice, ctx->stream),
                 "copy"))
      return RSVDT_ERR_CUDA;
    ctx->U_rows = rows;
  } else {
    if (!ctx->Ublk) return set_err(ctx, RSVDT_ERR_STATE, "U has not been stored (run the SVD before the adjoint first)");
    dfree(ctx, ctx->Vblk);
    ctx->Vblk = (z128 *)dalloc(ctx, sizeof(z128) * n);
    if (!ctx->Vblk) return set_err(ctx, RSVDT_ERR_OOM, "V allocation failed");
    RSVDT_TRY(svd_all(ctx, ctx->blk, rows, ctx->Nw_eff, ctx->K, ctx->Vblk, ctx->S));
    // Inverse weights (SourceCode/SVDAllFreqs.c:63-64).
    const int64_t C = ctx->Nw_eff * ctx->K;
    if (ctx->W[RSVDT_W_Q_SQRT_INV].present) {
      RSVDT_TRY(apply_weight(ctx, ctx->W[RSVDT_W_Q_SQRT_INV], ctx->Ublk, ctx->blk2, C));
      if (!cuda_ok(ctx, cudaMemcpyAsync(ctx->Ublk, ctx->blk2, sizeof(z128) * ctx->U_rows * C,
                                        cudaMemcpyDeviceToDevice, ctx->stream), "copy"))
        return RSVDT_ERR_CUDA;
    }
    if (ctx->W[RSVDT_W_F_SQRT_INV].present) {
      RSVDT_TRY(apply_weight(ctx, ctx->W[RSVDT_W_F_SQRT_INV], ctx->Vblk, ctx->blk2, C));
      if (!cuda_ok(ctx, cudaMemcpyAsync(ctx->Vblk, ctx->blk2, sizeof(z128) * rows * C,
                                        cudaMemcpyDeviceToDevice, ctx->stream), "copy"))
        return RSVDT_ERR_CUDA;
    }
    ctx->have_results = true;
  }
  return cuda_ok(ctx, cudaStreamSynchronize(ctx->stream), "sync") ? RSVDT_OK : RSVDT_ERR_CUDA;
}

rsvdt_status rsvdt_power_iteration(rsvdt_ctx *ctx) {
  RSVDT_TRY(require_ready(ctx, true));
  for (int64_t iq = 0; iq < ctx->par.q; ++iq) {  // SourceCode/PowerIterationRK4.c:20-29
    if (ctx->par.Display >= 1)
      printf("\n******** Inside power iteration, %d/%d *******\n", (int)iq + 1, (int)ctx->par.q);
    RSVDT_TRY(rsvdt_qr_all_freqs(ctx));
    RSVDT_TRY(rsvdt_action(ctx, RSVDT_ADJOINT));
    RSVDT_TRY(rsvdt_qr_all_freqs(ctx));
    if (ctx->ckpt_fn && ctx->ckpt_fn(ctx->ckpt_user, (int32_t)(iq + 1), ctx) != 0)
      return set_err(ctx, RSVDT_ERR_STATE, "stopped by the checkpoint callback after power sweep %d", (int)iq + 1);
    RSVDT_TRY(rsvdt_action(ctx, RSVDT_DIRECT));
  }
  return RSVDT_OK;
}

rsvdt_status rsvdt_set_checkpoint(rsvdt_ctx *ctx, rsvdt_checkpoint_fn fn, void *user) {
  if (!ctx) return RSVDT_ERR_ARG;
  ctx->ckpt_fn = fn;
  ctx->ckpt_user = fn ? user : nullptr;
  return RSVDT_OK;
}

rsvdt_status rsvdt_run(rsvdt_ctx *ctx) {
  RSVDT_TRY(require_ready(ctx, true));
  RSVDT_TRY(rsvdt_action(ctx, RSVDT_DIRECT));      // SourceCode/main.c:134
  RSVDT_TRY(rsvdt_power_iteration(ctx));           // :136
  RSVDT_TRY(rsvdt_svd_all_freqs(ctx, 1));          // :138-140
  // The refinement form's FP64 sweep: the last adjoint action, whose
  // output gives the gains, in complex128.
  if (ctx->par.precision == RSVDT_PREC_C64_REFINE) ctx->act_prec = RSVDT_PREC_C128;
  const rsvdt_status st = rsvdt_action(ctx, RSVDT_ADJOINT);  // :142
  ctx->act_prec = base_precision(ctx->par.precision);
  RSVDT_TRY(st);
  RSVDT_TRY(rsvdt_svd_all_freqs(ctx, 0));          // :144
  return RSVDT_OK;
}

rsvdt_status rsvdt_get_results(rsvdt_ctx *ctx, double *U, int64_t ldu, double *V, int64_t ldv, double *S) {
  if (!ctx) return RSVDT_ERR_ARG;
  if (!ctx->have_results) return set_err(ctx, RSVDT_ERR_STATE, "no results yet (call rsvdt_run)");
  const int64_t C = ctx->Nw_eff * ctx->K;
  if (ctx->capacity) {
    if ((U && ldu < ctx->U_rows) || (V && ldv < ctx->Nb)) return set_err(ctx, RSVDT_ERR_ARG, "leading dimension too small");
    if (U) host_u_cols(ctx, nullptr, C, U, ldu);
    if (V) RSVDT_TRY(block_cols_to_host(ctx, ctx->blk, ctx->Nb, C, nullptr, C, V, ldv));
    if (S && !cuda_ok(ctx, cudaMemcpy(S, ctx->S, sizeof(double) * C, cudaMemcpyDeviceToHost), "download"))
      return RSVDT_ERR_CUDA;
    return RSVDT_OK;
  }
  auto fetch = [&](const z128 *src, int64_t rows, double *dst, int64_t ld) -> rsvdt_status {
    if (!dst) return RSVDT_OK;
    if (ld < rows) return set_err(ctx, RSVDT_ERR_ARG, "leading dimension too small");
    z128 *stage = (z128 *)dalloc(ctx, sizeof(z128) * ld * C);
    if (!stage) return set_err(ctx, RSVDT_ERR_OOM, "staging allocation failed");
    rsvdt_status st = launch_blk_to_colmajor(ctx, src, rows, C, stage, ld);
    if (!st && !cuda_ok(ctx, cudaMemcpyAsync(dst, stage, sizeof(z128) * ld * C, cudaMemcpyDeviceToHost, ctx->stream),
                        "download"))
      st = RSVDT_ERR_CUDA;
    if (!st && !cuda_ok(ctx, cudaStreamSynchronize(ctx->stream), "sync")) st = RSVDT_ERR_CUDA;
    dfree(ctx, stage);
    return st;
  };
  RSVDT_TRY(fetch(ctx->Ublk, ctx->U_rows, U, ldu));
  RSVDT_TRY(fetch(ctx->Vblk, ctx->Nb, V, ldv));
  if (S && !cuda_ok(ctx, cudaMemcpy(S, ctx->S, sizeof(double) * C, cudaMemcpyDeviceToHost), "download"))
    return RSVDT_ERR_CUDA;
  return RSVDT_OK;
}

rsvdt_status rsvdt_rk4_reset(rsvdt_ctx *ctx, rsvdt_dir dir) {
  RSVDT_TRY(require_ready(ctx, true));
  if (ctx->blk_rows != ctx->N) return set_err(ctx, RSVDT_ERR_STATE, "working block must have N rows");
  const int prec = ctx->act_prec;
  ctx->Nstore = ctx->par.TransientRemoval ? ctx->Nw + 1 : ctx->Nw;
  RSVDT_TRY(stage_forcing_cached(ctx, prec));
  RSVDT_TRY(launch_forcing_init(ctx, dir == RSVDT_DIRECT ? 1 : 0, prec));
  return RSVDT_OK;
}

rsvdt_status rsvdt_rk4_advance(rsvdt_ctx *ctx, rsvdt_dir dir, int64_t i0, int64_t nsteps) {
  RSVDT_TRY(require_ready(ctx, true));
  if (i0 < 1 || nsteps < 0) return set_err(ctx, RSVDT_ERR_ARG, "invalid step range");
  return run_steps(ctx, dir == RSVDT_DIRECT ? 1 : 0, ctx->act_prec, i0, nsteps, true);
}

rsvdt_status rsvdt_rk4_profile_ex(rsvdt_ctx *ctx, rsvdt_dir dir, int64_t i0, int64_t nsteps, double *times_ms) {
  RSVDT_TRY(require_ready(ctx, true));
  if (i0 < 1 || nsteps < 1 || !times_ms) return set_err(ctx, RSVDT_ERR_ARG, "invalid profile arguments");
  return profile_steps(ctx, dir == RSVDT_DIRECT ? 1 : 0, ctx->act_prec, i0, nsteps, times_ms);
}

rsvdt_status rsvdt_rk4_profile(rsvdt_ctx *ctx, rsvdt_dir dir, int64_t i0, int64_t nsteps, double *stage_ms) {
  if (!stage_ms) return set_err(ctx, RSVDT_ERR_ARG, "invalid profile arguments");
  double t[5] = {0, 0, 0, 0, 0};
  RSVDT_TRY(rsvdt_rk4_profile_ex(ctx, dir, i0, nsteps, t));
  stage_ms[0] = t[0] + t[4];  // the forcing block replaces stage 1's synthesis
  for (int s = 1; s < 4; ++s) stage_ms[s] = t[s];
  return RSVDT_OK;
}

rsvdt_status rsvdt_set_forcing_block(rsvdt_ctx *ctx, int32_t steps) {
  if (!ctx) return RSVDT_ERR_ARG;
  if (steps != -1 && steps != 0 && steps != 1 && steps != 2 && steps != 4 && steps != 8 && steps != 16)
    return set_err(ctx, RSVDT_ERR_ARG, "forcing block of %d steps (allowed: -1, 0, 1, 2, 4, 8, 16)", (int)steps);
  ctx->fb_steps = steps;
  return RSVDT_OK;
}

int32_t rsvdt_get_forcing_block(const rsvdt_ctx *ctx) {
  if (!ctx) return 0;
  return ctx->fb_last;
}

rsvdt_status rsvdt_rk4_steps(rsvdt_ctx *ctx, rsvdt_dir dir, int64_t i0, int64_t nsteps, double *y, double *F3) {
  RSVDT_TRY(require_ready(ctx, true));
  if (!y || !F3) return set_err(ctx, RSVDT_ERR_ARG, "null state");
  if (ctx->capacity) return set_err(ctx, RSVDT_ERR_STATE, "rsvdt_rk4_steps is not available in capacity mode");
  if (ctx->blk_rows != ctx->N) return set_err(ctx, RSVDT_ERR_STATE, "working block must have N rows");
  const int prec = ctx->act_prec;
  const int64_t N = ctx->N, K = ctx->K;
  ctx->Nstore = ctx->par.TransientRemoval ? ctx->Nw + 1 : ctx->Nw;
  RSVDT_TRY(stage_forcing_cached(ctx, prec));
  // One persistent staging buffer for both host arrays (no allocation, and
  // so no device-wide synchronisation of cudaFree, per call).
  const size_t need = sizeof(z128) * (size_t)N * K * 2;
  if (ctx->io_bytes < need) {
    dfree(ctx, ctx->io_stage);
    ctx->io_stage = (z128 *)dalloc(ctx, need);
    ctx->io_bytes = ctx->io_stage ? need : 0;
    if (!ctx->io_stage) return set_err(ctx, RSVDT_ERR_OOM, "staging allocation failed");
  }
  z128 *sy = ctx->io_stage, *sf = ctx->io_stage + N * K;
  const size_t bytes = sizeof(z128) * (size_t)N * K;
  const int d = dir == RSVDT_DIRECT ? 1 : 0;
  int C = 0, cth = 0;
  if (prec == RSVDT_PREC_C64) {
    // Precision form: the complex128 host state is rounded to complex64 on
    // the way in and widened on the way out.
    if (!cuda_ok(ctx, cudaMemcpyAsync(sy, y, bytes, cudaMemcpyHostToDevice, ctx->stream), "upload") ||
        !cuda_ok(ctx, cudaMemcpyAsync(sf, F3, bytes, cudaMemcpyHostToDevice, ctx->stream), "upload"))
      return RSVDT_ERR_CUDA;
    RSVDT_TRY(launch_colmajor_to_blk64(ctx, sy, N, N, K, (z64 *)ctx->y));
    RSVDT_TRY(launch_colmajor_to_blk64(ctx, sf, N, N, K, (z64 *)ctx->F3));
    RSVDT_TRY(run_steps(ctx, d, prec, i0, nsteps, true));
    RSVDT_TRY(launch_blk64_to_colmajor(ctx, (const z64 *)ctx->y, N, K, sy, N));
    RSVDT_TRY(launch_blk64_to_colmajor(ctx, (const z64 *)ctx->F3, N, K, sf, N));
    if (!cuda_ok(ctx, cudaMemcpyAsync(y, sy, bytes, cudaMemcpyDeviceToHost, ctx->stream), "download") ||
        !cuda_ok(ctx, cudaMemcpyAsync(F3, sf, bytes, cudaMemcpyDeviceToHost, ctx->stream), "download"))
      return RSVDT_ERR_CUDA;
  } else if (nsteps >= 1 && step_lanes(ctx) == 1 && !use_cluster_engine(ctx, prec, &C, &cth)) {
    if (!ctx->io_stream &&
        (!cuda_ok(ctx, cudaStreamCreateWithFlags(&ctx->io_stream, cudaStreamNonBlocking), "stream create") ||
         !cuda_ok(ctx, cudaEventCreateWithFlags(&ctx->io_event, cudaEventDisableTiming), "event create") ||
         !cuda_ok(ctx, cudaEventCreateWithFlags(&ctx->up_event, cudaEventDisableTiming), "event create")))
      return RSVDT_ERR_CUDA;
    // y is downloaded in row slabs, each as soon as its rows of the last
    // stage 4 are final, while the next slab computes.
    const int nslab = stage4_slab_count(ctx, d, prec, rsvdt_ctx::kIoSlabs);
    for (int k = 0; k < nslab; ++k)
      if (!ctx->slab_event[k] &&
          !cuda_ok(ctx, cudaEventCreateWithFlags(&ctx->slab_event[k], cudaEventDisableTiming), "event create"))
        return RSVDT_ERR_CUDA;
    // The first step's forcing needs no state: it is synthesised on the
    // context's stream while y and F3 upload on the second stream.
    RSVDT_TRY(launch_forcing_ahead(ctx, d, prec, i0));
    if (!cuda_ok(ctx, cudaMemcpyAsync(sy, y, bytes, cudaMemcpyHostToDevice, ctx->io_stream), "upload") ||
        !cuda_ok(ctx, cudaMemcpyAsync(sf, F3, bytes, cudaMemcpyHostToDevice, ctx->io_stream), "upload") ||
        !cuda_ok(ctx, cudaEventRecord(ctx->up_event, ctx->io_stream), "event") ||
        !cuda_ok(ctx, cudaStreamWaitEvent(ctx->stream, ctx->up_event, 0), "wait"))
      return RSVDT_ERR_CUDA;
    RSVDT_TRY(launch_colmajor_to_blk(ctx, sy, N, N, K, (z128 *)ctx->y));
    RSVDT_TRY(launch_colmajor_to_blk(ctx, sf, N, N, K, (z128 *)ctx->F3));
    // F3 is final after the last step's stage 1: its transpose and download
    // run on the second stream while stages 2-4 run.
    if (nsteps == 1) {
      RSVDT_TRY(launch_first_step_rest(ctx, d, prec, i0, ctx->io_event, nslab, ctx->slab_event));
    } else {
      RSVDT_TRY(launch_first_step_rest(ctx, d, prec, i0, nullptr));
      RSVDT_TRY(run_steps(ctx, d, prec, i0 + 1, nsteps - 2, true));
      RSVDT_TRY(run_last_step_split(ctx, d, prec, i0 + nsteps - 1, ctx->io_event, nslab, ctx->slab_event));
    }
    if (!cuda_ok(ctx, cudaStreamWaitEvent(ctx->io_stream, ctx->io_event, 0), "wait")) return RSVDT_ERR_CUDA;
    RSVDT_TRY(launch_blk_to_colmajor(ctx, (const z128 *)ctx->F3, N, K, sf, N, ctx->io_stream));
    if (!cuda_ok(ctx, cudaMemcpyAsync(F3, sf, bytes, cudaMemcpyDeviceToHost, ctx->io_stream), "download"))
      return RSVDT_ERR_CUDA;
    for (int k = 0; k < nslab; ++k) {
      const int64_t r0 = N * k / nslab, r1 = N * (k + 1) / nslab;
      if (!cuda_ok(ctx, cudaStreamWaitEvent(ctx->io_stream, ctx->slab_event[k], 0), "wait")) return RSVDT_ERR_CUDA;
      RSVDT_TRY(launch_blk_to_colmajor(ctx, (const z128 *)ctx->y + r0 * K, r1 - r0, K, sy + r0, N, ctx->io_stream));
      if (!cuda_ok(ctx,
                   cudaMemcpy2DAsync((z128 *)y + r0, sizeof(z128) * N, sy + r0, sizeof(z128) * N,
                                     sizeof(z128) * (r1 - r0), K, cudaMemcpyDeviceToHost, ctx->io_stream),
                   "download"))
        return RSVDT_ERR_CUDA;
    }
    if (!cuda_ok(ctx, cudaStreamSynchronize(ctx->io_stream), "sync")) return RSVDT_ERR_CUDA;
  } else {
    // Host (N x K column-major) -> device [n][k], both arrays in flight.
    if (!cuda_ok(ctx, cudaMemcpyAsync(sy, y, bytes, cudaMemcpyHostToDevice, ctx->stream), "upload") ||
        !cuda_ok(ctx, cudaMemcpyAsync(sf, F3, bytes, cudaMemcpyHostToDevice, ctx->stream), "upload"))
      return RSVDT_ERR_CUDA;
    RSVDT_TRY(launch_colmajor_to_blk(ctx, sy, N, N, K, (z128 *)ctx->y));
    RSVDT_TRY(launch_colmajor_to_blk(ctx, sf, N, N, K, (z128 *)ctx->F3));
    RSVDT_TRY(run_steps(ctx, d, prec, i0, nsteps, true));
    RSVDT_TRY(launch_blk_to_colmajor(ctx, (const z128 *)ctx->y, N, K, sy, N));
    RSVDT_TRY(launch_blk_to_colmajor(ctx, (const z128 *)ctx->F3, N, K, sf, N));
    if (!cuda_ok(ctx, cudaMemcpyAsync(y, sy, bytes, cudaMemcpyDeviceToHost, ctx->stream), "download") ||
        !cuda_ok(ctx, cudaMemcpyAsync(F3, sf, bytes, cudaMemcpyDeviceToHost, ctx->stream), "download"))
      return RSVDT_ERR_CUDA;
  }
  return cuda_ok(ctx, cudaStreamSynchronize(ctx->stream), "sync") ? RSVDT_OK : RSVDT_ERR_CUDA;
}

rsvdt_status rsvdt_synchronize(rsvdt_ctx *ctx) {
  if (!ctx) return RSVDT_ERR_ARG;
  if (!cuda_ok(ctx, cudaStreamSynchronize(ctx->stream), "sync")) return RSVDT_ERR_CUDA;
  return debug_index_status(ctx);
}

int32_t rsvdt_debug_build(void) {
#ifdef RSVDT_DEBUG
  return 1;
#else
  return 0;
#endif
}

void *rsvdt_stream(rsvdt_ctx *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

int64_t rsvdt_launch_count(const rsvdt_ctx *ctx) { return ctx ? ctx->launches : 0; }

rsvdt_status rsvdt_set_capacity_mode(rsvdt_ctx *ctx, int64_t kc, int32_t u_c64) {
  if (!ctx) return RSVDT_ERR_ARG;
  if (kc < 0) return set_err(ctx, RSVDT_ERR_ARG, "chunk size must be non-negative");
  if (ctx->have_block) return set_err(ctx, RSVDT_ERR_STATE, "set the capacity mode before the sketch");
  ctx->capacity = true;
  ctx->cap_kc = kc;
  ctx->cap_u_c64 = u_c64 ? 1 : 0;
  ctx->u_host.clear();
  if (ctx->have_operator) {
    update_dims(ctx);
    RSVDT_TRY(ensure_buffers(ctx, ctx->K > 0 ? ctx->K : ctx->par.k));
  }
  return RSVDT_OK;
}

rsvdt_status rsvdt_get_timings(const rsvdt_ctx *ctx, char *json, int64_t len) {
  if (!ctx || !json || len < 1) return RSVDT_ERR_ARG;
  const auto &t = ctx->tm;
  const double ms = t.steps ? 1e3 * t.stepping / (double)t.steps : 0.0;
  const int n = snprintf(json, (size_t)len,
                         "{\"actions\": {\"direct\": %lld, \"adjoint\": %lld}, \"steps\": %lld, "
                         "\"seconds\": {\"prepare\": %.6f, \"stepping\": %.6f, \"finish\": %.6f, \"qr\": %.6f, "
                         "\"svd\": %.6f}, \"ms_per_step\": %.6f, \"lanes_per_row\": %d, \"capacity_chunk\": %lld}",
                         (long long)t.actions[1], (long long)t.actions[0], (long long)t.steps, t.prepare, t.stepping,
                         t.finish, t.qr, t.svd, ms, step_lanes(ctx), (long long)(ctx->capacity ? ctx->Ks : 0));
  return n < len ? RSVDT_OK : RSVDT_ERR_ARG;
}

rsvdt_status rsvdt_reset_timings(rsvdt_ctx *ctx) {
  if (!ctx) return RSVDT_ERR_ARG;
  ctx->tm = rsvdt_ctx::PhaseTimes();
  return RSVDT_OK;
}

rsvdt_status rsvdt_set_lanes_per_row(rsvdt_ctx *ctx, int32_t lanes) {
  if (!ctx) return RSVDT_ERR_ARG;
  if (lanes != 0 && lanes != 1 && lanes != 2 && lanes != 4 && lanes != 8)
    return set_err(ctx, RSVDT_ERR_ARG, "lanes per row must be 0 (automatic), 1, 2, 4 or 8, not %d", (int)lanes);
  ctx->lanes_override = lanes;
  return RSVDT_OK;
}

int32_t rsvdt_get_lanes_per_row(const rsvdt_ctx *ctx) { return ctx ? step_lanes(ctx) : 0; }

rsvdt_status rsvdt_set_step_engine(rsvdt_ctx *ctx, int32_t engine) {
  if (!ctx) return RSVDT_ERR_ARG;
  if (engine != RSVDT_ENGINE_AUTO && engine != RSVDT_ENGINE_STAGES && engine != RSVDT_ENGINE_CLUSTER)
    return set_err(ctx, RSVDT_ERR_ARG, "step engine must be 0 (automatic), 1 (stages) or 2 (cluster), not %d",
                   (int)engine);
  ctx->engine = engine;
  return RSVDT_OK;
}

int32_t rsvdt_get_step_engine(const rsvdt_ctx *ctx) {
  if (!ctx) return 0;
  int C = 0, threads = 0;
  return use_cluster_engine(ctx, ctx->act_prec, &C, &threads) ? RSVDT_ENGINE_CLUSTER : RSVDT_ENGINE_STAGES;
}

rsvdt_status rsvdt_device_memory(int64_t *free_bytes, int64_t *total_bytes) {
  size_t fr = 0, tot = 0;
  if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
    cudaGetLastError();
    return RSVDT_ERR_CUDA;
  }
  if (free_bytes) *free_bytes = (int64_t)fr;
  if (total_bytes) *total_bytes = (int64_t)tot;
  return RSVDT_OK;
}

rsvdt_status rsvdt_get_capacity(const rsvdt_ctx *ctx, int64_t *kc) {
  if (!ctx || !kc) return RSVDT_ERR_ARG;
  *kc = ctx->capacity ? ctx->Ks : 0;
  return RSVDT_OK;
}

rsvdt_status rsvdt_get_result_cols(rsvdt_ctx *ctx, const int64_t *cols, int64_t ncols, double *U, int64_t ldu,
                                   double *V, int64_t ldv) {
  if (!ctx) return RSVDT_ERR_ARG;
  if (!ctx->have_results) return set_err(ctx, RSVDT_ERR_STATE, "no results yet (call rsvdt_run)");
  const int64_t C = ctx->Nw_eff * ctx->K;
  if (ncols < 0 || (ncols > 0 && !cols)) return set_err(ctx, RSVDT_ERR_ARG, "invalid column list");
  for (int64_t j = 0; j < ncols; ++j)
    if (cols[j] < 0 || cols[j] >= C)
      return set_err(ctx, RSVDT_ERR_ARG, "column %lld out of range [0, %lld)", (long long)cols[j], (long long)C);
  if ((U && ldu < ctx->U_rows) || (V && ldv < ctx->Nb)) return set_err(ctx, RSVDT_ERR_ARG, "leading dimension too small");
  if (U) {
    if (ctx->capacity)
      host_u_cols(ctx, cols, ncols, U, ldu);
    else
      RSVDT_TRY(block_cols_to_host(ctx, ctx->Ublk, ctx->U_rows, C, cols, ncols, U, ldu));
  }
  if (V) RSVDT_TRY(block_cols_to_host(ctx, ctx->capacity ? ctx->blk : ctx->Vblk, ctx->Nb, C, cols, ncols, V, ldv));
  return RSVDT_OK;
}

}  // extern "C"
