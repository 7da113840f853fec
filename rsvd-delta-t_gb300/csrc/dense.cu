// Dense per-frequency stages and layout kernels.
//
// Spectral blocks live on the device as [row][iw][k] (complex128): row n
// holds every frequency's k values contiguously, so the forcing synthesis,
// the DFT, the Gram products of all frequencies and the weight products
// each read a row once, coalesced.
//
//  - QRAllFreqs (SourceCode/QRAllFreqs.c:22-32) becomes batched CholQR over
//    all frequencies (one shifted pass, then plain passes): FP64 Gram
//    G_iw = Y_iw^H Y_iw by row chunks (the k(k+1)/2 upper pairs only), a
//    deterministic chunk reduction, a per-frequency Cholesky G = R^H R, then
//    Y_iw <- Y_iw R^{-1}. R keeps a real positive diagonal, which is the
//    normalisation of SLEPc's Gram-Schmidt, so Q matches column for column.
//  - SVDAllFreqs (SourceCode/SVDAllFreqs.c:34-56) becomes the same CholQR
//    (Y = QR) followed by a one-sided Jacobi SVD of each k x k R
//    (R = U_R S W^H) and U = Q U_R.
//  All of it is FP64-bound on GB300 (k x k work per row and frequency).
#include <algorithm>
#include <cmath>
#include <cstdarg>

#include "common.cuh"

namespace rsvdt {

// ------------------------------------------------------------ transposes

// dst[r][c] = src[c*ld + r]  (column-major host layout -> [row][col]).
__global__ void k_col_to_row(const z128 *__restrict__ src, int64_t rows, int64_t ld, int64_t C,
                             z128 *__restrict__ dst) {
  __shared__ z128 tile[32][33];
  const int64_t r0 = blockIdx.x * 32, c0 = blockIdx.y * 32;
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    int64_t c = c0 + j, r = r0 + threadIdx.x;
    if (c < C && r < rows) tile[j][threadIdx.x] = src[c * ld + r];
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    int64_t r = r0 + j, c = c0 + threadIdx.x;
    if (c < C && r < rows) dst[r * C + c] = tile[threadIdx.x][j];
  }
}

// dst[c*ld + r] = src[r][c]
__global__ void k_row_to_col(const z128 *__restrict__ src, int64_t rows, int64_t C,
                             z128 *__restrict__ dst, int64_t ld) {
  __shared__ z128 tile[32][33];
  const int64_t r0 = blockIdx.x * 32, c0 = blockIdx.y * 32;
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    int64_t r = r0 + j, c = c0 + threadIdx.x;
    if (c < C && r < rows) tile[j][threadIdx.x] = src[r * C + c];
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    int64_t c = c0 + j, r = r0 + threadIdx.x;
    if (c < C && r < rows) dst[c * ld + r] = tile[threadIdx.x][j];
  }
}

// Complex64 variants: dst[r][c] = (complex64) src[c*ld + r], and
// dst[c*ld + r] = (complex128) src[r][c].
__global__ void k_col_to_row_c64(const z128 *__restrict__ src, int64_t rows, int64_t ld, int64_t C,
                                 z64 *__restrict__ dst) {
  __shared__ z128 tile[32][33];
  const int64_t r0 = blockIdx.x * 32, c0 = blockIdx.y * 32;
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    int64_t c = c0 + j, r = r0 + threadIdx.x;
    if (c < C && r < rows) tile[j][threadIdx.x] = src[c * ld + r];
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    int64_t r = r0 + j, c = c0 + threadIdx.x;
    if (c < C && r < rows) {
      const z128 v = tile[threadIdx.x][j];
      dst[r * C + c] = zmake<z64>((float)v.re, (float)v.im);
    }
  }
}

__global__ void k_row_to_col_c64(const z64 *__restrict__ src, int64_t rows, int64_t C,
                                 z128 *__restrict__ dst, int64_t ld) {
  __shared__ z64 tile[32][33];
  const int64_t r0 = blockIdx.x * 32, c0 = blockIdx.y * 32;
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    int64_t r = r0 + j, c = c0 + threadIdx.x;
    if (c < C && r < rows) tile[j][threadIdx.x] = src[r * C + c];
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    int64_t c = c0 + j, r = r0 + threadIdx.x;
    if (c < C && r < rows) {
      const z64 v = tile[threadIdx.x][j];
      dst[c * ld + r] = zmake<z128>((double)v.re, (double)v.im);
    }
  }
}

static dim3 tgrid(int64_t rows, int64_t C) {
  return dim3((unsigned)((rows + 31) / 32), (unsigned)((C + 31) / 32));
}

rsvdt_status launch_colmajor_to_blk(rsvdt_ctx *ctx, const z128 *src, int64_t rows, int64_t ld,
                                    int64_t C, z128 *dst) {
  if ((C + 31) / 32 > 65535) return set_err(ctx, RSVDT_ERR_ARG, "too many columns (%lld)", (long long)C);
  k_col_to_row<<<tgrid(rows, C), dim3(32, 8), 0, ctx->stream>>>(src, rows, ld, C, dst);
  ctx->launches += 1;
  return cuda_ok(ctx, cudaGetLastError(), "transpose") ? RSVDT_OK : RSVDT_ERR_CUDA;
}

rsvdt_status launch_blk_to_colmajor(rsvdt_ctx *ctx, const z128 *src, int64_t rows, int64_t C,
                                    z128 *dst, int64_t ld, cudaStream_t st) {
  if ((C + 31) / 32 > 65535) return set_err(ctx, RSVDT_ERR_ARG, "too many columns (%lld)", (long long)C);
  k_row_to_col<<<tgrid(rows, C), dim3(32, 8), 0, st ? st : ctx->stream>>>(src, rows, C, dst, ld);
  ctx->launches += 1;
  return cuda_ok(ctx, cudaGetLastError(), "transpose") ? RSVDT_OK : RSVDT_ERR_CUDA;
}

rsvdt_status launch_colmajor_to_blk64(rsvdt_ctx *ctx, const z128 *src, int64_t rows, int64_t ld,
                                      int64_t C, z64 *dst) {
  if ((C + 31) / 32 > 65535) return set_err(ctx, RSVDT_ERR_ARG, "too many columns (%lld)", (long long)C);
  k_col_to_row_c64<<<tgrid(rows, C), dim3(32, 8), 0, ctx->stream>>>(src, rows, ld, C, dst);
  ctx->launches += 1;
  return cuda_ok(ctx, cudaGetLastError(), "transpose") ? RSVDT_OK : RSVDT_ERR_CUDA;
}

rsvdt_status launch_blk64_to_colmajor(rsvdt_ctx *ctx, const z64 *src, int64_t rows, int64_t C,
                                      z128 *dst, int64_t ld) {
  if ((C + 31) / 32 > 65535) return set_err(ctx, RSVDT_ERR_ARG, "too many columns (%lld)", (long long)C);
  k_row_to_col_c64<<<tgrid(rows, C), dim3(32, 8), 0, ctx->stream>>>(src, rows, C, dst, ld);
  ctx->launches += 1;
  return cuda_ok(ctx, cudaGetLastError(), "transpose") ? RSVDT_OK : RSVDT_ERR_CUDA;
}

// ------------------------------------------------------ weight products

// out[r][c] = sum_j M[r,j] * in[j][c], c < C (MatMatMult,
// SourceCode/ApplyWeightMats.c:18-76, with out != in).
__global__ void __launch_bounds__(256) k_csr_block(const int32_t *__restrict__ rowptr,
                                                   const int32_t *__restrict__ col,
                                                   const z128 *__restrict__ val, int64_t rows,
                                                   int64_t C, const z128 *__restrict__ in,
                                                   z128 *__restrict__ out) {
  const int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (u >= rows * C) return;
  const int64_t r = u / C, c = u - r * C;
  z128 s = zmake<z128>(0, 0);
  for (int32_t j = rowptr[r]; j < rowptr[r + 1]; ++j) zmac(s, val[j], in[(int64_t)col[j] * C + c]);
  out[u] = s;
}

rsvdt_status apply_weight(rsvdt_ctx *ctx, const DevCSR &M, const z128 *in, z128 *out, int64_t C) {
  const int th = 256;
  k_csr_block<<<grid_for(M.rows * C, th), th, 0, ctx->stream>>>(M.rowptr, M.col, M.val, M.rows,
                                                                C, in, out);
  ctx->launches += 1;
  return cuda_ok(ctx, cudaGetLastError(), "weight product") ? RSVDT_OK : RSVDT_ERR_CUDA;
}

// ------------------------------------------------------------- CholQR2

static const int kGramRows = 2048;  // rows per Gram chunk

// part[chunk][iw][a][b] = sum_{n in chunk} conj(X[n][iw][a]) * Y[n][iw][b].
// X and Y have row strides sx, sy (complex values) and KA / KB columns per
// frequency block; grid = (chunks, nw, pair groups of 1024).
static const int kGramTile = 16;  // rows staged in shared memory at a time

__global__ void __launch_bounds__(256) k_gram_part(const z128 *__restrict__ X, int64_t sx,
                                                   const z128 *__restrict__ Y, int64_t sy,
                                                   int64_t rows, int KA, int KB,
                                                   z128 *__restrict__ part) {
  extern __shared__ z128 sm[];  // [kGramTile][KA] and [kGramTile][KB]
  const int iw = blockIdx.y, nw = gridDim.y;
  const int64_t n0 = (int64_t)blockIdx.x * kGramRows;
  const int64_t n1 = min(rows, n0 + kGramRows);
  z128 *sx_ = sm, *sy_ = sm + kGramTile * KA;
  const int pairs = KA * KB;
  const int pbase = blockIdx.z * 1024;
  // Each thread owns up to 4 (a,b) pairs of this block's group.
  z128 acc[4];
  for (int q = 0; q < 4; ++q) acc[q] = zmake<z128>(0, 0);
  for (int64_t nb = n0; nb < n1; nb += kGramTile) {
    const int nr = (int)min((int64_t)kGramTile, n1 - nb);
    __syncthreads();
    for (int e = threadIdx.x; e < nr * KA; e += blockDim.x) {
      int rr = e / KA, a = e - rr * KA;
      sx_[rr * KA + a] = X[(nb + rr) * sx + (int64_t)iw * KA + a];
    }
    for (int e = threadIdx.x; e < nr * KB; e += blockDim.x) {
      int rr = e / KB, b = e - rr * KB;
      sy_[rr * KB + b] = Y[(nb + rr) * sy + (int64_t)iw * KB + b];
    }
    __syncthreads();
    for (int q = 0; q < 4; ++q) {
      const int p = pbase + threadIdx.x + q * blockDim.x;
      if (p >= pairs) break;
      const int a = p / KB, b = p - a * KB;
      z128 s = acc[q];
      for (int rr = 0; rr < nr; ++rr) zmacc(s, sx_[rr * KA + a], sy_[rr * KB + b]);
      acc[q] = s;
    }
  }
  for (int q = 0; q < 4; ++q) {
    const int p = pbase + threadIdx.x + q * blockDim.x;
    if (p >= pairs) break;
    part[((int64_t)blockIdx.x * nw + iw) * pairs + p] = acc[q];
  }
}

// Gram partials of X with itself: only the K(K+1)/2 pairs a <= b are
// computed (the lower triangle is written as their conjugates; the
// Cholesky reads the upper one). With few pairs the block's threads split
// into row groups (rows g, g + groups, ... of each staged tile) whose sums
// are added in group order at the end, so that all threads have work.
__global__ void __launch_bounds__(256) k_gram_sym(const z128 *__restrict__ X, int64_t sx, int64_t rows, int K,
                                                  z128 *__restrict__ part) {
  extern __shared__ z128 sm[];  // [kGramTile][K] rows, then [256] group sums
  const int iw = blockIdx.y, nw = gridDim.y;
  const int64_t n0 = (int64_t)blockIdx.x * kGramRows;
  const int64_t n1 = min(rows, n0 + kGramRows);
  const int P = K * (K + 1) / 2;
  const int groups = P <= (int)blockDim.x ? (int)blockDim.x / P : 1;
  z128 *tile = sm, *red = sm + kGramTile * K;
  int g = 0, p;
  if (groups > 1) {
    g = threadIdx.x / P;
    p = threadIdx.x - g * P;
  } else {
    p = blockIdx.z * blockDim.x + threadIdx.x;
  }
  const bool act = groups > 1 ? g < groups : p < P;
  int a = 0, b = 0;
  if (act) {
    int rem = p;
    while (rem >= K - a) {
      rem -= K - a;
      ++a;
    }
    b = a + rem;
  }
  z128 s = zmake<z128>(0, 0);
  for (int64_t nb = n0; nb < n1; nb += kGramTile) {
    const int nr = (int)min((int64_t)kGramTile, n1 - nb);
    __syncthreads();
    for (int e = threadIdx.x; e < nr * K; e += blockDim.x) {
      const int rr = e / K, c = e - rr * K;
      tile[rr * K + c] = X[(nb + rr) * sx + (int64_t)iw * K + c];
    }
    __syncthreads();
    if (act)
      for (int rr = g; rr < nr; rr += groups) zmacc(s, tile[rr * K + a], tile[rr * K + b]);
  }
  z128 *out = part + ((int64_t)blockIdx.x * nw + iw) * K * K;
  if (groups > 1) {
    if (act) red[threadIdx.x] = s;
    __syncthreads();
    if (!act || g != 0) return;
    for (int q = 1; q < groups; ++q) {
      const z128 v = red[q * P + p];
      s.re += v.re;
      s.im += v.im;
    }
  } else if (!act) {
    return;
  }
  out[a * K + b] = s;
  if (b != a) out[b * K + a] = zmake<z128>(s.re, -s.im);
}

// G[iw][p] = sum over chunks (fixed order).
__global__ void k_gram_reduce(const z128 *__restrict__ part, int chunks, int nw, int pairs,
                              z128 *__restrict__ G) {
  const int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (u >= (int64_t)nw * pairs) return;
  z128 s = zmake<z128>(0, 0);
  for (int c = 0; c < chunks; ++c) {
    const z128 v = part[(int64_t)c * nw * pairs + u];
    s.re += v.re;
    s.im += v.im;
  }
  G[u] = s;
}

// Per frequency: G = R^H R (upper R, real positive diagonal), Rinv = R^{-1}.
// With shift > 0 the factorised matrix is G + shift*trace(G)*I (shifted
// CholQR for ill-conditioned blocks). Racc (optional) <- R * Racc.
__global__ void k_chol(const z128 *__restrict__ G, int nw, int K, double shift,
                       z128 *__restrict__ Rm, z128 *__restrict__ Rinv, z128 *Racc,
                       int32_t *flags) {
  const int iw = blockIdx.x * blockDim.x + threadIdx.x;
  if (iw >= nw) return;
  const z128 *g = G + (int64_t)iw * K * K;
  z128 *r = Rm + (int64_t)iw * K * K;
  z128 *ri = Rinv + (int64_t)iw * K * K;
  double sh = 0;
  if (shift > 0) {
    double tr = 0;
    for (int a = 0; a < K; ++a) tr += g[a * K + a].re;
    sh = shift * tr;
  }
  for (int e = 0; e < K * K; ++e) r[e] = zmake<z128>(0, 0);
  bool ok = true;
  for (int a = 0; a < K; ++a) {
    double d = g[a * K + a].re + sh;
    for (int m = 0; m < a; ++m) d -= r[m * K + a].re * r[m * K + a].re + r[m * K + a].im * r[m * K + a].im;
    if (!(d > 0) || !isfinite(d)) {
      ok = false;
      d = 1;
    }
    const double raa = sqrt(d);
    r[a * K + a] = zmake<z128>(raa, 0);
    for (int b = a + 1; b < K; ++b) {
      z128 s = g[a * K + b];
      for (int m = 0; m < a; ++m) {
        // s -= conj(R[m][a]) * R[m][b]
        const z128 x = r[m * K + a], y = r[m * K + b];
        s.re -= x.re * y.re + x.im * y.im;
        s.im -= x.re * y.im - x.im * y.re;
      }
      r[a * K + b] = zmake<z128>(s.re / raa, s.im / raa);
    }
  }
  if (!ok) atomicOr(flags, 2);
  // Rinv: upper triangular inverse by back substitution, column by column.
  for (int e = 0; e < K * K; ++e) ri[e] = zmake<z128>(0, 0);
  for (int b = 0; b < K; ++b) {
    ri[b * K + b] = zmake<z128>(1.0 / r[b * K + b].re, 0);
    for (int a = b - 1; a >= 0; --a) {
      z128 s = zmake<z128>(0, 0);
      for (int m = a + 1; m <= b; ++m) zmac(s, r[a * K + m], ri[m * K + b]);
      const double raa = r[a * K + a].re;
      ri[a * K + b] = zmake<z128>(-s.re / raa, -s.im / raa);
    }
  }
  if (Racc) {
    // Racc <- R * Racc (both upper triangular).
    z128 *ra = Racc + (int64_t)iw * K * K;
    for (int b = K - 1; b >= 0; --b)
      for (int a = 0; a <= b; ++a) {
        z128 s = zmake<z128>(0, 0);
        for (int m = a; m <= b; ++m) zmac(s, r[a * K + m], ra[m * K + b]);
        ra[a * K + b] = s;  // entries (m > a) of column b are not yet overwritten
      }
  }
}

// Y[n][iw][:] <- Y[n][iw][:] * M[iw] (K x K), in place; one row-frequency
// pair per K threads.
__global__ void __launch_bounds__(256) k_apply_small(z128 *__restrict__ Y, int64_t stride,
                                                     int64_t rows, int nw, int K,
                                                     const z128 *__restrict__ M, int upper) {
  extern __shared__ z128 sm[];
  const int per = blockDim.x / K;
  const int local = threadIdx.x / K, b = threadIdx.x - local * K;
  const int64_t pairid = (int64_t)blockIdx.x * per + local;
  const bool active = local < per && pairid < rows * nw;
  int64_t n = 0;
  int iw = 0;
  if (active) {
    n = pairid / nw;
    iw = (int)(pairid - n * nw);
    sm[local * K + b] = Y[n * stride + (int64_t)iw * K + b];
  }
  __syncthreads();
  if (!active) return;
  const z128 *m = M + (int64_t)iw * K * K;
  z128 s = zmake<z128>(0, 0);
  const int aend = upper ? b + 1 : K;
  for (int a = 0; a < aend; ++a) zmac(s, sm[local * K + a], m[a * K + b]);
  Y[n * stride + (int64_t)iw * K + b] = s;
}

// Y[n][iw][:] <- Y[n][iw][:] * M[iw] for an upper-triangular M, in place.
// Output b needs b + 1 products, so thread j of a row-frequency pair's
// H = ceil(K/2) threads takes outputs j and K-1-j: K + 1 products each
// (the warp's lanes finish together).
__global__ void __launch_bounds__(256) k_apply_upper(z128 *__restrict__ Y, int64_t stride, int64_t rows, int nw,
                                                     int K, const z128 *__restrict__ M) {
  extern __shared__ z128 sm[];
  const int H = (K + 1) / 2;
  const int per = blockDim.x / H;
  const int local = threadIdx.x / H, j = threadIdx.x - local * H;
  const int64_t pairid = (int64_t)blockIdx.x * per + local;
  const bool active = local < per && pairid < rows * nw;
  int64_t n = 0;
  int iw = 0;
  if (active) {
    n = pairid / nw;
    iw = (int)(pairid - n * nw);
    const z128 *y = Y + n * stride + (int64_t)iw * K;
    sm[local * K + j] = y[j];
    if (K - 1 - j != j) sm[local * K + K - 1 - j] = y[K - 1 - j];
  }
  __syncthreads();
  if (!active) return;
  const z128 *m = M + (int64_t)iw * K * K;
  const z128 *x = sm + local * K;
  z128 s1 = zmake<z128>(0, 0), s2 = zmake<z128>(0, 0);
  const int b1 = j, b2 = K - 1 - j;
  // One loop of K + 1 products for every lane (b1 + 1 for output b1, then
  // b2 + 1 for output b2), so the warp's lanes do not diverge at the switch;
  // each output's products are summed in ascending a.
  const int n1 = b1 + 1, ntot = b2 != b1 ? K + 1 : n1;
  for (int q = 0; q < ntot; ++q) {
    const bool first = q < n1;
    const int a = first ? q : q - n1, b = first ? b1 : b2;
    z128 acc = first ? s1 : s2;
    zmac(acc, x[a], m[a * K + b]);
    if (first)
      s1 = acc;
    else
      s2 = acc;
  }
  z128 *y = Y + n * stride + (int64_t)iw * K;
  y[b1] = s1;
  if (b2 != b1) y[b2] = s2;
}

struct DenseScratch {
  z128 *part, *G, *R, *Rinv, *Racc;
  int chunks;
};

static rsvdt_status dense_scratch(rsvdt_ctx *ctx, int64_t rows, int64_t nw, int64_t K,
                                  DenseScratch &s, size_t extra_bytes, void **extra) {
  const int chunks = (int)((rows + kGramRows - 1) / kGramRows);
  const size_t pk = (size_t)nw * K * K;
  size_t need = sizeof(z128) * ((size_t)chunks * pk + 4 * pk) + extra_bytes + 256;
  if (ctx->scratch_bytes < need) {
    dfree(ctx, ctx->scratch);
    ctx->scratch = dalloc(ctx, need);
    ctx->scratch_bytes = ctx->scratch ? need : 0;
    if (!ctx->scratch) return set_err(ctx, RSVDT_ERR_OOM, "scratch allocation of %zu bytes failed", need);
  }
  z128 *p = (z128 *)ctx->scratch;
  s.part = p;
  s.G = p + (size_t)chunks * pk;
  s.R = s.G + pk;
  s.Rinv = s.R + pk;
  s.Racc = s.Rinv + pk;
  s.chunks = chunks;
  if (extra) *extra = (void *)(s.Racc + pk);
  return RSVDT_OK;
}

static rsvdt_status gram(rsvdt_ctx *ctx, const z128 *X, int64_t sx, const z128 *Y, int64_t sy,
                         int64_t rows, int nw, int KA, int KB, DenseScratch &s) {
  if (KA + KB > 256) return set_err(ctx, RSVDT_ERR_ARG, "block too wide for the Gram kernel (%d x %d)", KA, KB);
  const int pairs_ = KA * KB;
  if (X == Y && sx == sy && KA == KB) {
    const int P = KA * (KA + 1) / 2;
    dim3 g(s.chunks, nw, P <= 256 ? 1 : (P + 255) / 256);
    k_gram_sym<<<g, 256, sizeof(z128) * (kGramTile * KA + 256), ctx->stream>>>(X, sx, rows, KA, s.part);
  } else {
    dim3 g(s.chunks, nw, (pairs_ + 1023) / 1024);
    size_t sm = sizeof(z128) * kGramTile * (KA + KB);
    k_gram_part<<<g, 256, sm, ctx->stream>>>(X, sx, Y, sy, rows, KA, KB, s.part);
  }
  const int pairs = KA * KB;
  k_gram_reduce<<<grid_for((int64_t)nw * pairs, 256), 256, 0, ctx->stream>>>(s.part, s.chunks, nw,
                                                                              pairs, s.G);
  ctx->launches += 2;
  return cuda_ok(ctx, cudaGetLastError(), "gram") ? RSVDT_OK : RSVDT_ERR_CUDA;
}

static rsvdt_status apply_small(rsvdt_ctx *ctx, z128 *Y, int64_t stride, int64_t rows, int nw,
                                int K, const z128 *M, bool upper) {
  if (K > 256) return set_err(ctx, RSVDT_ERR_ARG, "block too wide (%d)", K);
  const int64_t pairs = rows * nw;
  if (upper) {
    const int H = (K + 1) / 2, per = 256 / H;
    k_apply_upper<<<grid_for(pairs, per), per * H, sizeof(z128) * per * K, ctx->stream>>>(Y, stride, rows, nw, K, M);
  } else {
    const int per = 256 / K;
    k_apply_small<<<grid_for(pairs, per), per * K, sizeof(z128) * per * K, ctx->stream>>>(Y, stride, rows, nw, K,
                                                                                       M, 0);
  }
  ctx->launches += 1;
  return cuda_ok(ctx, cudaGetLastError(), "apply") ? RSVDT_OK : RSVDT_ERR_CUDA;
}

// CholQR on every frequency block of blk ([rows][nw][K]): `passes` Cholesky
// passes, the first `shifted` of them on G + s*trace(G)*I with
// s = 11 (m n + n (n+1)) u (shifted CholQR, Fukaya et al. 2020). Each pass
// maps the block by an invertible upper-triangular matrix, so the span is
// kept; a shifted pass lifts tiny singular values by ~1/sqrt(s), so
// shifted passes followed by one plain pass orthonormalise even a
// numerically rank-deficient block (its noise directions are normalised,
// as Gram-Schmidt does). Rout (optional, device, [nw][K][K]) receives the
// accumulated R with Y = Q R.
static rsvdt_status cholqr_n(rsvdt_ctx *ctx, z128 *blk, int64_t stride, int64_t rows, int64_t nw,
                             int64_t K, int passes, int shifted, z128 *Rout) {
  const double shift = 11.0 * ((double)rows * K + (double)K * (K + 1)) * 1.1102230246251565e-16;
  DenseScratch s;
  rsvdt_status st = dense_scratch(ctx, rows, nw, K, s, 0, nullptr);
  if (st) return st;
  if (!cuda_ok(ctx, cudaMemsetAsync(ctx->d_flags, 0, sizeof(int32_t), ctx->stream), "memset"))
    return RSVDT_ERR_CUDA;
  // Racc = I
  {
    std::vector<z128> eye((size_t)nw * K * K);
    for (auto &e : eye) e = zmake<z128>(0, 0);
    for (int64_t iw = 0; iw < nw; ++iw)
      for (int64_t a = 0; a < K; ++a) eye[(size_t)(iw * K + a) * K + a] = zmake<z128>(1, 0);
    if (!cuda_ok(ctx, cudaMemcpyAsync(s.Racc, eye.data(), sizeof(z128) * eye.size(),
                                      cudaMemcpyHostToDevice, ctx->stream),
                 "copy"))
      return RSVDT_ERR_CUDA;
    if (!cuda_ok(ctx, cudaStreamSynchronize(ctx->stream), "sync")) return RSVDT_ERR_CUDA;
  }
  for (int p = 0; p < passes; ++p) {
    st = gram(ctx, blk, stride, blk, stride, rows, (int)nw, (int)K, (int)K, s);
    if (st) return st;
    k_chol<<<grid_for(nw, 64), 64, 0, ctx->stream>>>(s.G, (int)nw, (int)K, p < shifted ? shift : 0.0,
                                                     s.R, s.Rinv, s.Racc, ctx->d_flags);
    ctx->launches += 1;
    st = apply_small(ctx, blk, stride, rows, (int)nw, (int)K, s.Rinv, true);
    if (st) return st;
  }
  int32_t flags = 0;
  if (!cuda_ok(ctx, cudaMemcpyAsync(&flags, ctx->d_flags, sizeof(flags), cudaMemcpyDeviceToHost,
                                    ctx->stream),
               "copy") ||
      !cuda_ok(ctx, cudaStreamSynchronize(ctx->stream), "sync"))
    return RSVDT_ERR_CUDA;
  if (flags & 2)
    return set_err(ctx, RSVDT_ERR_NOT_SPD,
                   "Cholesky of a Gram matrix failed: a frequency block is rank deficient");
  if (Rout &&
      !cuda_ok(ctx, cudaMemcpyAsync(Rout, s.Racc, sizeof(z128) * nw * K * K,
                                    cudaMemcpyDeviceToDevice, ctx->stream),
               "copy"))
    return RSVDT_ERR_CUDA;
  return RSVDT_OK;
}

// QRAllFreqs: shifted CholQR3 (one shifted pass, two plain), which covers
// blocks with condition numbers up to ~1/u; a well-conditioned block gets
// the same Q as CholQR2 or Gram-Schmidt (the QR factor with a positive
// diagonal is unique).
rsvdt_status cholqr2(rsvdt_ctx *ctx, z128 *blk, int64_t rows, int64_t nw, int64_t K, z128 *Rout) {
  return cholqr_n(ctx, blk, nw * K, rows, nw, K, 3, 1, Rout);
}

// One-sided Jacobi SVD of each K x K upper-triangular R[iw]: columns of
// R W = U_R S; writes U_R (columns sorted by descending S) and S.
__global__ void k_small_svd(z128 *__restrict__ Rm, int nw, int K, z128 *__restrict__ Uo,
                            double *__restrict__ S) {
  const int iw = blockIdx.x * blockDim.x + threadIdx.x;
  if (iw >= nw) return;
  z128 *A = Rm + (int64_t)iw * K * K;  // A[a*K + b] = row a, column b
  for (int sweep = 0; sweep < 60; ++sweep) {
    double off = 0;
    for (int p = 0; p < K - 1; ++p)
      for (int q = p + 1; q < K; ++q) {
        double app = 0, aqq = 0;
        z128 apq = zmake<z128>(0, 0);
        for (int a = 0; a < K; ++a) {
          const z128 x = A[a * K + p], y = A[a * K + q];
          app += x.re * x.re + x.im * x.im;
          aqq += y.re * y.re + y.im * y.im;
          zmacc(apq, x, y);
        }
        const double mag = hypot(apq.re, apq.im);
        if (mag == 0 || mag <= 1e-15 * sqrt(app * aqq)) continue;
        off = fmax(off, mag / sqrt(app * aqq));
        const z128 ph = zmake<z128>(apq.re / mag, apq.im / mag);
        const double tau = (aqq - app) / (2 * mag);
        const double t = (tau >= 0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1 + tau * tau));
        const double c = 1 / sqrt(1 + t * t), sn = c * t;
        for (int a = 0; a < K; ++a) {
          const z128 x = A[a * K + p], y = A[a * K + q];
          // x' = c x - sn conj(ph) y ; y' = sn ph x + c y
          z128 cy = zmul(zmake<z128>(ph.re, -ph.im), y);
          z128 px = zmul(ph, x);
          A[a * K + p] = zmake<z128>(c * x.re - sn * cy.re, c * x.im - sn * cy.im);
          A[a * K + q] = zmake<z128>(sn * px.re + c * y.re, sn * px.im + c * y.im);
        }
      }
    if (off <= 1e-15) break;
  }
  // Column norms, descending order (insertion sort on a small index list).
  int order[64];
  double nr[64];
  for (int b = 0; b < K; ++b) {
    double s = 0;
    for (int a = 0; a < K; ++a) s += A[a * K + b].re * A[a * K + b].re + A[a * K + b].im * A[a * K + b].im;
    nr[b] = sqrt(s);
    order[b] = b;
  }
  for (int i = 1; i < K; ++i) {
    int t = order[i], j = i;
    while (j > 0 && nr[order[j - 1]] < nr[t]) {
      order[j] = order[j - 1];
      --j;
    }
    order[j] = t;
  }
  z128 *u = Uo + (int64_t)iw * K * K;
  for (int j = 0; j < K; ++j) {
    const int src = order[j];
    const double sv = nr[src];
    S[(int64_t)iw * K + j] = sv;
    for (int a = 0; a < K; ++a) {
      const z128 v = A[a * K + src];
      u[a * K + j] = sv > 0 ? zmake<z128>(v.re / sv, v.im / sv) : zmake<z128>(0, 0);
    }
  }
}

rsvdt_status svd_all(rsvdt_ctx *ctx, z128 *blk, int64_t rows, int64_t nw, int64_t K, z128 *Uout,
                     double *S) {
  if (K > 64) return set_err(ctx, RSVDT_ERR_ARG, "k = %lld exceeds 64", (long long)K);
  // R of every frequency is kept in a small buffer placed after the dense
  // scratch region.
  DenseScratch s;
  void *extra = nullptr;
  const size_t rbytes = sizeof(z128) * nw * K * K;
  rsvdt_status st = dense_scratch(ctx, rows, nw, K, s, 2 * rbytes, &extra);
  if (st) return st;
  z128 *Rk = (z128 *)extra;
  z128 *Uk = Rk + nw * K * K;
  st = cholqr_n(ctx, blk, nw * K, rows, nw, K, 3, 1, Rk);
  if (st) return st;
  k_small_svd<<<grid_for(nw, 32), 32, 0, ctx->stream>>>(Rk, (int)nw, (int)K, Uk, S);
  ctx->launches += 1;
  if (!cuda_ok(ctx, cudaGetLastError(), "small svd")) return RSVDT_ERR_CUDA;
  st = apply_small(ctx, blk, nw * K, rows, (int)nw, (int)K, Uk, false);
  if (st) return st;
  if (Uout && Uout != blk &&
      !cuda_ok(ctx, cudaMemcpyAsync(Uout, blk, sizeof(z128) * rows * nw * K,
                                    cudaMemcpyDeviceToDevice, ctx->stream),
               "copy"))
    return RSVDT_ERR_CUDA;
  return RSVDT_OK;
}

// ------------------------------------------------------- test-vector chunks

// Columns k0 .. k0+Kc-1 of every frequency of a [row][iw][Kb] block, to or
// from a [row][iw][Kc] chunk (gather: chunk = block columns; scatter: the
// reverse). Used by the capacity mode's weights and U store.
__global__ void k_chunk_copy(const z128 *__restrict__ src, z128 *__restrict__ dst, int64_t rows, int Nwe, int Kb,
                             int k0, int Kc, int gather) {
  const int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t total = rows * Nwe * (int64_t)Kc;
  if (u >= total) return;
  const int kc = (int)(u % Kc);
  const int64_t ri = u / Kc;  // row * Nwe + iw
  const int64_t b = ri * Kb + k0 + kc;
  if (gather)
    dst[u] = src[b];
  else
    dst[b] = src[u];
}

rsvdt_status launch_chunk_copy(rsvdt_ctx *ctx, const z128 *src, z128 *dst, int64_t rows, int64_t Nwe, int64_t Kb,
                               int64_t k0, int64_t Kc, bool gather) {
  const int th = 256;
  k_chunk_copy<<<grid_for(rows * Nwe * Kc, th), th, 0, ctx->stream>>>(src, dst, rows, (int)Nwe, (int)Kb, (int)k0,
                                                                     (int)Kc, gather ? 1 : 0);
  ctx->launches += 1;
  return cuda_ok(ctx, cudaGetLastError(), "chunk copy") ? RSVDT_OK : RSVDT_ERR_CUDA;
}

// ---------------------------------------------------------------- misc

__device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// Standard complex normal entries, re and im ~ N(0, 1/2), Box-Muller on two
// 53-bit uniforms from a counter-based generator.
__global__ void k_random(z128 *dst, int64_t n, uint64_t seed) {
  const int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (u >= n) return;
  const uint64_t a = splitmix64(seed ^ splitmix64((uint64_t)u * 2 + 1));
  const uint64_t b = splitmix64(a ^ 0xD1B54A32D192ED03ull);
  const double u1 = ((double)(a >> 11) + 1.0) * (1.0 / 9007199254740992.0);  // (0, 1]
  const double u2 = (double)(b >> 11) * (1.0 / 9007199254740992.0);          // [0, 1)
  const double rad = sqrt(-log(u1));  // sqrt(-2 ln u1) / sqrt(2)
  double sn, cs;
  sincospi(2.0 * u2, &sn, &cs);
  dst[u] = zmake<z128>(rad * cs, rad * sn);
}

rsvdt_status launch_random(rsvdt_ctx *ctx, z128 *dst, int64_t n, uint64_t seed) {
  k_random<<<grid_for(n, 256), 256, 0, ctx->stream>>>(dst, n, seed);
  ctx->launches += 1;
  return cuda_ok(ctx, cudaGetLastError(), "random") ? RSVDT_OK : RSVDT_ERR_CUDA;
}

__global__ void k_to64(const z128 *__restrict__ s, z64 *__restrict__ d, int64_t n) {
  const int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (u < n) d[u] = zmake<z64>((float)s[u].re, (float)s[u].im);
}

rsvdt_status launch_convert_to64(rsvdt_ctx *ctx, const z128 *src, z64 *dst, int64_t n) {
  k_to64<<<grid_for(n, 256), 256, 0, ctx->stream>>>(src, dst, n);
  ctx->launches += 1;
  return cuda_ok(ctx, cudaGetLastError(), "convert") ? RSVDT_OK : RSVDT_ERR_CUDA;
}

__global__ void k_finite(const z128 *__restrict__ p, int64_t n, int32_t *flags) {
  const int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (u < n && (!isfinite(p[u].re) || !isfinite(p[u].im))) atomicOr(flags, 1);
}

rsvdt_status check_finite(rsvdt_ctx *ctx, const z128 *p, int64_t n, bool *ok) {
  int32_t flags = 0;
  if (!cuda_ok(ctx, cudaMemsetAsync(ctx->d_flags, 0, sizeof(int32_t), ctx->stream), "memset"))
    return RSVDT_ERR_CUDA;
  k_finite<<<grid_for(n, 256), 256, 0, ctx->stream>>>(p, n, ctx->d_flags);
  ctx->launches += 1;
  if (!cuda_ok(ctx, cudaMemcpyAsync(&flags, ctx->d_flags, sizeof(flags), cudaMemcpyDeviceToHost,
                                    ctx->stream),
               "copy") ||
      !cuda_ok(ctx, cudaStreamSynchronize(ctx->stream), "sync"))
    return RSVDT_ERR_CUDA;
  *ok = (flags & 1) == 0;
  return RSVDT_OK;
}

// ---------------------------------------------------- transient removal

// V[n][p] = ring[p][n][ik] for p < Ns1 (complex128 or complex64 ring).
template <class Z>
__global__ void k_extract(const Z *__restrict__ ring, int64_t N, int K, int ik, int Ns1,
                          z128 *__restrict__ V) {
  const int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (u >= N * Ns1) return;
  const int64_t n = u / Ns1;
  const int p = (int)(u - n * Ns1);
  const Z v = ring[((int64_t)p * N + n) * K + ik];
  V[u] = zmake<z128>((double)v.re, (double)v.im);
}

// y1[n][iw] = R * sum_j S[n][j + o1] dft[j][iw], y2 likewise with o2
// (SourceCode/GalerkinProj.c:30-46). S is the [n][Ns1] snapshot matrix.
__global__ void k_dft_pair(const z128 *__restrict__ S, int64_t N, int Ns1, int Nw, int Nwe,
                           int o1, int o2, const z128 *__restrict__ dft, double R,
                           z128 *__restrict__ y1, z128 *__restrict__ y2) {
  const int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (u >= N * Nwe) return;
  const int64_t n = u / Nwe;
  const int iw = (int)(u - n * Nwe);
  z128 s1 = zmake<z128>(0, 0), s2 = zmake<z128>(0, 0);
  for (int j = 0; j < Nw; ++j) {
    const z128 d = dft[(int64_t)iw * Nw + j];
    zmac(s1, S[n * Ns1 + j + o1], d);
    zmac(s2, S[n * Ns1 + j + o2], d);
  }
  y1[u] = zmake<z128>(s1.re * R, s1.im * R);
  y2[u] = zmake<z128>(s2.re * R, s2.im * R);
}

// B[iw][a] = sum_n conj(V[n][a]) * (e_iw * y1[n][iw] - y2[n][iw]); grid (chunks, nwe).
__global__ void __launch_bounds__(256) k_proj_rhs(const z128 *__restrict__ V, int64_t N, int Ns1,
                                                  const z128 *__restrict__ y1,
                                                  const z128 *__restrict__ y2, int Nwe,
                                                  const z128 *__restrict__ e,
                                                  z128 *__restrict__ part) {
  const int iw = blockIdx.y;
  const int64_t n0 = (int64_t)blockIdx.x * kGramRows, n1 = min(N, n0 + kGramRows);
  const z128 ew = e[iw];
  for (int a = threadIdx.x; a < Ns1; a += blockDim.x) {
    z128 s = zmake<z128>(0, 0);
    for (int64_t n = n0; n < n1; ++n) {
      const z128 a1 = y1[n * Nwe + iw], a2 = y2[n * Nwe + iw];
      z128 t = zmul(ew, a1);
      t.re -= a2.re;
      t.im -= a2.im;
      zmacc(s, V[n * Ns1 + a], t);
    }
    part[((int64_t)blockIdx.x * Nwe + iw) * Ns1 + a] = s;
  }
}

// Solve (e_iw I - Mt) x = b for every iw (LU with partial pivoting; the
// reference runs PGMRES to 1e-15, SourceCode/GalerkinProj.c:57-61). Work
// matrices in W ([iw][Ns1][Ns1], column-major).
__global__ void k_galerkin_solve(const z128 *__restrict__ Mt, int Ns1, int Nwe,
                                 const z128 *__restrict__ e, z128 *__restrict__ W,
                                 z128 *__restrict__ b, int32_t *flags) {
  const int iw = blockIdx.x * blockDim.x + threadIdx.x;
  if (iw >= Nwe) return;
  const int m = Ns1;
  z128 *M = W + (int64_t)iw * m * m;
  z128 *x = b + (int64_t)iw * m;
  for (int c = 0; c < m; ++c)
    for (int r = 0; r < m; ++r) {
      z128 v = Mt[r * m + c];  // Mt row-major: Mt[r*m + c] = row r, col c
      v.re = -v.re;
      v.im = -v.im;
      if (r == c) {
        v.re += e[iw].re;
        v.im += e[iw].im;
      }
      M[c * m + r] = v;
    }
  for (int c = 0; c < m; ++c) {
    int piv = c;
    double best = hypot(M[c * m + c].re, M[c * m + c].im);
    for (int r = c + 1; r < m; ++r) {
      const double v = hypot(M[c * m + r].re, M[c * m + r].im);
      if (v > best) {
        best = v;
        piv = r;
      }
    }
    if (best == 0) {
      atomicOr(flags, 4);
      return;
    }
    if (piv != c) {
      for (int cc = 0; cc < m; ++cc) {
        z128 t = M[cc * m + c];
        M[cc * m + c] = M[cc * m + piv];
        M[cc * m + piv] = t;
      }
      z128 t = x[c];
      x[c] = x[piv];
      x[piv] = t;
    }
    const z128 d = M[c * m + c];
    const double dd = d.re * d.re + d.im * d.im;
    for (int r = c + 1; r < m; ++r) {
      const z128 v = M[c * m + r];
      const z128 l = zmake<z128>((v.re * d.re + v.im * d.im) / dd, (v.im * d.re - v.re * d.im) / dd);
      M[c * m + r] = l;
      for (int cc = c + 1; cc < m; ++cc) {
        const z128 t = zmul(l, M[cc * m + c]);
        M[cc * m + r].re -= t.re;
        M[cc * m + r].im -= t.im;
      }
      const z128 t = zmul(l, x[c]);
      x[r].re -= t.re;
      x[r].im -= t.im;
    }
  }
  for (int r = m - 1; r >= 0; --r) {
    z128 s = x[r];
    for (int cc = r + 1; cc < m; ++cc) {
      const z128 t = zmul(M[cc * m + r], x[cc]);
      s.re -= t.re;
      s.im -= t.im;
    }
    const z128 d = M[r * m + r];
    const double dd = d.re * d.re + d.im * d.im;
    x[r] = zmake<z128>((s.re * d.re + s.im * d.im) / dd, (s.im * d.re - s.re * d.im) / dd);
  }
}

// out[n][iw][ik] = y1[n][iw] - sum_a V[n][a] * x[iw][a]
__global__ void k_galerkin_update(const z128 *__restrict__ V, int64_t N, int Ns1,
                                  const z128 *__restrict__ y1, int Nwe,
                                  const z128 *__restrict__ x, int K, int ik,
                                  z128 *__restrict__ out) {
  const int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (u >= N * Nwe) return;
  const int64_t n = u / Nwe;
  const int iw = (int)(u - n * Nwe);
  z128 s = zmake<z128>(0, 0);
  for (int a = 0; a < Ns1; ++a) zmac(s, V[n * Ns1 + a], x[(int64_t)iw * Ns1 + a]);
  const z128 v = y1[u];
  out[(n * Nwe + iw) * K + ik] = zmake<z128>(v.re - s.re, v.im - s.im);
}

// TransientRemovalStrategy (SourceCode/TransientRemovalStrategy.c:30-40):
// for every test vector, V = QR(snapshots), M_tilde = V^H e^{A dT} V with
// e^{A dT} applied by ResRatio unforced RK4 steps, then the Galerkin
// correction of each frequency. Writes out[n][iw][k].
rsvdt_status transient_removal(rsvdt_ctx *ctx, int dir, int prec, z128 *out) {
  // The ring holds the state's Ks test vectors; they are columns k0.. of out.
  const int64_t N = ctx->N, K = ctx->Ks, Kb = ctx->K, k0 = ctx->k0, Nw = ctx->Nw, Nwe = ctx->Nw_eff,
                R = ctx->R;
  const int Ns1 = (int)(Nw + 1);
  if (Ns1 > 32 * 32) return set_err(ctx, RSVDT_ERR_ARG, "Nw too large for transient removal");
  // Buffers: V, MV [N][Ns1]; y1, y2 [N][Nwe]; Mt [Ns1^2]; rhs parts; W.
  const int chunks = (int)((N + kGramRows - 1) / kGramRows);
  const size_t nV = (size_t)N * Ns1, nY = (size_t)N * Nwe;
  const size_t bytes = sizeof(z128) * (2 * nV + 2 * nY + (size_t)chunks * Nwe * Ns1 +
                                       (size_t)Nwe * Ns1 + (size_t)Nwe * Ns1 * Ns1 + Nwe);
  z128 *buf = (z128 *)dalloc(ctx, bytes);
  if (!buf) return set_err(ctx, RSVDT_ERR_OOM, "transient-removal buffers (%zu bytes)", bytes);
  z128 *V = buf, *MV = V + nV, *y1 = MV + nV, *y2 = y1 + nY;
  z128 *rpart = y2 + nY, *rhs = rpart + (size_t)chunks * Nwe * Ns1;
  z128 *W = rhs + (size_t)Nwe * Ns1, *ev = W + (size_t)Nwe * Ns1 * Ns1;
  // Shift phasors e^{+-i w iw dT} (SourceCode/GalerkinProj.c:49-54).
  std::vector<z128> eh((size_t)Nwe);
  const double deltaT = ctx->dt * (double)R;
  for (int64_t iw = 0; iw < Nwe; ++iw) {
    const double ang = (dir ? 1.0 : -1.0) * ctx->w * (double)iw * deltaT;
    eh[(size_t)iw] = zmake<z128>(cos(ang), sin(ang));
  }
  rsvdt_status st = RSVDT_OK;
  if (!cuda_ok(ctx, cudaMemcpyAsync(ev, eh.data(), sizeof(z128) * Nwe, cudaMemcpyHostToDevice,
                                    ctx->stream),
               "copy") ||
      !cuda_ok(ctx, cudaStreamSynchronize(ctx->stream), "sync")) {
    dfree(ctx, buf);
    return RSVDT_ERR_CUDA;
  }
  for (int64_t ik = 0; ik < K && st == RSVDT_OK; ++ik) {
    const int th = 256;
    if (prec == RSVDT_PREC_C64)
      k_extract<z64><<<grid_for((int64_t)nV, th), th, 0, ctx->stream>>>((const z64 *)ctx->ring, N,
                                                                         (int)K, (int)ik, Ns1, V);
    else
      k_extract<z128><<<grid_for((int64_t)nV, th), th, 0, ctx->stream>>>(
          (const z128 *)ctx->ring, N, (int)K, (int)ik, Ns1, V);
    // y1, y2 from the raw snapshots (direct: y1 on columns 0..Nw-1).
    k_dft_pair<<<grid_for((int64_t)nY, th), th, 0, ctx->stream>>>(
        V, N, Ns1, (int)Nw, (int)Nwe, dir ? 0 : 1, dir ? 1 : 0, ctx->dft, (double)R, y1, y2);
    ctx->launches += 2;
    // Orthonormal basis of the snapshots: three shifted CholQR passes and a
    // plain one. Once the transient has decayed, Nw+1 samples of a periodic
    // response with Nw harmonics are numerically rank deficient.
    st = cholqr_n(ctx, V, Ns1, N, 1, Ns1, 4, 3, nullptr);
    if (st) break;
    if (!cuda_ok(ctx, cudaMemcpyAsync(MV, V, sizeof(z128) * nV, cudaMemcpyDeviceToDevice, ctx->stream),
                 "copy")) {
      st = RSVDT_ERR_CUDA;
      break;
    }
    st = launch_unforced_steps(ctx, dir, MV, Ns1, R);
    if (st) break;
    // M_tilde = V^H MV (SourceCode/CreateMtilde.c:49-51).
    DenseScratch s;
    st = dense_scratch(ctx, N, 1, Ns1, s, 0, nullptr);
    if (st) break;
    st = gram(ctx, V, Ns1, MV, Ns1, N, 1, Ns1, Ns1, s);
    if (st) break;
    k_proj_rhs<<<dim3(chunks, (unsigned)Nwe), 128, 0, ctx->stream>>>(V, N, Ns1, y1, y2, (int)Nwe,
                                                                     ev, rpart);
    k_gram_reduce<<<grid_for(Nwe * Ns1, 256), 256, 0, ctx->stream>>>(rpart, chunks, (int)Nwe, Ns1,
                                                                       rhs);
    k_galerkin_solve<<<grid_for(Nwe, 32), 32, 0, ctx->stream>>>(s.G, Ns1, (int)Nwe, ev, W, rhs,
                                                                 ctx->d_flags);
    k_galerkin_update<<<grid_for((int64_t)nY, th), th, 0, ctx->stream>>>(V, N, Ns1, y1, (int)Nwe,
                                                                         rhs, (int)Kb, (int)(k0 + ik), out);
    ctx->launches += 4;
    if (!cuda_ok(ctx, cudaGetLastError(), "transient removal")) st = RSVDT_ERR_CUDA;
  }
  if (!cuda_ok(ctx, cudaStreamSynchronize(ctx->stream), "sync") && st == RSVDT_OK) st = RSVDT_ERR_CUDA;
  dfree(ctx, buf);
  return st;
}

}  // namespace rsvdt

// ------------------------------------- QR without any device allocation
//
// rsvdt_qr_all_freqs_noalloc orthonormalises caller-owned device blocks
// with the same CholQR passes as QRAllFreqs, but takes its scratch (Gram
// partials, Gram matrices, R^{-1}, a status flag) from the file-scope
// device array below instead of allocating. It is meant for callers that
// cannot call cudaMalloc: code running while a stream capture is open
// elsewhere, host frameworks that own all device memory through their own
// pool (a PETSc/SLEPc application with its own allocator, for example), or
// long-running services that forbid allocation after start-up. The array
// is fixed at kNoAllocScratchBytes per device that loads this library and
// stays resident until the process exits.

namespace {

constexpr size_t kNoAllocScratchBytes = 4u << 20;  // 4 MiB
constexpr size_t kNoAllocElems = kNoAllocScratchBytes / sizeof(rsvdt::z128);

static __device__ __align__(256) rsvdt::z128 g_noalloc_scratch[kNoAllocElems];

// Gram partials with a caller-chosen chunk length (variant of k_gram_part,
// which uses a fixed chunk of kGramRows rows).
__global__ void __launch_bounds__(256) k_gram_part_chunk(const rsvdt::z128 *__restrict__ X, int64_t sx,
                                                         int64_t rows, int K, int64_t chunk_rows,
                                                         rsvdt::z128 *__restrict__ part) {
  using namespace rsvdt;
  extern __shared__ z128 sm[];  // [kGramTile][K]
  const int iw = blockIdx.y, nw = gridDim.y;
  const int64_t n0 = (int64_t)blockIdx.x * chunk_rows;
  const int64_t n1 = min(rows, n0 + chunk_rows);
  const int pairs = K * K;
  const int pbase = blockIdx.z * 1024;
  z128 acc[4];
  for (int q = 0; q < 4; ++q) acc[q] = zmake<z128>(0, 0);
  for (int64_t nb = n0; nb < n1; nb += kGramTile) {
    const int nr = (int)min((int64_t)kGramTile, n1 - nb);
    __syncthreads();
    for (int e = threadIdx.x; e < nr * K; e += blockDim.x) {
      int rr = e / K, a = e - rr * K;
      sm[rr * K + a] = X[(nb + rr) * sx + (int64_t)iw * K + a];
    }
    __syncthreads();
    for (int q = 0; q < 4; ++q) {
      const int p = pbase + threadIdx.x + q * blockDim.x;
      if (p >= pairs) break;
      const int a = p / K, b = p - a * K;
      z128 s = acc[q];
      for (int rr = 0; rr < nr; ++rr) zmacc(s, sm[rr * K + a], sm[rr * K + b]);
      acc[q] = s;
    }
  }
  for (int q = 0; q < 4; ++q) {
    const int p = pbase + threadIdx.x + q * blockDim.x;
    if (p >= pairs) break;
    part[((int64_t)blockIdx.x * nw + iw) * pairs + p] = acc[q];
  }
}

static rsvdt_status noalloc_fail(char *errbuf, int64_t errlen, rsvdt_status st, const char *fmt, ...) {
  if (errbuf && errlen > 0) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(errbuf, (size_t)errlen, fmt, ap);
    va_end(ap);
  }
  return st;
}

}  // namespace

extern "C" rsvdt_status rsvdt_qr_all_freqs_noalloc(const double *Y, double *Q, int64_t rows, int64_t nw,
                                                   int64_t k, void *stream, char *errbuf, int64_t errlen) {
  using namespace rsvdt;
  if (errbuf && errlen > 0) errbuf[0] = '\0';
  if (!Y || !Q || rows < 1 || nw < 1 || k < 1)
    return noalloc_fail(errbuf, errlen, RSVDT_ERR_ARG, "invalid arguments (null pointer or non-positive size)");
  if (k > 32 || rows > INT32_MAX)
    return noalloc_fail(errbuf, errlen, RSVDT_ERR_ARG, "k = %lld exceeds 32 or rows exceed 2^31",
                        (long long)k);
  // Scratch layout (complex values): partials [chunks][nw][k][k], G, Rinv,
  // R [nw][k][k] each, then one element holding the status flag.
  const int64_t pk = nw * k * k;
  const int64_t avail = (int64_t)kNoAllocElems - 1;
  if (4 * pk > avail)
    return noalloc_fail(errbuf, errlen, RSVDT_ERR_ARG,
                        "nw*k*k = %lld needs %lld bytes of scratch; the fixed scratch array holds %zu bytes "
                        "(limit nw*k*k <= %lld)",
                        (long long)pk, (long long)(4 * pk + 1) * 16, kNoAllocScratchBytes, (long long)(avail / 4));
  // The array's device address in the current device's context. It is
  // looked up on every call rather than cached: after a cudaDeviceReset (or
  // any other teardown of the context) the module is loaded again and the
  // array can sit at a new address. The lookup is a host-side query and
  // allocates nothing; only the first call in a context may load the
  // library's device code into it. A host symbol's address is not a device
  // address, so the kernels get this pointer, never &g_noalloc_scratch.
  void *scr_ptr = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&scr_ptr, g_noalloc_scratch);
  if (e != cudaSuccess || !scr_ptr)
    return noalloc_fail(errbuf, errlen, RSVDT_ERR_CUDA, "cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
  cudaStream_t s = (cudaStream_t)stream;
  z128 *scr = (z128 *)scr_ptr;
  int64_t chunks = std::min((rows + kGramRows - 1) / kGramRows, avail / pk - 3);
  if (chunks < 1) chunks = 1;
  const int64_t chunk_rows = (rows + chunks - 1) / chunks;
  chunks = (rows + chunk_rows - 1) / chunk_rows;
  z128 *part = scr, *G = scr + chunks * pk, *R = G + pk, *Rinv = R + pk;
  int32_t *flag = (int32_t *)(scr + avail);
  z128 *out = (z128 *)Q;
  if (Q != Y) {
    e = cudaMemcpyAsync(Q, Y, sizeof(z128) * rows * nw * k, cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return noalloc_fail(errbuf, errlen, RSVDT_ERR_CUDA, "copy: %s", cudaGetErrorString(e));
  }
  // The flag keeps the previous call's value: clear it.
  e = cudaMemsetAsync(flag, 0, sizeof(int32_t), s);
  if (e != cudaSuccess) return noalloc_fail(errbuf, errlen, RSVDT_ERR_CUDA, "memset: %s", cudaGetErrorString(e));
  const int K = (int)k;
  const int per = 256 / K;
  for (int p = 0; p < 3; ++p) {  // one shifted pass, two plain (as rsvdt_qr_all_freqs)
    const double shift = p < 1 ? 11.0 * ((double)rows * k + (double)k * (k + 1)) * 1.1102230246251565e-16 : 0.0;
    dim3 g((unsigned)chunks, (unsigned)nw, (unsigned)((K * K + 1023) / 1024));
    k_gram_part_chunk<<<g, 256, sizeof(z128) * kGramTile * K, s>>>(out, nw * k, rows, K, chunk_rows, part);
    k_gram_reduce<<<grid_for(pk, 256), 256, 0, s>>>(part, (int)chunks, (int)nw, K * K, G);
    k_chol<<<grid_for(nw, 64), 64, 0, s>>>(G, (int)nw, K, shift, R, Rinv, nullptr, flag);
    k_apply_small<<<grid_for(rows * nw, per), per * K, sizeof(z128) * per * K, s>>>(out, nw * k, rows, (int)nw, K,
                                                                                     Rinv, 1);
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return noalloc_fail(errbuf, errlen, RSVDT_ERR_CUDA, "launch: %s", cudaGetErrorString(e));
  int32_t hflag = 0;
  e = cudaMemcpyAsync(&hflag, flag, sizeof(int32_t), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return noalloc_fail(errbuf, errlen, RSVDT_ERR_CUDA, "sync: %s", cudaGetErrorString(e));
  if (hflag & 2)
    return noalloc_fail(errbuf, errlen, RSVDT_ERR_NOT_SPD, "Cholesky of a Gram matrix failed: a block is rank deficient");
  return RSVDT_OK;
}
