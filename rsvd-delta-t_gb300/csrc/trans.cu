// Transient simulation (SourceCode/TransientRunRK4.c:11-228): unforced RK4
// of one state vector from an initial condition, with the state norm
// checked every TransSaveMod steps and, optionally, the transient-removal
// estimate of SourceCode/TransientRemovalEst.c:6-129 at the end of every
// period.
//
// Device layout: the state y (N complex128) and the five RK4 work vectors
// of the stage kernels (step.cu, K = 1); for the estimate, the snapshot
// columns Q[col][n] (Nw columns, one per deltaT = T/Nw of the running
// period) and qss = -q0. Steps between host decisions replay a CUDA graph
// of 16 steps; the host synchronises only at norm checks.
//
// Norms are deterministic: fixed-size grids, partial sums per block in a
// fixed order, a one-block final sum.
//
// The estimate orthonormalises, for each of the Nw/2 non-negative
// frequencies, the synthetic snapshots Q[:, s1] + qss e^{i w s deltaT}
// with qss appended as a last column, by classical Gram-Schmidt with one
// full re-orthogonalisation (CGS2), all frequencies of a group in one
// launch. The updated transient norm |qss - U U^H qss| / |qss| is the norm
// that CGS2 leaves of that last column. Once the transient has decayed the
// synthetic snapshots are nearly parallel; a column whose norm after CGS2
// is below 1e-13 of its norm before is dependent and is set to zero rather
// than normalised (it spans nothing), which keeps the residual exact to
// rounding where a Cholesky-based QR would break down.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "common.cuh"

using namespace rsvdt;

namespace {

const double kPi = 3.14159265358979323846;
const int kNormBlocks = 304;  // 2 per SM; a fixed grid keeps the sums deterministic
const int kNormThreads = 256;
const int kChunkRows = 4096;   // rows per block of the Gram-Schmidt dot kernels
const double kDepTol = 1e-13;  // dependent-column threshold (relative)

#define TR_TRY(x)                    \
  do {                               \
    rsvdt_status s_ = (x);           \
    if (s_ != RSVDT_OK) return s_;   \
  } while (0)

__device__ __forceinline__ double block_sum(double v, double *sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) sh[warp] = v;
  __syncthreads();
  double s = 0;
  if (threadIdx.x == 0)
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += sh[w];
  return s;  // valid in thread 0
}

// part[b] = sum over the rows of block b (grid-stride) of |y|^2.
__global__ void __launch_bounds__(kNormThreads) k_sqnorm_part(const z128 *__restrict__ y, int64_t n,
                                                              double *__restrict__ part) {
  __shared__ double sh[kNormThreads / 32];
  double s = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const z128 v = y[i];
    s = fma(v.re, v.re, fma(v.im, v.im, s));
  }
  s = block_sum(s, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// out[0] = sqrt(sum part[0..nparts)) (one block, fixed order).
__global__ void k_sqnorm_final(const double *__restrict__ part, int nparts, double *__restrict__ out) {
  __shared__ double sh[kNormThreads / 32];
  double s = 0;
  for (int i = threadIdx.x; i < nparts; i += blockDim.x) s += part[i];
  s = block_sum(s, sh);
  if (threadIdx.x == 0) out[0] = sqrt(s);
}

// dst = scale * src.
__global__ void k_scaled_copy(const z128 *__restrict__ src, int64_t n, double scale, z128 *__restrict__ dst) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const z128 v = src[i];
  dst[i] = zmake<z128>(scale * v.re, scale * v.im);
}

// Initial transient norms (SourceCode/TransientRemovalEst.c:58-70):
// part[iw][b] = sum over block b's rows of |sum_j Q[j][n] dft[iw][j]|^2
// for the column iw = blockIdx.y.
__global__ void __launch_bounds__(kNormThreads) k_dft_norm_part(const z128 *__restrict__ Q, int64_t N, int Nw,
                                                                const z128 *__restrict__ dft,
                                                                double *__restrict__ part) {
  __shared__ double sh[kNormThreads / 32];
  const int iw = blockIdx.y;
  const z128 *d = dft + (int64_t)iw * Nw;
  double s = 0;
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < N; n += (int64_t)gridDim.x * blockDim.x) {
    z128 v = zmake<z128>(0, 0);
    for (int j = 0; j < Nw; ++j) zmac(v, Q[(int64_t)j * N + n], d[j]);
    s = fma(v.re, v.re, fma(v.im, v.im, s));
  }
  s = block_sum(s, sh);
  if (threadIdx.x == 0) part[(int64_t)iw * gridDim.x + blockIdx.x] = s;
}

// out[iw] = sqrt(sum_b part[iw][b]) * scale; one block per iw.
__global__ void k_rows_norm_final(const double *__restrict__ part, int nparts, double scale,
                                  double *__restrict__ out) {
  __shared__ double sh[kNormThreads / 32];
  const double *p = part + (int64_t)blockIdx.x * nparts;
  double s = 0;
  for (int i = threadIdx.x; i < nparts; i += blockDim.x) s += p[i];
  s = block_sum(s, sh);
  if (threadIdx.x == 0) out[blockIdx.x] = sqrt(s) * scale;
}

// Synthetic snapshots of one frequency group (SourceCode/TransientRemovalEst.c:85-97):
// B[g][s][n] = Q[s + skip][n] + qss[n] * ph[g][s] for s < m, B[g][m][n] = qss[n].
__global__ void k_est_build(const z128 *__restrict__ Q, const z128 *__restrict__ qss, int64_t N, int m,
                            int skip, const z128 *__restrict__ ph, int G, z128 *__restrict__ B) {
  const int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t cols = (int64_t)(m + 1);
  if (u >= (int64_t)G * cols * N) return;
  const int64_t n = u % N;
  const int64_t gs = u / N;
  const int s = (int)(gs % cols);
  const int g = (int)(gs / cols);
  const z128 q = qss[n];
  if (s == m) {
    B[u] = q;
    return;
  }
  const z128 e = ph[(int64_t)g * m + s];
  z128 v = Q[(int64_t)(s + skip) * N + n];
  zmac(v, q, e);
  B[u] = v;
}

// part[g][chunk][l - l0] = sum over the chunk's rows of conj(B[g][l][n]) B[g][c][n]
// for l in [l0, l1): one warp per l (strided by the block's warps).
__global__ void __launch_bounds__(256) k_cgs_dot(const z128 *__restrict__ B, int64_t N, int cols, int c,
                                                  int l0, int l1, z128 *__restrict__ part) {
  const int g = blockIdx.y;
  const int chunk = blockIdx.x, nchunks = gridDim.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const z128 *base = B + (int64_t)g * cols * N;
  const z128 *xc = base + (int64_t)c * N;
  const int64_t r0 = (int64_t)chunk * kChunkRows;
  const int64_t r1 = r0 + kChunkRows < N ? r0 + kChunkRows : N;
  const int nl = l1 - l0;
  for (int l = l0 + warp; l < l1; l += nwarps) {
    const z128 *xl = base + (int64_t)l * N;
    z128 s = zmake<z128>(0, 0);
    for (int64_t n = r0 + lane; n < r1; n += 32) zmacc(s, xl[n], xc[n]);
    for (int o = 16; o > 0; o >>= 1) {
      s.re += __shfl_down_sync(0xffffffffu, s.re, o);
      s.im += __shfl_down_sync(0xffffffffu, s.im, o);
    }
    if (lane == 0) part[((int64_t)g * nchunks + chunk) * nl + (l - l0)] = s;
  }
}

// h[g][j] = sum over chunks of part[g][chunk][j] (fixed order), j < nl.
__global__ void k_cgs_reduce(const z128 *__restrict__ part, int nchunks, int nl, int G, z128 *__restrict__ h) {
  const int u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= G * nl) return;
  const int g = u / nl, j = u - g * nl;
  z128 s = zmake<z128>(0, 0);
  for (int ch = 0; ch < nchunks; ++ch) {
    const z128 v = part[((int64_t)g * nchunks + ch) * nl + j];
    s.re += v.re;
    s.im += v.im;
  }
  h[(int64_t)g * nl + j] = s;
}

// B[g][c][n] -= sum_{l < c} B[g][l][n] h[g][l]   (h of stride hs per group).
__global__ void k_cgs_update(z128 *__restrict__ B, int64_t N, int cols, int c, const z128 *__restrict__ h,
                             int hs, int G) {
  const int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (u >= (int64_t)G * N) return;
  const int g = (int)(u / N);
  const int64_t n = u - (int64_t)g * N;
  z128 *base = B + (int64_t)g * cols * N;
  z128 v = base[(int64_t)c * N + n];
  const z128 *hg = h + (int64_t)g * hs;
  for (int l = 0; l < c; ++l) {
    const z128 a = base[(int64_t)l * N + n], b = hg[l];
    v.re -= a.re * b.re - a.im * b.im;
    v.im -= a.re * b.im + a.im * b.re;
  }
  base[(int64_t)c * N + n] = v;
}

// Normalises column c of every group (norm^2 in nrm2[g], norm before the
// orthogonalisation in nrm0[g]); a dependent column becomes zero.
__global__ void k_cgs_scale(z128 *__restrict__ B, int64_t N, int cols, int c, const z128 *__restrict__ nrm2,
                            const double *__restrict__ nrm0, int G) {
  const int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (u >= (int64_t)G * N) return;
  const int g = (int)(u / N);
  const int64_t n = u - (int64_t)g * N;
  const double nr = sqrt(nrm2[g].re);
  const double s = (nr > kDepTol * nrm0[g] && nr > 0) ? 1.0 / nr : 0.0;
  z128 *p = B + ((int64_t)g * cols + c) * N + n;
  const z128 v = *p;
  *p = zmake<z128>(v.re * s, v.im * s);
}

// nrm0[g] = sqrt(Re h[g][c]) where h holds the dots l in [0, c] of column c.
__global__ void k_take_norm(const z128 *__restrict__ h, int hs, int c, int G, double *__restrict__ nrm0) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g < G) nrm0[g] = sqrt(h[(int64_t)g * hs + c].re);
}

struct TransBuffers {
  z128 *y = nullptr, *work = nullptr, *Q = nullptr, *qss = nullptr, *dft = nullptr;
  double *part = nullptr, *dnorm = nullptr;
};

rsvdt_status device_norm(rsvdt_ctx *ctx, const z128 *y, int64_t n, double *part, double *dout, double *hout) {
  k_sqnorm_part<<<kNormBlocks, kNormThreads, 0, ctx->stream>>>(y, n, part);
  k_sqnorm_final<<<1, kNormThreads, 0, ctx->stream>>>(part, kNormBlocks, dout);
  ctx->launches += 2;
  if (!cuda_ok(ctx, cudaMemcpyAsync(hout, dout, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream), "norm copy") ||
      !cuda_ok(ctx, cudaStreamSynchronize(ctx->stream), "sync"))
    return RSVDT_ERR_CUDA;
  return RSVDT_OK;
}

// TransientRemovalEst (SourceCode/TransientRemovalEst.c:26-117) on the
// snapshot columns Q (Nw columns) for period `period`; writes the Nw/2
// initial and updated norms to the host arrays.
rsvdt_status removal_estimate(rsvdt_ctx *ctx, const TransBuffers &tb, int64_t period, double *init,
                              double *upd) {
  const int64_t N = ctx->N, Nw = ctx->Nw;
  const int H = (int)(Nw / 2);
  if (H < 1) return RSVDT_OK;
  rsvdt_status st = RSVDT_OK;
  // Initial norms: columns iw < Nw/2 of Q dft / Nw.
  const int nb = 152;
  double *part = (double *)dalloc(ctx, sizeof(double) * ((size_t)nb * H + H));
  if (!part) return set_err(ctx, RSVDT_ERR_OOM, "estimate buffers");
  double *dinit = part + (size_t)nb * H;
  k_dft_norm_part<<<dim3(nb, H), kNormThreads, 0, ctx->stream>>>(tb.Q, N, (int)Nw, ctx->dft, part);
  k_rows_norm_final<<<H, kNormThreads, 0, ctx->stream>>>(part, nb, 1.0 / (double)Nw, dinit);
  ctx->launches += 2;
  if (!cuda_ok(ctx, cudaMemcpyAsync(init, dinit, sizeof(double) * H, cudaMemcpyDeviceToHost, ctx->stream), "copy")) {
    dfree(ctx, part);
    return RSVDT_ERR_CUDA;
  }
  // Updated norms. deltaT = 2 pi / w / Ns with Ns = Nw columns (:27); the
  // first period leaves out the initial snapshot (:29, :86).
  const double deltaT = 2 * kPi / ctx->w / (double)Nw;
  const int skip = period == 1 ? 1 : 0;
  const int m = (int)Nw - skip, cols = m + 1;
  const size_t colbytes = sizeof(z128) * (size_t)N * cols;
  int G = H;
  const size_t cap_bytes = (size_t)1 << 31;  // at most 2 GiB of synthetic snapshots at a time
  if (colbytes * (size_t)G > cap_bytes) G = (int)std::max<size_t>(1, cap_bytes / colbytes);
  const int nchunks = (int)((N + kChunkRows - 1) / kChunkRows);
  z128 *B = (z128 *)dalloc(ctx, colbytes * G);
  z128 *dpart = (z128 *)dalloc(ctx, sizeof(z128) * ((size_t)G * nchunks * cols + (size_t)G * cols + (size_t)G * m));
  double *nrm0 = (double *)dalloc(ctx, sizeof(double) * (size_t)G * 2);
  if (!B || !dpart || !nrm0) {
    dfree(ctx, part);
    dfree(ctx, B);
    dfree(ctx, dpart);
    dfree(ctx, nrm0);
    return set_err(ctx, RSVDT_ERR_OOM, "estimate buffers (%zu bytes)", colbytes * G);
  }
  z128 *h = dpart + (size_t)G * nchunks * cols;
  z128 *ph = h + (size_t)G * cols;
  std::vector<z128> hph((size_t)G * m);
  double qss_norm = 0;
  st = device_norm(ctx, tb.qss, N, tb.part, tb.dnorm, &qss_norm);
  for (int g0 = 0; g0 < H && !st; g0 += G) {
    const int Gc = std::min(G, H - g0);
    for (int g = 0; g < Gc; ++g) {
      const double w = ctx->w * (double)(g0 + g);
      for (int s = 0; s < m; ++s) {
        const double th = w * (double)s * deltaT;
        hph[(size_t)g * m + s] = zmake<z128>(std::cos(th), std::sin(th));
      }
    }
    if (!cuda_ok(ctx, cudaMemcpyAsync(ph, hph.data(), sizeof(z128) * (size_t)Gc * m, cudaMemcpyHostToDevice,
                                      ctx->stream),
                 "copy")) {
      st = RSVDT_ERR_CUDA;
      break;
    }
    const int64_t tot = (int64_t)Gc * cols * N;
    k_est_build<<<grid_for(tot, 256), 256, 0, ctx->stream>>>(tb.Q, tb.qss, N, m, skip, ph, Gc, B);
    ctx->launches += 1;
    for (int c = 0; c < cols; ++c) {
      // Pass 1 (dots with l in [0, c], the last being |B_c|^2), pass 2.
      for (int pass = 0; pass < 2; ++pass) {
        const int l1 = pass == 0 ? c + 1 : c;
        if (l1 == 0) continue;
        k_cgs_dot<<<dim3(nchunks, Gc), 256, 0, ctx->stream>>>(B, N, cols, c, 0, l1, dpart);
        k_cgs_reduce<<<grid_for((int64_t)Gc * l1, 128), 128, 0, ctx->stream>>>(dpart, nchunks, l1, Gc, h);
        ctx->launches += 2;
        if (pass == 0) {
          k_take_norm<<<grid_for(Gc, 128), 128, 0, ctx->stream>>>(h, l1, c, Gc, nrm0);
          ctx->launches += 1;
        }
        if (c > 0) {
          k_cgs_update<<<grid_for((int64_t)Gc * N, 256), 256, 0, ctx->stream>>>(B, N, cols, c, h, l1, Gc);
          ctx->launches += 1;
        }
      }
      // Norm after orthogonalisation.
      k_cgs_dot<<<dim3(nchunks, Gc), 256, 0, ctx->stream>>>(B, N, cols, c, c, c + 1, dpart);
      k_cgs_reduce<<<grid_for(Gc, 128), 128, 0, ctx->stream>>>(dpart, nchunks, 1, Gc, h);
      ctx->launches += 2;
      if (c < m) {
        k_cgs_scale<<<grid_for((int64_t)Gc * N, 256), 256, 0, ctx->stream>>>(B, N, cols, c, h, nrm0, Gc);
        ctx->launches += 1;
      }
    }
    // h[g] = |residual of qss|^2.
    std::vector<z128> hr((size_t)Gc);
    if (!cuda_ok(ctx, cudaMemcpyAsync(hr.data(), h, sizeof(z128) * Gc, cudaMemcpyDeviceToHost, ctx->stream), "copy") ||
        !cuda_ok(ctx, cudaStreamSynchronize(ctx->stream), "sync")) {
      st = RSVDT_ERR_CUDA;
      break;
    }
    for (int g = 0; g < Gc; ++g) upd[g0 + g] = std::sqrt(hr[(size_t)g].re) / qss_norm;
  }
  if (!st && !cuda_ok(ctx, cudaGetLastError(), "removal estimate")) st = RSVDT_ERR_CUDA;
  if (!st && !cuda_ok(ctx, cudaStreamSynchronize(ctx->stream), "sync")) st = RSVDT_ERR_CUDA;
  dfree(ctx, part);
  dfree(ctx, B);
  dfree(ctx, dpart);
  dfree(ctx, nrm0);
  return st;
}

rsvdt_status trans_grid(rsvdt_ctx *ctx, const rsvdt_trans_params *tp, rsvdt_trans_info *info) {
  if (!ctx || !tp || !info) return RSVDT_ERR_ARG;
  if (!ctx->have_operator) return set_err(ctx, RSVDT_ERR_STATE, "the operator has not been set");
  if (tp->save_mod < 1) return set_err(ctx, RSVDT_ERR_ARG, "TransSaveMod must be positive, current value: %lld",
                                       (long long)tp->save_mod);
  if (tp->periods < 0) return set_err(ctx, RSVDT_ERR_ARG, "TransPeriods must be non-negative");
  // SourceCode/TransientRunRK4.c:39-46, applied to the grid's time step.
  const double TSS = 2 * kPi / ctx->w;
  const double deltaT = TSS / (double)ctx->Nw;
  const double dt = deltaT / std::ceil(deltaT / ctx->dt);
  std::memset(info, 0, sizeof(*info));
  info->dt = dt;
  info->Nt_period = (int64_t)std::llround(TSS / dt);
  info->rend = info->Nt_period * tp->periods;
  info->n_saved = info->rend / tp->save_mod + 1;
  return RSVDT_OK;
}

}  // namespace

extern "C" {

rsvdt_status rsvdt_trans_grid(rsvdt_ctx *ctx, const rsvdt_trans_params *tp, rsvdt_trans_info *info) {
  return trans_grid(ctx, tp, info);
}

rsvdt_status rsvdt_trans_run(rsvdt_ctx *ctx, const rsvdt_trans_params *tp, double *q, double *norms,
                             rsvdt_trans_snapshot_fn on_snapshot, rsvdt_trans_estimate_fn on_estimate, void *user,
                             rsvdt_trans_info *info) {
  rsvdt_trans_info loc;
  if (!info) info = &loc;
  TR_TRY(trans_grid(ctx, tp, info));
  NvtxRange range("rsvdt transient run");
  if (!q || !norms) return set_err(ctx, RSVDT_ERR_ARG, "null initial vector or norms");
  const int64_t N = ctx->N, Nw = ctx->Nw;
  const int64_t rend = info->rend, save_mod = tp->save_mod, Ntp = info->Nt_period;
  const int64_t Rd = Ntp / Nw;  // Nt_saved_delta (:44)
  const bool est = tp->removal_est != 0;
  const bool show = ctx->par.Display >= 1;
  for (int64_t i = 0; i < info->n_saved; ++i) norms[i] = 0;

  TransBuffers tb;
  const size_t nbytes = sizeof(z128) * (size_t)N;
  tb.y = (z128 *)dalloc(ctx, nbytes * 6);
  tb.part = (double *)dalloc(ctx, sizeof(double) * (kNormBlocks + 1));
  if (est) {
    tb.Q = (z128 *)dalloc(ctx, nbytes * (size_t)(Nw + 1));
  }
  double *hbuf = nullptr;
  if (cudaMallocHost(&hbuf, sizeof(double) * 2 * (size_t)N + 64) != cudaSuccess) {
    cudaGetLastError();
    hbuf = nullptr;
  }
  auto cleanup = [&]() {
    dfree(ctx, tb.y);
    dfree(ctx, tb.part);
    dfree(ctx, tb.Q);
    if (hbuf) cudaFreeHost(hbuf);
  };
  if (!tb.y || !tb.part || (est && !tb.Q) || !hbuf) {
    cleanup();
    return set_err(ctx, RSVDT_ERR_OOM, "transient-run buffers");
  }
  tb.work = tb.y + N;
  tb.dnorm = tb.part + kNormBlocks;
  if (est) tb.qss = tb.Q + (size_t)Nw * N;
  double *hq = hbuf + 8;  // N complex values (pinned)
  double *hnorm = hbuf;
  cudaGraphExec_t graph = nullptr;
  rsvdt_status st = RSVDT_OK;
  auto fail = [&](rsvdt_status s) {
    if (graph) cudaGraphExecDestroy(graph);
    cleanup();
    return s;
  };

  std::memcpy(hq, q, nbytes);
  if (!cuda_ok(ctx, cudaMemcpyAsync(tb.y, hq, nbytes, cudaMemcpyHostToDevice, ctx->stream), "upload") ||
      !cuda_ok(ctx, cudaMemsetAsync(tb.work + 3 * N, 0, nbytes * 2, ctx->stream), "memset"))
    return fail(RSVDT_ERR_CUDA);
  if (show)
    printf("Total integration time = %g = %d x %g with dt = %g\n", info->dt * (double)rend, (int)tp->periods,
           2 * kPi / ctx->w, info->dt);
  // The first saved snapshot is the initial vector (:101-120).
  if ((st = device_norm(ctx, tb.y, N, tb.part, tb.dnorm, hnorm))) return fail(st);
  norms[0] = *hnorm;
  info->last_norm = *hnorm;
  if (show) printf("Norm of the initial snapshot: %f @ t = %d\n", *hnorm, 0);
  if (est) {
    // qss = -q0; column 0 = q0 (:96-114).
    k_scaled_copy<<<grid_for(N, 256), 256, 0, ctx->stream>>>(tb.y, N, -1.0, tb.qss);
    ctx->launches += 1;
    if (!cuda_ok(ctx, cudaMemcpyAsync(tb.Q, tb.y, nbytes, cudaMemcpyDeviceToDevice, ctx->stream), "copy"))
      return fail(RSVDT_ERR_CUDA);
  }
  if (tp->save && on_snapshot && on_snapshot(user, 0, q, N) != 0)
    return fail(set_err(ctx, RSVDT_ERR_IO, "snapshot callback failed at pos 0"));

  std::vector<double> init((size_t)std::max<int64_t>(1, Nw / 2)), upd(init.size());
  int64_t i = 0;
  info->stop = RSVDT_TRANS_DONE;
  // Time stepping (:128-186).
  while (i < rend) {
    int64_t nxt = std::min(rend, (i / save_mod + 1) * save_mod);
    if (est) nxt = std::min(nxt, (i / Rd + 1) * Rd);
    if ((st = launch_trans_steps(ctx, info->dt, tb.y, tb.work, nxt - i, &graph))) return fail(st);
    i = nxt;
    info->steps = i;
    if (i % save_mod == 0) {
      const int64_t pos = i / save_mod;
      if ((st = device_norm(ctx, tb.y, N, tb.part, tb.dnorm, hnorm))) return fail(st);
      const double nr = *hnorm;
      info->last_norm = nr;
      if (std::isnan(nr)) {
        if (show) printf("Stopped! The norm of the last snapshot is NAN!\n");
        info->stop = RSVDT_TRANS_NAN;
        break;
      }
      if (nr > tp->div_val) {
        if (show)
          printf("Diverged! The norm of the last snapshot = %g exceeds the divergence threshold = %g\n", nr,
                 tp->div_val);
        info->stop = RSVDT_TRANS_DIVERGED;
        break;
      }
      if (nr < tp->con_val) {
        if (show)
          printf("Converged! The norm of the last snapshot = %g is smaller than the convergence threshold = %g\n",
                 nr, tp->con_val);
        info->stop = RSVDT_TRANS_CONVERGED;
        break;
      }
      if (tp->save && on_snapshot) {
        if (!cuda_ok(ctx, cudaMemcpyAsync(hq, tb.y, nbytes, cudaMemcpyDeviceToHost, ctx->stream), "download") ||
            !cuda_ok(ctx, cudaStreamSynchronize(ctx->stream), "sync"))
          return fail(RSVDT_ERR_CUDA);
        if (on_snapshot(user, pos, hq, N) != 0)
          return fail(set_err(ctx, RSVDT_ERR_IO, "snapshot callback failed at pos %lld", (long long)pos));
      }
      if (show) printf("Norm of the snapshot: %f @ t = %f\n", nr, (double)i * info->dt);
      norms[pos] = nr;
    }
    if (est && i % Rd == 0) {
      const int64_t pos = (i / Rd) % Nw;
      if (pos == 0) {
        if ((st = removal_estimate(ctx, tb, i / Ntp, init.data(), upd.data()))) return fail(st);
        if (show)
          for (int64_t iw = 0; iw < Nw / 2; ++iw)
            printf("**** Norm of the ratio norm(qt_up)/norm(qs): %g @ w = %g ****\n", upd[(size_t)iw],
                   ctx->w * (double)iw);
        if (on_estimate && on_estimate(user, i / Ntp, init.data(), upd.data(), Nw / 2) != 0)
          return fail(set_err(ctx, RSVDT_ERR_IO, "estimate callback failed at period %lld", (long long)(i / Ntp)));
      }
      if (!cuda_ok(ctx, cudaMemcpyAsync(tb.Q + (size_t)pos * N, tb.y, nbytes, cudaMemcpyDeviceToDevice, ctx->stream),
                   "copy"))
        return fail(RSVDT_ERR_CUDA);
    }
  }
  // Last snapshot (:207-209).
  if (!cuda_ok(ctx, cudaMemcpyAsync(hq, tb.y, nbytes, cudaMemcpyDeviceToHost, ctx->stream), "download") ||
      !cuda_ok(ctx, cudaStreamSynchronize(ctx->stream), "sync"))
    return fail(RSVDT_ERR_CUDA);
  std::memcpy(q, hq, nbytes);
  if (graph) cudaGraphExecDestroy(graph);
  graph = nullptr;
  cleanup();
  return RSVDT_OK;
}

}  // extern "C"
