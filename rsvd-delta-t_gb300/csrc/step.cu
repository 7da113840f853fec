// Forced RK4 time stepping of all k test vectors at once.
//
// One RK4 step (SourceCode/TSRK4.c:18-47) is four stage kernels over the
// k-interleaved state y[n][k]. Each stage is a sparse product of A (or the
// explicitly stored A^H) with the stage input, gathered once per nonzero for
// all k test vectors, fused with everything the reference does between the
// products:
//   stage 1: k1 = A y + F3_old; F2 = F_hat*idft[:,j2]; F3 = F_hat*idft[:,j3]
//            z  = y + dt/2 k1;  acc = y + dt/6 k1
//   stage 2: k2 = A z + F2;     z' = y + dt/2 k2;  acc += (dt/6*2) k2
//   stage 3: k3 = A z' + F2;    z  = y + dt k3;    acc += (dt/6*2) k3
//   stage 4: k4 = A z + F3;     y  = acc + dt/6 k4; sample y into the ring
// acc accumulates the update in the reference's order (y += dt/6 k1;
// y += dt/6*2 k2; ...). The forcing synthesis (SourceCode/CreateForcingOnFly.c)
// reads each row's Fourier coefficients F_hat[n][iw][k] once per step for
// both forcing times. The step index lives in device memory (two slots, so
// that no kernel reads the slot it writes), which lets a fixed CUDA graph of
// G steps be replayed for the whole integration.
#include <cstdarg>

#include "common.cuh"

namespace rsvdt {

template <class Z>
struct StepArgs {
  int64_t N;
  int K, Nw, dir;
  int64_t two_ns, R, Nt, Nstore;
  // Operator (A for the direct run, A^H for the adjoint run).
  const int32_t *__restrict__ rowptr;
  const int32_t *__restrict__ col;
  const Z *__restrict__ val;
  int bs;  // 0: CSR; >0: block CSR with bs x bs blocks
  const Z *__restrict__ Fh;   // [n][iw][k], nullptr when unforced
  const Z *__restrict__ tab;  // [2Ns][Nw]
  Z *y, *zA, *zB, *acc, *F2, *F3, *ring;
  typename real_of<Z>::type dt, dt_2, dt_6, dt_62;  // dt, dt/2, dt/6, dt/6*2
  int64_t *step;
};

// Half-step forcing indices of step i (SourceCode/TSRK4.c:21-26). For the
// adjoint, fmod(1e6*Ns - 1 - m, 2Ns) equals (-1 - m) mod 2Ns because 1e6*Ns
// is a multiple of 2Ns.
__device__ __forceinline__ void step_idx(int dir, int64_t i, int64_t two_ns, int64_t &j2,
                                         int64_t &j3) {
  if (dir) {
    j2 = (2 * (i - 1) + 1) % two_ns;
    j3 = (2 * (i - 1) + 2) % two_ns;
  } else {
    j2 = ((-(2 * (i - 1) + 1)) % two_ns + two_ns) % two_ns;
    j3 = ((-(2 * (i - 1) + 2)) % two_ns + two_ns) % two_ns;
  }
}

// Ring slot of the sample taken after step i, or -1
// (SourceCode/SaveSnapshots.c:19-29).
__device__ __forceinline__ int64_t ring_slot(int dir, int64_t i, int64_t Nt, int64_t R,
                                             int64_t Nstore) {
  if (i <= Nt) return -1;
  int64_t pos = i - Nt;
  if (pos % R != 0) return -1;
  pos = (pos / R - 1) % Nstore;
  if (!dir) pos = Nstore - 1 - pos;
  return pos % Nstore;
}

// Sparse row product: acc += sum_j A[n,j] * x[j][kc].
template <class Z>
__device__ __forceinline__ void row_product(const StepArgs<Z> &P, int64_t n, int kc, const Z *x,
                                            Z &acc) {
  const int K = P.K;
  if (P.bs == 0) {
    int32_t b = __ldg(P.rowptr + n), e = __ldg(P.rowptr + n + 1);
    for (int32_t j = b; j < e; ++j) {
      const Z a = P.val[j];
      const Z v = x[(int64_t)__ldg(P.col + j) * K + kc];
      zmac(acc, a, v);
    }
  } else {
    const int bs = P.bs;
    const int64_t br = n / bs;
    const int r = (int)(n - br * bs);
    int32_t b = __ldg(P.rowptr + br), e = __ldg(P.rowptr + br + 1);
    for (int32_t j = b; j < e; ++j) {
      const int64_t c0 = (int64_t)__ldg(P.col + j) * bs;
      const Z *blkrow = P.val + ((int64_t)j * bs + r) * bs;
      for (int c = 0; c < bs; ++c) {
        const Z a = blkrow[c];
        const Z v = x[(c0 + c) * K + kc];
        zmac(acc, a, v);
      }
    }
  }
}

template <class Z, int S>
__global__ void __launch_bounds__(256) k_stage(const StepArgs<Z> P) {
  using Rl = typename real_of<Z>::type;
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t NK = P.N * P.K;
  int64_t i = (S == 1) ? P.step[0] : P.step[1];
  if (t >= NK) return;
  const int64_t n = t / P.K;
  const int kc = (int)(t - n * P.K);
  if (S == 1 && t == 0) P.step[1] = i;

  // Gathered input and added forcing of this stage.
  const Z *x = (S == 1) ? P.y : (S == 2) ? P.zA : (S == 3) ? P.zB : P.zA;
  Z k = (S == 1 || S == 4) ? P.F3[t] : P.F2[t];
  row_product(P, n, kc, x, k);
  const Z yv = P.y[t];

  if (S == 1) {
    Z f2 = zmake<Z>(0, 0), f3 = zmake<Z>(0, 0);
    if (P.Fh) {
      int64_t j2, j3;
      step_idx(P.dir, i, P.two_ns, j2, j3);
      const Z *e2 = P.tab + j2 * P.Nw;
      const Z *e3 = P.tab + j3 * P.Nw;
      const Z *c = P.Fh + n * (int64_t)P.Nw * P.K + kc;
      for (int iw = 0; iw < P.Nw; ++iw) {
        const Z cv = c[(int64_t)iw * P.K];
        zmac(f2, cv, e2[iw]);
        zmac(f3, cv, e3[iw]);
      }
    }
    P.F2[t] = f2;
    P.F3[t] = f3;
    P.zA[t] = zaxpy(P.dt_2, k, yv);
    P.acc[t] = zaxpy(P.dt_6, k, yv);
  } else if (S == 2) {
    P.zB[t] = zaxpy(P.dt_2, k, yv);
    P.acc[t] = zaxpy(P.dt_62, k, P.acc[t]);
  } else if (S == 3) {
    P.zA[t] = zaxpy(P.dt, k, yv);
    P.acc[t] = zaxpy(P.dt_62, k, P.acc[t]);
  } else {
    const Z ynew = zaxpy(P.dt_6, k, P.acc[t]);
    P.y[t] = ynew;
    const int64_t p = P.ring ? ring_slot(P.dir, i, P.Nt, P.R, P.Nstore) : -1;
    if (p >= 0) P.ring[p * NK + t] = ynew;
    if (t == 0) P.step[0] = i + 1;
  }
  (void)sizeof(Rl);
}

__global__ void k_set_step(int64_t *step, int64_t i) {
  step[0] = i;
  step[1] = i;
}

// y = 0 and F3 = F_hat * idft[:, 0] (SourceCode/TSActionRK4.c:91,103).
template <class Z>
__global__ void k_forcing_init(const StepArgs<Z> P) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= P.N * P.K) return;
  const int64_t n = t / P.K;
  const int kc = (int)(t - n * P.K);
  Z f = zmake<Z>(0, 0);
  const Z *c = P.Fh + n * (int64_t)P.Nw * P.K + kc;
  for (int iw = 0; iw < P.Nw; ++iw) zmac(f, c[(int64_t)iw * P.K], P.tab[iw]);
  P.F3[t] = f;
  P.y[t] = zmake<Z>(0, 0);
}

template <class Z>
static StepArgs<Z> make_args(rsvdt_ctx *ctx, int dir, bool forced) {
  StepArgs<Z> P;
  P.N = ctx->N;
  P.K = (int)ctx->K;
  P.Nw = (int)ctx->Nw_eff;
  P.dir = dir;
  P.two_ns = 2 * ctx->Ns;
  P.R = ctx->R;
  P.Nt = ctx->Nt;
  P.Nstore = ctx->Nstore;
  const bool c64 = sizeof(Z) == sizeof(z64);
  if (ctx->BA.present) {
    const DevBCSR &M = dir ? ctx->BA : ctx->BAH;
    P.rowptr = M.browptr;
    P.col = M.bcol;
    P.val = (const Z *)(c64 ? (void *)M.val32 : (void *)M.val);
    P.bs = M.bs;
  } else {
    const DevCSR &M = dir ? ctx->A : ctx->AH;
    P.rowptr = M.rowptr;
    P.col = M.col;
    P.val = (const Z *)(c64 ? (void *)M.val32 : (void *)M.val);
    P.bs = 0;
  }
  P.Fh = forced ? (const Z *)ctx->Fh : nullptr;
  P.tab = (const Z *)(c64 ? (void *)ctx->tab32 : (void *)ctx->tab);
  P.y = (Z *)ctx->y;
  P.zA = (Z *)ctx->zA;
  P.zB = (Z *)ctx->zB;
  P.acc = (Z *)ctx->acc;
  P.F2 = (Z *)ctx->F2;
  P.F3 = (Z *)ctx->F3;
  P.ring = (Z *)ctx->ring;
  using Rl = typename real_of<Z>::type;
  const double dt = ctx->dt;
  P.dt = (Rl)dt;
  P.dt_2 = (Rl)(dt / 2);
  P.dt_6 = (Rl)(dt / 6);
  P.dt_62 = (Rl)(dt / 6 * 2);
  P.step = ctx->d_step;
  return P;
}

template <class Z>
static void enqueue_step(rsvdt_ctx *ctx, const StepArgs<Z> &P) {
  const int th = 256;
  const int g = grid_for(P.N * P.K, th);
  k_stage<Z, 1><<<g, th, 0, ctx->stream>>>(P);
  k_stage<Z, 2><<<g, th, 0, ctx->stream>>>(P);
  k_stage<Z, 3><<<g, th, 0, ctx->stream>>>(P);
  k_stage<Z, 4><<<g, th, 0, ctx->stream>>>(P);
}

rsvdt_status launch_forcing_init(rsvdt_ctx *ctx, int dir, int prec) {
  const int th = 256;
  if (prec == RSVDT_PREC_C64) {
    auto P = make_args<z64>(ctx, dir, true);
    k_forcing_init<z64><<<grid_for(P.N * P.K, th), th, 0, ctx->stream>>>(P);
  } else {
    auto P = make_args<z128>(ctx, dir, true);
    k_forcing_init<z128><<<grid_for(P.N * P.K, th), th, 0, ctx->stream>>>(P);
  }
  ctx->launches += 1;
  if (!cuda_ok(ctx, cudaGetLastError(), "forcing init")) return RSVDT_ERR_CUDA;
  return RSVDT_OK;
}

static const int64_t kGraphSteps = 16;

template <class Z>
static rsvdt_status run_steps_t(rsvdt_ctx *ctx, int dir, int64_t i0, int64_t nsteps) {
  auto P = make_args<Z>(ctx, dir, true);
  k_set_step<<<1, 1, 0, ctx->stream>>>(ctx->d_step, i0);
  ctx->launches += 1;
  int64_t full = nsteps / kGraphSteps, rest = nsteps % kGraphSteps;
  if (full > 0) {
    cudaGraphExec_t &ge = ctx->step_graph[dir ? 1 : 0];
    if (!ge) {
      cudaGraph_t g;
      if (!cuda_ok(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal),
                   "begin capture"))
        return RSVDT_ERR_CUDA;
      for (int64_t s = 0; s < kGraphSteps; ++s) enqueue_step(ctx, P);
      if (!cuda_ok(ctx, cudaStreamEndCapture(ctx->stream, &g), "end capture")) return RSVDT_ERR_CUDA;
      if (!cuda_ok(ctx, cudaGraphInstantiate(&ge, g, 0), "graph instantiate")) return RSVDT_ERR_CUDA;
      cudaGraphDestroy(g);
    }
    for (int64_t c = 0; c < full; ++c)
      if (!cuda_ok(ctx, cudaGraphLaunch(ge, ctx->stream), "graph launch")) return RSVDT_ERR_CUDA;
    ctx->launches += full * kGraphSteps * 4;
  }
  for (int64_t s = 0; s < rest; ++s) enqueue_step(ctx, P);
  ctx->launches += rest * 4;
  if (!cuda_ok(ctx, cudaGetLastError(), "rk4 steps")) return RSVDT_ERR_CUDA;
  return RSVDT_OK;
}

rsvdt_status run_steps(rsvdt_ctx *ctx, int dir, int prec, int64_t i0, int64_t nsteps, bool) {
  if (prec == RSVDT_PREC_C64) return run_steps_t<z64>(ctx, dir, i0, nsteps);
  return run_steps_t<z128>(ctx, dir, i0, nsteps);
}

// Steps launched one stage at a time with CUDA events between the stage
// launches on the context's stream; stage_ms[s] accumulates the duration
// of stage s+1 over the steps.
template <class Z>
static rsvdt_status profile_steps_t(rsvdt_ctx *ctx, int dir, int64_t i0, int64_t nsteps,
                                    double *stage_ms) {
  auto P = make_args<Z>(ctx, dir, true);
  const int th = 256;
  const int g = grid_for(P.N * P.K, th);
  cudaEvent_t ev[5];
  for (auto &e : ev)
    if (!cuda_ok(ctx, cudaEventCreate(&e), "event create")) return RSVDT_ERR_CUDA;
  k_set_step<<<1, 1, 0, ctx->stream>>>(ctx->d_step, i0);
  ctx->launches += 1;
  for (int s = 0; s < 4; ++s) stage_ms[s] = 0;
  rsvdt_status st = RSVDT_OK;
  for (int64_t n = 0; n < nsteps && st == RSVDT_OK; ++n) {
    cudaEventRecord(ev[0], ctx->stream);
    k_stage<Z, 1><<<g, th, 0, ctx->stream>>>(P);
    cudaEventRecord(ev[1], ctx->stream);
    k_stage<Z, 2><<<g, th, 0, ctx->stream>>>(P);
    cudaEventRecord(ev[2], ctx->stream);
    k_stage<Z, 3><<<g, th, 0, ctx->stream>>>(P);
    cudaEventRecord(ev[3], ctx->stream);
    k_stage<Z, 4><<<g, th, 0, ctx->stream>>>(P);
    cudaEventRecord(ev[4], ctx->stream);
    ctx->launches += 4;
    if (!cuda_ok(ctx, cudaEventSynchronize(ev[4]), "event sync")) {
      st = RSVDT_ERR_CUDA;
      break;
    }
    for (int s = 0; s < 4; ++s) {
      float ms = 0;
      cudaEventElapsedTime(&ms, ev[s], ev[s + 1]);
      stage_ms[s] += ms;
    }
  }
  for (auto &e : ev) cudaEventDestroy(e);
  if (st == RSVDT_OK && !cuda_ok(ctx, cudaGetLastError(), "profile steps")) st = RSVDT_ERR_CUDA;
  return st;
}

rsvdt_status profile_steps(rsvdt_ctx *ctx, int dir, int prec, int64_t i0, int64_t nsteps,
                           double *stage_ms) {
  if (prec == RSVDT_PREC_C64) return profile_steps_t<z64>(ctx, dir, i0, nsteps, stage_ms);
  return profile_steps_t<z128>(ctx, dir, i0, nsteps, stage_ms);
}

// DFT of the sampled period (SourceCode/DFT.c:26-38), FP64 sums:
// out[n][iw][k] = ResRatio * sum_p ring[p][n][k] * dft[p][iw].
template <class Z>
__global__ void __launch_bounds__(256) k_dft(const Z *__restrict__ ring,
                                             const z128 *__restrict__ dft, int64_t N, int K,
                                             int Nw, int Nwe, double R, z128 *__restrict__ out,
                                             int32_t *flags) {
  const int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t total = N * (int64_t)Nwe * K;
  if (u >= total) return;
  const int kc = (int)(u % K);
  const int iw = (int)((u / K) % Nwe);
  const int64_t n = u / ((int64_t)K * Nwe);
  const int64_t NK = N * K;
  z128 s = zmake<z128>(0, 0);
  const Z *src = ring + n * K + kc;
  for (int p = 0; p < Nw; ++p) {
    const Z v = src[(int64_t)p * NK];
    z128 vd = zmake<z128>((double)v.re, (double)v.im);
    zmac(s, vd, dft[(int64_t)iw * Nw + p]);
  }
  s.re *= R;
  s.im *= R;
  if (!isfinite(s.re) || !isfinite(s.im)) atomicOr(flags, 1);
  out[u] = s;
}

rsvdt_status launch_dft(rsvdt_ctx *ctx, int prec, z128 *out) {
  const int th = 256;
  const int64_t total = ctx->N * ctx->Nw_eff * ctx->K;
  if (prec == RSVDT_PREC_C64)
    k_dft<z64><<<grid_for(total, th), th, 0, ctx->stream>>>(
        (const z64 *)ctx->ring, ctx->dft, ctx->N, (int)ctx->K, (int)ctx->Nw, (int)ctx->Nw_eff,
        (double)ctx->R, out, ctx->d_flags);
  else
    k_dft<z128><<<grid_for(total, th), th, 0, ctx->stream>>>(
        (const z128 *)ctx->ring, ctx->dft, ctx->N, (int)ctx->K, (int)ctx->Nw, (int)ctx->Nw_eff,
        (double)ctx->R, out, ctx->d_flags);
  ctx->launches += 1;
  if (!cuda_ok(ctx, cudaGetLastError(), "dft")) return RSVDT_ERR_CUDA;
  return RSVDT_OK;
}

// Unforced RK4 (SourceCode/TSTransRK4.c:15-36) on ncols independent columns
// stored [n][col] in `cols`, for the transient-removal propagator
// (SourceCode/TSExpADeltaT.c:25-34). Uses the stage kernels with no forcing
// and a zero added vector; work vectors are taken from the scratch buffer.
rsvdt_status launch_unforced_steps(rsvdt_ctx *ctx, int dir, z128 *cols, int64_t ncols,
                                   int64_t nsteps) {
  const int64_t NC = ctx->N * ncols;
  const size_t need = sizeof(z128) * NC * 5;
  if (ctx->scratch_bytes < need) {
    dfree(ctx, ctx->scratch);
    ctx->scratch = dalloc(ctx, need);
    ctx->scratch_bytes = ctx->scratch ? need : 0;
    if (!ctx->scratch) return set_err(ctx, RSVDT_ERR_OOM, "scratch allocation of %zu bytes failed", need);
  }
  z128 *w = (z128 *)ctx->scratch;
  auto P = make_args<z128>(ctx, dir, false);
  P.K = (int)ncols;
  P.y = cols;
  P.zA = w;
  P.zB = w + NC;
  P.acc = w + 2 * NC;
  P.F2 = w + 3 * NC;
  P.F3 = w + 4 * NC;
  P.ring = nullptr;
  if (!cuda_ok(ctx, cudaMemsetAsync(P.F2, 0, sizeof(z128) * NC * 2, ctx->stream), "memset"))
    return RSVDT_ERR_CUDA;
  k_set_step<<<1, 1, 0, ctx->stream>>>(ctx->d_step, 1);
  ctx->launches += 1;
  for (int64_t s = 0; s < nsteps; ++s) enqueue_step(ctx, P);
  ctx->launches += 4 * nsteps;
  if (!cuda_ok(ctx, cudaGetLastError(), "unforced steps")) return RSVDT_ERR_CUDA;
  return RSVDT_OK;
}

}  // namespace rsvdt
