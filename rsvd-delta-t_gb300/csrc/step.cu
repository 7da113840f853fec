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
// y += dt/6*2 k2; ...). The step index lives in device memory (two slots, so
// that no kernel reads the slot it writes), which lets a fixed CUDA graph of
// G steps be replayed for the whole integration.
//
// Forcing synthesis (SourceCode/CreateForcingOnFly.c:17-19) reads the
// running action's Fourier coefficients once per step for both forcing
// times. They are staged per action as frequency slabs Fh[s][n][k], so that
// a warp's loads are contiguous. For a complex operator with an even number
// of frequencies the slabs hold symmetric pairs: slab 0 = c_0, slabs
// 1..H-1 = c_f + c_{-f}, slabs H..2H-2 = i (c_f - c_{-f}), slab Nw-1 =
// c_{-H} (H = Nw/2), since c_f e_f + c_{-f} conj(e_f) = (c_f + c_{-f}) Re e_f
// + i (c_f - c_{-f}) Im e_f. A pair then costs two complex-by-real
// multiply-adds instead of two complex ones: half the FP64 work of the
// synthesis, the largest FP64 consumer after the sparse products. The
// negative frequency's phasor is taken as the exact conjugate of the
// positive one (the reference evaluates it from a much larger argument,
// which carries its own rounding).
//
// Stage kernel families: k_stage (one thread per row and test vector, any
// CSR or block-CSR operator, any k); for 5x5 block-CSR with k a
// compile-time constant, k_bstage (complex64: one lane per block row and
// group of test vectors, which reads every gathered k-vector row as one
// contiguous 16-byte-per-lane access, for HBM-bound stages) and k_rstage
// (complex128: one thread per row with all k test vectors in registers,
// full warps for the FP64-bound stages); for small problems and batches,
// k_stage_batched (lanes split a row's nonzeros and slabs) and
// k_stage_batched_pair (two complex64 test vectors per lane). Stage
// kernels are launched with programmatic dependent launch. This file also
// holds the DFT of the sampled period (radix-2 FFT for Nw = 8..64).
#include <algorithm>
#include <atomic>
#include <cstdarg>
#include <cstring>

#include "common.cuh"

namespace rsvdt {

template <class Z>
struct StepArgs {
  int64_t N;
  int K, Nw, dir, pair;
  int64_t two_ns, R, Nt, Nstore;
  // Operator (A for the direct run, A^H for the adjoint run).
  const int32_t *__restrict__ rowptr;
  const int32_t *__restrict__ col;
  const Z *__restrict__ val;
  int bs;                     // 0: CSR; >0: block CSR with bs x bs blocks
  int bstride;                // values per block in `val` (bs*bs; 26 for 5x5 complex64)
  const Z *__restrict__ Fh;   // [slab][n][k], nullptr when unforced
  const Z *__restrict__ tab;  // [2Ns][Nw]
  Z *y, *zA, *zB, *acc, *F2, *F3, *ring;
  typename real_of<Z>::type dt, dt_2, dt_6, dt_62;  // dt, dt/2, dt/6, dt/6*2
  int64_t *step;
  int64_t rend;  // last step of this problem's action (batched stepping)
  // Rows [row0, row1) of the one-thread-per-row complex128 stage kernel
  // (k_rstage); 0 and N except when stage 4 of a step runs in row slabs.
  int64_t row0, row1;
  // Forcing block (complex64 block-row stages only): the half-step forcings
  // of a block of steps, synthesised ahead by k_forcing_block, slot 2s at
  // the half step and 2s+1 at the end of the block's step s; nullptr when
  // stage 1 synthesises each step's forcing itself.
  Z *fblk;
};

// Programmatic dependent launch: a stage kernel is launched while the one
// before it is still running (its launch latency overlaps that kernel's
// work), and waits here until that kernel has completed and its writes are
// visible, before it touches any state. Without a programmatic dependency
// (an ordinary launch) the wait returns at once.
__device__ __forceinline__ void pdl_wait_and_release() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Launches kernel k with the programmatic-serialization attribute on st.
template <typename... KArgs, typename... Args>
static void launch_pdl(void (*k)(KArgs...), int grid, int threads, size_t smem, cudaStream_t st, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3((unsigned)threads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, k, args...);
}

// Index checks of the debug build (RSVDT_DEBUG): a failed check sets its
// site's bit in g_index_faults and skips the access; the host reads and
// clears the word after every action (debug_index_status). Sites: 0 = CSR
// column, 1 = block column, 2 = ring slot. In the release build the checks
// compile to nothing.
#ifdef RSVDT_DEBUG
__device__ unsigned int g_index_faults;
#define RSVDT_CHECK_INDEX(cond, site) ((cond) || (atomicOr(&g_index_faults, 1u << (site)), false))
#else
#define RSVDT_CHECK_INDEX(cond, site) true
#endif

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

// Real weight of pair slab s (1 <= s <= 2H-2) at phasor row e.
template <class Z>
__device__ __forceinline__ typename real_of<Z>::type pair_weight(const Z *e, int s, int H) {
  return s < H ? e[s].re : e[s - H + 1].im;
}

// Forcing at one time for one (row, test vector) from the slabs.
template <class Z>
__device__ __forceinline__ Z forcing_at(const StepArgs<Z> &P, int64_t n, int kc, const Z *e) {
  Z f = zmake<Z>(0, 0);
  const int64_t NK = P.N * P.K;
  const Z *c = P.Fh + n * P.K + kc;
  if (P.pair) {
    const int H = P.Nw / 2;
    zmac(f, c[0], e[0]);
    for (int s = 1; s <= 2 * H - 2; ++s) {
      const auto w = pair_weight(e, s, H);
      const Z v = c[(int64_t)s * NK];
      f.re = fma(w, v.re, f.re);
      f.im = fma(w, v.im, f.im);
    }
    zmac(f, c[(int64_t)(P.Nw - 1) * NK], e[H]);
  } else {
    for (int s = 0; s < P.Nw; ++s) zmac(f, c[(int64_t)s * NK], e[s]);
  }
  return f;
}

// Forcing at both times of a step (phasor rows e2, e3) for one (row, test
// vector), in one pass over the slabs: lane fsub of an FS-lane group takes
// slabs fsub, fsub + FS, ... (FS = 1: all of them); the pair slabs run in
// two branch-free loops (weights Re e_f, then Im e_f), the two complex
// slabs are added by the lanes that own them.
template <class Z>
__device__ __forceinline__ void forcing2(const StepArgs<Z> &P, int64_t n, int kc, const Z *e2, const Z *e3,
                                         int fsub, int FS, Z &f2, Z &f3) {
  const int64_t NK = P.N * P.K;
  const Z *c = P.Fh + n * P.K + kc;
  f2 = zmake<Z>(0, 0);
  f3 = zmake<Z>(0, 0);
  if (!P.pair) {
#pragma unroll 4
    for (int s = fsub; s < P.Nw; s += FS) {
      const Z v = c[(int64_t)s * NK];
      zmac(f2, v, e2[s]);
      zmac(f3, v, e3[s]);
    }
    return;
  }
  const int H = P.Nw / 2, last = P.Nw - 1;
  if (fsub == 0) {
    const Z v = c[0];
    zmac(f2, v, e2[0]);
    zmac(f3, v, e3[0]);
  }
  // Slabs 1..H-1: c_f + c_{-f}, weight Re e_f (f = s).
  int s = fsub == 0 ? FS : fsub;
#pragma unroll 4
  for (; s < H; s += FS) {
    const Z v = c[(int64_t)s * NK];
    const auto w2 = e2[s].re, w3 = e3[s].re;
    f2.re = fma(w2, v.re, f2.re);
    f2.im = fma(w2, v.im, f2.im);
    f3.re = fma(w3, v.re, f3.re);
    f3.im = fma(w3, v.im, f3.im);
  }
  // Slabs H..2H-2: i (c_f - c_{-f}), weight Im e_f (f = s - H + 1).
#pragma unroll 4
  for (; s < last; s += FS) {
    const Z v = c[(int64_t)s * NK];
    const auto w2 = e2[s - H + 1].im, w3 = e3[s - H + 1].im;
    f2.re = fma(w2, v.re, f2.re);
    f2.im = fma(w2, v.im, f2.im);
    f3.re = fma(w3, v.re, f3.re);
    f3.im = fma(w3, v.im, f3.im);
  }
  if (s == last) {
    const Z v = c[(int64_t)last * NK];
    zmac(f2, v, e2[H]);
    zmac(f3, v, e3[H]);
  }
}

// Sparse row product: acc += sum_j A[n,j] * x[j][kc].
template <class Z>
__device__ __forceinline__ void row_product(const StepArgs<Z> &P, int64_t n, int kc, const Z *x,
                                            Z &acc) {
  const int K = P.K;
  if (P.bs == 0) {
    int32_t b = __ldg(P.rowptr + n), e = __ldg(P.rowptr + n + 1);
    for (int32_t j = b; j < e; ++j) {
      const int32_t cj = __ldg(P.col + j);
      if (!RSVDT_CHECK_INDEX(cj >= 0 && cj < P.N, 0)) continue;
      const Z a = P.val[j];
      const Z v = x[(int64_t)cj * K + kc];
      zmac(acc, a, v);
    }
  } else {
    const int bs = P.bs;
    const int64_t br = n / bs;
    const int r = (int)(n - br * bs);
    int32_t b = __ldg(P.rowptr + br), e = __ldg(P.rowptr + br + 1);
    for (int32_t j = b; j < e; ++j) {
      const int32_t cb = __ldg(P.col + j);
      if (!RSVDT_CHECK_INDEX(cb >= 0 && cb < P.N / bs, 1)) continue;
      const int64_t c0 = (int64_t)cb * bs;
      const Z *blkrow = P.val + (int64_t)j * P.bstride + r * bs;
      for (int c = 0; c < bs; ++c) {
        const Z a = blkrow[c];
        const Z v = x[(c0 + c) * K + kc];
        zmac(acc, a, v);
      }
    }
  }
}

// ------------------------------------------------ generic stage kernels

template <class Z, int S>
__global__ void __launch_bounds__(256) k_stage(const StepArgs<Z> P) {
  pdl_wait_and_release();
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
      forcing2(P, n, kc, P.tab + j2 * P.Nw, P.tab + j3 * P.Nw, 0, 1, f2, f3);
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
    if (p >= 0 && RSVDT_CHECK_INDEX(p < P.Nstore, 2)) P.ring[p * NK + t] = ynew;
    if (t == 0) P.step[0] = i + 1;
  }
}

// --------------------------------- 5x5 block-CSR row kernels (k in registers)

// KP consecutive complex values at a 16-byte aligned address.
template <class Z, int KP>
__device__ __forceinline__ void ld_chunk(const Z *p, Z (&v)[KP]) {
  if constexpr (sizeof(Z) == 8 && KP == 2) {
    const float4 t = *reinterpret_cast<const float4 *>(p);
    v[0] = zmake<Z>(t.x, t.y);
    v[1] = zmake<Z>(t.z, t.w);
  } else {
#pragma unroll
    for (int i = 0; i < KP; ++i) v[i] = p[i];
  }
}

template <class Z, int KP>
__device__ __forceinline__ void ldg_chunk(const Z *p, Z (&v)[KP]) {
  if constexpr (sizeof(Z) == 8 && KP == 2) {
    const float4 t = __ldg(reinterpret_cast<const float4 *>(p));
    v[0] = zmake<Z>(t.x, t.y);
    v[1] = zmake<Z>(t.z, t.w);
  } else if constexpr (sizeof(Z) == 16) {
#pragma unroll
    for (int i = 0; i < KP; ++i) {
      const double2 t = __ldg(reinterpret_cast<const double2 *>(p) + i);
      v[i] = zmake<Z>(t.x, t.y);
    }
  } else {
#pragma unroll
    for (int i = 0; i < KP; ++i) v[i] = p[i];
  }
}

template <class Z, int KP>
__device__ __forceinline__ void st_chunk(Z *p, const Z (&v)[KP]) {
  if constexpr (sizeof(Z) == 8 && KP == 2) {
    *reinterpret_cast<float4 *>(p) = make_float4(v[0].re, v[0].im, v[1].re, v[1].im);
  } else {
#pragma unroll
    for (int i = 0; i < KP; ++i) p[i] = v[i];
  }
}

static const int kRowThreads = 128;

// One lane per (5-row block row, group of KP test vectors). The L = K/KP
// lanes of a block row fetch each gathered k-vector row together, one
// 16-byte chunk each, so a row is one contiguous access instead of five
// copies of it, and every lane keeps 5 x KP accumulators. Block rows are
// packed 32/L to a warp. Vector rows (y, acc, the forcing slabs, ...) are
// read and written the same way: the lanes of consecutive block rows cover
// consecutive bytes.
// Stages 2-4 are held to 64 registers (8 blocks per SM): more warps in
// flight for their latency-bound gathers (measured faster on the 64^3
// operator than the unbounded 108-register build); stage 1 keeps its
// registers for the forcing synthesis.
//
// FB (forcing block, P.fblk): the forcings were synthesised ahead for a
// block of steps (k_forcing_block, which recorded the block's first step in
// step[2] and its length in step[3]); step s of the block adds slot 2s-1
// (s > 0; the state F3 for s = 0) in stage 1, slot 2s in stages 2 and 3 and
// slot 2s+1 in stage 4, and the block's last step writes its end forcing
// to the state F3. Stage 1 then neither synthesises nor writes F2 / F3.
template <class Z, int K, int KP, int S, bool FB = false>
__global__ void __launch_bounds__(kRowThreads, (S == 1 && !FB) ? 1 : 8) k_bstage(const StepArgs<Z> P) {
  pdl_wait_and_release();
  constexpr int L = K / KP;
  constexpr int BPW = 32 / L;
  extern __shared__ unsigned char smem_raw[];
  Z *e2 = reinterpret_cast<Z *>(smem_raw);  // phasor rows of this step (stage 1)
  Z *e3 = e2 + P.Nw;
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int sub = lane / L, q = lane - sub * L;
  const int64_t br = warp * BPW + sub;
  const int64_t i = (S == 1) ? P.step[0] : P.step[1];
  if constexpr (FB) {
    if (br >= P.N / 5 || sub >= BPW) return;
    if (S == 1 && br == 0 && q == 0) P.step[1] = i;
    const int64_t NK = P.N * K;
    const int64_t sb = i - P.step[2];  // step of the block, 0 .. step[3]-1
    const int64_t base = br * 5 * K + q * KP;
    const Z *x = (S == 1) ? P.y : (S == 2) ? P.zA : (S == 3) ? P.zB : P.zA;
    const Z *addv = (S == 1)   ? (sb == 0 ? P.F3 : P.fblk + (2 * sb - 1) * NK)
                    : (S == 4) ? P.fblk + (2 * sb + 1) * NK
                               : P.fblk + 2 * sb * NK;
    Z k[5][KP];
#pragma unroll
    for (int r = 0; r < 5; ++r) ldg_chunk<Z, KP>(addv + base + r * K, k[r]);
    if (S == 4 && sb == P.step[3] - 1) {
#pragma unroll
      for (int r = 0; r < 5; ++r) st_chunk<Z, KP>(P.F3 + base + r * K, k[r]);
    }
    const int32_t b = __ldg(P.rowptr + br), e = __ldg(P.rowptr + br + 1);
    for (int32_t j = b; j < e; ++j) {
      const int32_t cb = __ldg(P.col + j);
      if (!RSVDT_CHECK_INDEX(cb >= 0 && cb < P.N / 5, 1)) continue;
      const int64_t c0 = (int64_t)cb * 5;
      const Z *blk = P.val + (int64_t)j * P.bstride;
      if constexpr (S == 4 && sizeof(Z) == 8) {
        // The padded 26-value block as 13 aligned 16-byte loads.
        Z a[26];
        const float4 *b4 = reinterpret_cast<const float4 *>(blk);
#pragma unroll
        for (int m = 0; m < 13; ++m) {
          const float4 t = __ldg(b4 + m);
          a[2 * m] = zmake<Z>(t.x, t.y);
          a[2 * m + 1] = zmake<Z>(t.z, t.w);
        }
#pragma unroll
        for (int c = 0; c < 5; ++c) {
          Z xv[KP];
          ldg_chunk<Z, KP>(x + (c0 + c) * K + q * KP, xv);
#pragma unroll
          for (int r = 0; r < 5; ++r)
#pragma unroll
            for (int p = 0; p < KP; ++p) zmac(k[r][p], a[r * 5 + c], xv[p]);
        }
      } else {
#pragma unroll
        for (int c = 0; c < 5; ++c) {
          Z xv[KP];
          ldg_chunk<Z, KP>(x + (c0 + c) * K + q * KP, xv);
#pragma unroll
          for (int r = 0; r < 5; ++r) {
            const Z a = blk[r * 5 + c];
#pragma unroll
            for (int p = 0; p < KP; ++p) zmac(k[r][p], a, xv[p]);
          }
        }
      }
    }
    if (S == 1) {
#pragma unroll
      for (int r = 0; r < 5; ++r) {
        Z yv[KP], t[KP];
        ldg_chunk<Z, KP>(P.y + base + r * K, yv);
#pragma unroll
        for (int p = 0; p < KP; ++p) t[p] = zaxpy(P.dt_2, k[r][p], yv[p]);
        st_chunk<Z, KP>(P.zA + base + r * K, t);
#pragma unroll
        for (int p = 0; p < KP; ++p) t[p] = zaxpy(P.dt_6, k[r][p], yv[p]);
        st_chunk<Z, KP>(P.acc + base + r * K, t);
      }
    } else if (S == 2 || S == 3) {
#pragma unroll
      for (int r = 0; r < 5; ++r) {
        Z yv[KP], t[KP], av[KP];
        ldg_chunk<Z, KP>(P.y + base + r * K, yv);
#pragma unroll
        for (int p = 0; p < KP; ++p) t[p] = zaxpy(S == 2 ? P.dt_2 : P.dt, k[r][p], yv[p]);
        st_chunk<Z, KP>((S == 2 ? P.zB : P.zA) + base + r * K, t);
        ld_chunk<Z, KP>(P.acc + base + r * K, av);
#pragma unroll
        for (int p = 0; p < KP; ++p) av[p] = zaxpy(P.dt_62, k[r][p], av[p]);
        st_chunk<Z, KP>(P.acc + base + r * K, av);
      }
    } else {
      const int64_t ps = P.ring ? ring_slot(P.dir, i, P.Nt, P.R, P.Nstore) : -1;
#pragma unroll
      for (int r = 0; r < 5; ++r) {
        Z av[KP];
        ld_chunk<Z, KP>(P.acc + base + r * K, av);
#pragma unroll
        for (int p = 0; p < KP; ++p) av[p] = zaxpy(P.dt_6, k[r][p], av[p]);
        st_chunk<Z, KP>(P.y + base + r * K, av);
        if (ps >= 0 && RSVDT_CHECK_INDEX(ps < P.Nstore, 2))
          st_chunk<Z, KP>(P.ring + ps * P.N * K + base + r * K, av);
      }
      if (br == 0 && q == 0) P.step[0] = i + 1;
    }
    return;
  }
  if (S == 1) {
    if (P.Fh) {
      int64_t j2, j3;
      step_idx(P.dir, i, P.two_ns, j2, j3);
      for (int s = threadIdx.x; s < P.Nw; s += blockDim.x) {
        e2[s] = P.tab[j2 * P.Nw + s];
        e3[s] = P.tab[j3 * P.Nw + s];
      }
    }
    __syncthreads();
  }
  if (sub >= BPW || br >= P.N / 5) return;
  if (S == 1 && br == 0 && q == 0) P.step[1] = i;
  const int64_t base = br * 5 * K + q * KP;  // element (row br*5, test vector q*KP)
  const Z *x = (S == 1) ? P.y : (S == 2) ? P.zA : (S == 3) ? P.zB : P.zA;
  const Z *addv = (S == 1 || S == 4) ? P.F3 : P.F2;
  Z k[5][KP];
#pragma unroll
  for (int r = 0; r < 5; ++r) {
    if (S == 1)
      ld_chunk<Z, KP>(addv + base + r * K, k[r]);  // F3 is rewritten below by this lane
    else
      ldg_chunk<Z, KP>(addv + base + r * K, k[r]);
  }
  {
    const int32_t b = __ldg(P.rowptr + br), e = __ldg(P.rowptr + br + 1);
    for (int32_t j = b; j < e; ++j) {
      const int32_t cb = __ldg(P.col + j);
      if (!RSVDT_CHECK_INDEX(cb >= 0 && cb < P.N / 5, 1)) continue;
      const int64_t c0 = (int64_t)cb * 5;
      const Z *blk = P.val + (int64_t)j * P.bstride;
      if constexpr (S == 4 && sizeof(Z) == 8) {
        // The padded 26-value block as 13 aligned 16-byte loads.
        Z a[26];
        const float4 *b4 = reinterpret_cast<const float4 *>(blk);
#pragma unroll
        for (int m = 0; m < 13; ++m) {
          const float4 t = __ldg(b4 + m);
          a[2 * m] = zmake<Z>(t.x, t.y);
          a[2 * m + 1] = zmake<Z>(t.z, t.w);
        }
#pragma unroll
        for (int c = 0; c < 5; ++c) {
          Z xv[KP];
          ldg_chunk<Z, KP>(x + (c0 + c) * K + q * KP, xv);
#pragma unroll
          for (int r = 0; r < 5; ++r)
#pragma unroll
            for (int p = 0; p < KP; ++p) zmac(k[r][p], a[r * 5 + c], xv[p]);
        }
      } else {
#pragma unroll
        for (int c = 0; c < 5; ++c) {
          Z xv[KP];
          ldg_chunk<Z, KP>(x + (c0 + c) * K + q * KP, xv);
#pragma unroll
          for (int r = 0; r < 5; ++r) {
            const Z a = blk[r * 5 + c];
#pragma unroll
            for (int p = 0; p < KP; ++p) zmac(k[r][p], a, xv[p]);
          }
        }
      }
    }
  }
  if (S == 1) {
#pragma unroll
    for (int r = 0; r < 5; ++r) {
      Z yv[KP], t[KP];
      ldg_chunk<Z, KP>(P.y + base + r * K, yv);
#pragma unroll
      for (int p = 0; p < KP; ++p) t[p] = zaxpy(P.dt_2, k[r][p], yv[p]);
      st_chunk<Z, KP>(P.zA + base + r * K, t);
#pragma unroll
      for (int p = 0; p < KP; ++p) t[p] = zaxpy(P.dt_6, k[r][p], yv[p]);
      st_chunk<Z, KP>(P.acc + base + r * K, t);
    }
    // Forcing at the half step and the full step, pair or plain slabs.
    Z f2[5][KP], f3[5][KP];
#pragma unroll
    for (int r = 0; r < 5; ++r)
#pragma unroll
      for (int p = 0; p < KP; ++p) f2[r][p] = f3[r][p] = zmake<Z>(0, 0);
    if (P.Fh) {
      const int64_t NK = P.N * K;
      const Z *c = P.Fh + base;
      if (P.pair) {
        const int H = P.Nw / 2;
#pragma unroll
        for (int r = 0; r < 5; ++r) {
          Z v[KP];
          ldg_chunk<Z, KP>(c + r * K, v);
#pragma unroll
          for (int p = 0; p < KP; ++p) {
            zmac(f2[r][p], v[p], e2[0]);
            zmac(f3[r][p], v[p], e3[0]);
          }
        }
#pragma unroll 2
        for (int s = 1; s <= 2 * H - 2; ++s) {
          const auto w2 = pair_weight(e2, s, H), w3 = pair_weight(e3, s, H);
#pragma unroll
          for (int r = 0; r < 5; ++r) {
            Z v[KP];
            ldg_chunk<Z, KP>(c + (int64_t)s * NK + r * K, v);
#pragma unroll
            for (int p = 0; p < KP; ++p) {
              f2[r][p].re = fma(w2, v[p].re, f2[r][p].re);
              f2[r][p].im = fma(w2, v[p].im, f2[r][p].im);
              f3[r][p].re = fma(w3, v[p].re, f3[r][p].re);
              f3[r][p].im = fma(w3, v[p].im, f3[r][p].im);
            }
          }
        }
#pragma unroll
        for (int r = 0; r < 5; ++r) {
          Z v[KP];
          ldg_chunk<Z, KP>(c + (int64_t)(P.Nw - 1) * NK + r * K, v);
#pragma unroll
          for (int p = 0; p < KP; ++p) {
            zmac(f2[r][p], v[p], e2[H]);
            zmac(f3[r][p], v[p], e3[H]);
          }
        }
      } else {
#pragma unroll 2
        for (int s = 0; s < P.Nw; ++s) {
#pragma unroll
          for (int r = 0; r < 5; ++r) {
            Z v[KP];
            ldg_chunk<Z, KP>(c + (int64_t)s * NK + r * K, v);
#pragma unroll
            for (int p = 0; p < KP; ++p) {
              zmac(f2[r][p], v[p], e2[s]);
              zmac(f3[r][p], v[p], e3[s]);
            }
          }
        }
      }
    }
#pragma unroll
    for (int r = 0; r < 5; ++r) {
      st_chunk<Z, KP>(P.F2 + base + r * K, f2[r]);
      st_chunk<Z, KP>(P.F3 + base + r * K, f3[r]);
    }
  } else if (S == 2 || S == 3) {
#pragma unroll
    for (int r = 0; r < 5; ++r) {
      Z yv[KP], t[KP], av[KP];
      ldg_chunk<Z, KP>(P.y + base + r * K, yv);
#pragma unroll
      for (int p = 0; p < KP; ++p) t[p] = zaxpy(S == 2 ? P.dt_2 : P.dt, k[r][p], yv[p]);
      st_chunk<Z, KP>((S == 2 ? P.zB : P.zA) + base + r * K, t);
      ld_chunk<Z, KP>(P.acc + base + r * K, av);
#pragma unroll
      for (int p = 0; p < KP; ++p) av[p] = zaxpy(P.dt_62, k[r][p], av[p]);
      st_chunk<Z, KP>(P.acc + base + r * K, av);
    }
  } else {
    const int64_t ps = P.ring ? ring_slot(P.dir, i, P.Nt, P.R, P.Nstore) : -1;
#pragma unroll
    for (int r = 0; r < 5; ++r) {
      Z av[KP];
      ld_chunk<Z, KP>(P.acc + base + r * K, av);
#pragma unroll
      for (int p = 0; p < KP; ++p) av[p] = zaxpy(P.dt_6, k[r][p], av[p]);
      st_chunk<Z, KP>(P.y + base + r * K, av);
      if (ps >= 0 && RSVDT_CHECK_INDEX(ps < P.Nstore, 2)) st_chunk<Z, KP>(P.ring + ps * P.N * K + base + r * K, av);
    }
    if (br == 0 && q == 0) P.step[0] = i + 1;
  }
}

// Row of K complex values; 16-byte loads/stores (K even for complex64).
template <class Z, int K>
__device__ __forceinline__ void ld_row(const Z *p, Z (&v)[K]) {
  if constexpr (sizeof(Z) == 8 && K % 2 == 0) {
    const float4 *q = reinterpret_cast<const float4 *>(p);
#pragma unroll
    for (int i = 0; i < K / 2; ++i) {
      const float4 t = q[i];
      v[2 * i] = zmake<Z>(t.x, t.y);
      v[2 * i + 1] = zmake<Z>(t.z, t.w);
    }
  } else {
#pragma unroll
    for (int i = 0; i < K; ++i) v[i] = p[i];
  }
}

// Read-only variant through the non-coherent path.
template <class Z, int K>
__device__ __forceinline__ void ldg_row(const Z *p, Z (&v)[K]) {
  if constexpr (sizeof(Z) == 8 && K % 2 == 0) {
    const float4 *q = reinterpret_cast<const float4 *>(p);
#pragma unroll
    for (int i = 0; i < K / 2; ++i) {
      const float4 t = __ldg(q + i);
      v[2 * i] = zmake<Z>(t.x, t.y);
      v[2 * i + 1] = zmake<Z>(t.z, t.w);
    }
  } else if constexpr (sizeof(Z) == 16) {
    const double2 *q = reinterpret_cast<const double2 *>(p);
#pragma unroll
    for (int i = 0; i < K; ++i) {
      const double2 t = __ldg(q + i);
      v[i] = zmake<Z>(t.x, t.y);
    }
  } else {
#pragma unroll
    for (int i = 0; i < K; ++i) v[i] = p[i];
  }
}

template <class Z, int K>
__device__ __forceinline__ void st_row(Z *p, const Z (&v)[K]) {
  if constexpr (sizeof(Z) == 8 && K % 2 == 0) {
    float4 *q = reinterpret_cast<float4 *>(p);
#pragma unroll
    for (int i = 0; i < K / 2; ++i) q[i] = make_float4(v[2 * i].re, v[2 * i].im, v[2 * i + 1].re, v[2 * i + 1].im);
  } else {
#pragma unroll
    for (int i = 0; i < K; ++i) p[i] = v[i];
  }
}

// Forcing at two times for one row, all K test vectors (pair or plain slabs);
// e2 / e3 are the phasor rows staged in shared memory.
template <class Z, int K>
__device__ __forceinline__ void forcing_row(const StepArgs<Z> &P, int64_t n, const Z *e2, const Z *e3,
                                            Z (&f2)[K], Z (&f3)[K]) {
  const int64_t NK = P.N * K;
  const Z *c = P.Fh + n * K;
#pragma unroll
  for (int q = 0; q < K; ++q) f2[q] = f3[q] = zmake<Z>(0, 0);
  if (P.pair) {
    const int H = P.Nw / 2;
    Z v[K];
    ldg_row<Z, K>(c, v);
#pragma unroll
    for (int q = 0; q < K; ++q) {
      zmac(f2[q], v[q], e2[0]);
      zmac(f3[q], v[q], e3[0]);
    }
#pragma unroll 2
    for (int s = 1; s <= 2 * H - 2; ++s) {
      const auto w2 = pair_weight(e2, s, H), w3 = pair_weight(e3, s, H);
      ldg_row<Z, K>(c + (int64_t)s * NK, v);
#pragma unroll
      for (int q = 0; q < K; ++q) {
        f2[q].re = fma(w2, v[q].re, f2[q].re);
        f2[q].im = fma(w2, v[q].im, f2[q].im);
        f3[q].re = fma(w3, v[q].re, f3[q].re);
        f3[q].im = fma(w3, v[q].im, f3[q].im);
      }
    }
    ldg_row<Z, K>(c + (int64_t)(P.Nw - 1) * NK, v);
#pragma unroll
    for (int q = 0; q < K; ++q) {
      zmac(f2[q], v[q], e2[H]);
      zmac(f3[q], v[q], e3[H]);
    }
  } else {
#pragma unroll 2
    for (int s = 0; s < P.Nw; ++s) {
      Z v[K];
      ldg_row<Z, K>(c + (int64_t)s * NK, v);
#pragma unroll
      for (int q = 0; q < K; ++q) {
        zmac(f2[q], v[q], e2[s]);
        zmac(f3[q], v[q], e3[s]);
      }
    }
  }
}

// One thread per row with all K test vectors in registers (complex128):
// full warps, which is what matters when the FP64 pipe is the limit; the
// lane-group kernel above leaves lanes idle for complex128 row groups.
template <class Z, int K, int S>
__global__ void __launch_bounds__(kRowThreads) k_rstage(const StepArgs<Z> P) {
  pdl_wait_and_release();
  extern __shared__ unsigned char smem_raw[];
  Z *e2 = reinterpret_cast<Z *>(smem_raw);  // phasor rows of this step (stage 1)
  Z *e3 = e2 + P.Nw;
  const int64_t n = P.row0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t i = (S == 1) ? P.step[0] : P.step[1];
  if (S == 1) {
    if (P.Fh) {
      int64_t j2, j3;
      step_idx(P.dir, i, P.two_ns, j2, j3);
      for (int s = threadIdx.x; s < P.Nw; s += blockDim.x) {
        e2[s] = P.tab[j2 * P.Nw + s];
        e3[s] = P.tab[j3 * P.Nw + s];
      }
    }
    __syncthreads();
  }
  if (n >= P.row1) return;
  if (S == 1 && n == 0) P.step[1] = i;
  const Z *x = (S == 1) ? P.y : (S == 2) ? P.zA : (S == 3) ? P.zB : P.zA;
  const Z *addv = (S == 1 || S == 4) ? P.F3 : P.F2;
  Z k[K];
  if (S == 1)
    ld_row<Z, K>(addv + n * K, k);  // F3 is rewritten below by this thread
  else
    ldg_row<Z, K>(addv + n * K, k);
  // Sparse product over the 5x5 blocks of block row n / 5.
  {
    const int64_t br = n / 5;
    const int r = (int)(n - br * 5);
    const int32_t b = __ldg(P.rowptr + br), e = __ldg(P.rowptr + br + 1);
    for (int32_t j = b; j < e; ++j) {
      const int32_t cb = __ldg(P.col + j);
      if (!RSVDT_CHECK_INDEX(cb >= 0 && cb < P.N / 5, 1)) continue;
      const int64_t c0 = (int64_t)cb * 5;
      const Z *arow = P.val + (int64_t)j * P.bstride + r * 5;
      Z a[5];
#pragma unroll
      for (int c = 0; c < 5; ++c) a[c] = arow[c];
#pragma unroll
      for (int c = 0; c < 5; ++c) {
        Z xv[K];
        ldg_row<Z, K>(x + (c0 + c) * K, xv);
#pragma unroll
        for (int q = 0; q < K; ++q) zmac(k[q], a[c], xv[q]);
      }
    }
  }
  Z yv[K];
  if (S != 4) ldg_row<Z, K>(P.y + n * K, yv);
  if (S == 1) {
    Z t[K];
#pragma unroll
    for (int q = 0; q < K; ++q) t[q] = zaxpy(P.dt_2, k[q], yv[q]);
    st_row<Z, K>(P.zA + n * K, t);
#pragma unroll
    for (int q = 0; q < K; ++q) t[q] = zaxpy(P.dt_6, k[q], yv[q]);
    st_row<Z, K>(P.acc + n * K, t);
    Z f2[K], f3[K];
    if (P.Fh) {
      forcing_row<Z, K>(P, n, e2, e3, f2, f3);
    } else {
#pragma unroll
      for (int q = 0; q < K; ++q) f2[q] = f3[q] = zmake<Z>(0, 0);
    }
    st_row<Z, K>(P.F2 + n * K, f2);
    st_row<Z, K>(P.F3 + n * K, f3);
  } else if (S == 2 || S == 3) {
    Z t[K], av[K];
#pragma unroll
    for (int q = 0; q < K; ++q) t[q] = zaxpy(S == 2 ? P.dt_2 : P.dt, k[q], yv[q]);
    st_row<Z, K>((S == 2 ? P.zB : P.zA) + n * K, t);
    ld_row<Z, K>(P.acc + n * K, av);
#pragma unroll
    for (int q = 0; q < K; ++q) av[q] = zaxpy(P.dt_62, k[q], av[q]);
    st_row<Z, K>(P.acc + n * K, av);
  } else {
    Z av[K];
    ld_row<Z, K>(P.acc + n * K, av);
#pragma unroll
    for (int q = 0; q < K; ++q) av[q] = zaxpy(P.dt_6, k[q], av[q]);
    st_row<Z, K>(P.y + n * K, av);
    const int64_t p = P.ring ? ring_slot(P.dir, i, P.Nt, P.R, P.Nstore) : -1;
    if (p >= 0 && RSVDT_CHECK_INDEX(p < P.Nstore, 2)) st_row<Z, K>(P.ring + (p * P.N + n) * K, av);
    if (n == 0) P.step[0] = i + 1;
  }
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
  P.F3[t] = forcing_at(P, n, kc, P.tab);
  P.y[t] = zmake<Z>(0, 0);
}

// Forcing slabs from test vectors k0 .. k0+K-1 of the working block
// blk[n][iw][kb] (complex128, Kb test vectors): Fh[s][n][k], pair or plain
// (see the file comment), in precision Z.
template <class Z>
__global__ void k_stage_slabs(const z128 *__restrict__ blk, int64_t N, int Nw, int K, int pair,
                              Z *__restrict__ Fh, int Kb, int k0) {
  const int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t NK = N * K;
  if (u >= NK * Nw) return;
  const int s = (int)(u / NK);
  const int64_t r = u - (int64_t)s * NK;
  const int64_t n = r / K;
  const int kc = (int)(r - n * K);
  const z128 *row = blk + n * (int64_t)Nw * Kb + k0 + kc;
  z128 v;
  if (!pair) {
    v = row[(int64_t)s * Kb];
  } else {
    const int H = Nw / 2;
    if (s == 0) {
      v = row[0];
    } else if (s == Nw - 1) {
      v = row[(int64_t)H * Kb];
    } else {
      const int f = s < H ? s : s - H + 1;
      const z128 cp = row[(int64_t)f * Kb], cn = row[(int64_t)(Nw - f) * Kb];
      if (s < H)
        v = zmake<z128>(cp.re + cn.re, cp.im + cn.im);
      else  // i (cp - cn)
        v = zmake<z128>(-(cp.im - cn.im), cp.re - cn.re);
    }
  }
  Fh[u] = zmake<Z>((typename real_of<Z>::type)v.re, (typename real_of<Z>::type)v.im);
}

template <class Z>
static StepArgs<Z> make_args(rsvdt_ctx *ctx, int dir, bool forced) {
  StepArgs<Z> P;
  P.N = ctx->N;
  P.K = (int)ctx->Ks;
  P.Nw = (int)ctx->Nw_eff;
  P.pair = ctx->pair ? 1 : 0;
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
    P.bstride = c64 ? M.stride32 : M.bs * M.bs;
  } else {
    const DevCSR &M = dir ? ctx->A : ctx->AH;
    P.rowptr = M.rowptr;
    P.col = M.col;
    P.val = (const Z *)(c64 ? (void *)M.val32 : (void *)M.val);
    P.bs = 0;
    P.bstride = 0;
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
  P.rend = INT64_MAX;
  P.row0 = 0;
  P.row1 = P.N;
  P.fblk = nullptr;
  return P;
}

// ------------------------------------------- forcing block (complex64)
//
// The forcing synthesis (SourceCode/CreateForcingOnFly.c:17-19) for a block
// of nblk <= kFbMaxSteps steps at once: every slab value is read once per
// block instead of once per step, and the 2*nblk half-step forcings are
// written to P.fblk (slot 2s: F2 of the block's step s, slot 2s+1: its F3).
// A matrix product (2 nblk phasor rows) x (Nw slabs) x (N k values), FP32
// FMA with the same operations in the same order as stage 1's own
// synthesis (bit-identical forcings). One thread per (row, test vector)
// holds that value's Nw slab coefficients in registers; the block's phasor
// weights sit in shared memory, one row per half step: for pair slabs
// [Re e_0, Im e_0, Re e_1 .. Re e_{H-1}, Im e_1 .. Im e_{H-1}, Re e_H,
// Im e_H] (slab s >= 1 takes weight s + 1), for plain slabs the Nw complex
// phasors. The block's first step and length go to step[2] and step[3].

static const int kFbThreads = 256;
static const int kFbMaxSteps = 16;  // largest forcing block (steps)

template <int NW, bool PAIR>
__global__ void __launch_bounds__(kFbThreads) k_forcing_block(const StepArgs<z64> P, int nblk) {
  pdl_wait_and_release();
  constexpr int ROW = ((PAIR ? NW + 2 : 2 * NW) + 3) / 4 * 4;
  __shared__ __align__(16) float wt[2 * kFbMaxSteps][ROW];
  const int64_t i_s = P.step[0];
  for (int idx = threadIdx.x; idx < 2 * nblk * NW; idx += blockDim.x) {
    const int m = idx / NW, s = idx - m * NW;
    int64_t j2, j3;
    step_idx(P.dir, i_s + m / 2, P.two_ns, j2, j3);
    const z64 e = P.tab[((m & 1) ? j3 : j2) * NW + s];
    if (PAIR) {
      constexpr int H = NW / 2;
      if (s == 0) {
        wt[m][0] = e.re;
        wt[m][1] = e.im;
      } else if (s < H) {
        wt[m][s + 1] = e.re;
        wt[m][H + s] = e.im;
      } else if (s == H) {
        wt[m][NW] = e.re;
        wt[m][NW + 1] = e.im;
      }
    } else {
      wt[m][2 * s] = e.re;
      wt[m][2 * s + 1] = e.im;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    P.step[2] = i_s;
    P.step[3] = nblk;
  }
  __syncthreads();
  const int64_t NK = P.N * P.K;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < NK; t += (int64_t)gridDim.x * blockDim.x) {
    z64 v[NW];
#pragma unroll
    for (int s = 0; s < NW; ++s) {
      const float2 u = __ldg(reinterpret_cast<const float2 *>(P.Fh + (int64_t)s * NK + t));
      v[s] = zmake<z64>(u.x, u.y);
    }
    for (int m = 0; m < 2 * nblk; ++m) {
      const float *w = wt[m];
      z64 f = zmake<z64>(0, 0);
      if (PAIR) {
        zmac(f, v[0], zmake<z64>(w[0], w[1]));
#pragma unroll
        for (int s = 1; s <= NW - 2; ++s) {
          f.re = fmaf(w[s + 1], v[s].re, f.re);
          f.im = fmaf(w[s + 1], v[s].im, f.im);
        }
        zmac(f, v[NW - 1], zmake<z64>(w[NW], w[NW + 1]));
      } else {
#pragma unroll
        for (int s = 0; s < NW; ++s) zmac(f, v[s], zmake<z64>(w[2 * s], w[2 * s + 1]));
      }
      *reinterpret_cast<float2 *>(P.fblk + (int64_t)m * NK + t) = make_float2(f.re, f.im);
    }
  }
}

// Whether a forcing block can serve these stage arguments: complex64 5x5
// block-row stages (k_bstage) with the forcing on and Nw in 8..64 (powers
// of two, the slab counts compiled into k_forcing_block).
static bool forcing_block_applies(const StepArgs<z64> &P) {
  if (!P.Fh || P.bs != 5) return false;
  switch (P.K) {
    case 2: case 4: case 6: case 8: case 10: case 16: break;
    default: return false;
  }
  return P.Nw == 8 || P.Nw == 16 || P.Nw == 32 || P.Nw == 64;
}

template <int NW>
static void launch_forcing_block_nw(const StepArgs<z64> &P, int nblk, int grid, cudaStream_t st) {
  if (P.pair)
    launch_pdl(k_forcing_block<NW, true>, grid, kFbThreads, 0, st, P, nblk);
  else
    launch_pdl(k_forcing_block<NW, false>, grid, kFbThreads, 0, st, P, nblk);
}

// The forcing of the next nblk steps (from the device step counter) into
// P.fblk; grid: a few blocks per SM, each striding over the values.
static void launch_forcing_block(const StepArgs<z64> &P, int nblk, int sm_count, cudaStream_t st) {
  const int64_t NK = P.N * P.K;
  const int grid = (int)std::min<int64_t>((NK + kFbThreads - 1) / kFbThreads, (int64_t)4 * std::max(sm_count, 1));
  switch (P.Nw) {
    case 8: launch_forcing_block_nw<8>(P, nblk, grid, st); break;
    case 16: launch_forcing_block_nw<16>(P, nblk, grid, st); break;
    case 32: launch_forcing_block_nw<32>(P, nblk, grid, st); break;
    default: launch_forcing_block_nw<64>(P, nblk, grid, st); break;
  }
}

// ---------------------------------------------------------- dispatch

template <class Z, int K>
static void launch_bstage(int stage, const StepArgs<Z> &P, cudaStream_t st) {
  constexpr int KP = (sizeof(Z) == 8 && K % 2 == 0) ? 2 : 1;
  constexpr int L = K / KP;
  constexpr int BPW = 32 / L;
  const int64_t warps = (P.N / 5 + BPW - 1) / BPW;
  const int g = grid_for(warps * 32, kRowThreads);
  const size_t sm = sizeof(Z) * 2 * (P.Nw > 0 ? P.Nw : 1);
  if constexpr (sizeof(Z) == 16) {
    const int gr = grid_for(P.row1 - P.row0, kRowThreads);
    switch (stage) {
      case 1: launch_pdl(k_rstage<Z, K, 1>, gr, kRowThreads, sm, st, P); break;
      case 2: launch_pdl(k_rstage<Z, K, 2>, gr, kRowThreads, 0, st, P); break;
      case 3: launch_pdl(k_rstage<Z, K, 3>, gr, kRowThreads, 0, st, P); break;
      default: launch_pdl(k_rstage<Z, K, 4>, gr, kRowThreads, 0, st, P); break;
    }
    return;
  }
  if constexpr (sizeof(Z) == 8) {
    if (P.fblk) {
      switch (stage) {
        case 1: launch_pdl(k_bstage<Z, K, KP, 1, true>, g, kRowThreads, 0, st, P); break;
        case 2: launch_pdl(k_bstage<Z, K, KP, 2, true>, g, kRowThreads, 0, st, P); break;
        case 3: launch_pdl(k_bstage<Z, K, KP, 3, true>, g, kRowThreads, 0, st, P); break;
        default: launch_pdl(k_bstage<Z, K, KP, 4, true>, g, kRowThreads, 0, st, P); break;
      }
      return;
    }
  }
  switch (stage) {
    case 1: launch_pdl(k_bstage<Z, K, KP, 1>, g, kRowThreads, sm, st, P); break;
    case 2: launch_pdl(k_bstage<Z, K, KP, 2>, g, kRowThreads, 0, st, P); break;
    case 3: launch_pdl(k_bstage<Z, K, KP, 3>, g, kRowThreads, 0, st, P); break;
    default: launch_pdl(k_bstage<Z, K, KP, 4>, g, kRowThreads, 0, st, P); break;
  }
}

// Launches stage `stage` (1..4) with the fastest kernel for the operator.
template <class Z>
static void launch_stage(int stage, const StepArgs<Z> &P, cudaStream_t st) {
  if (P.bs == 5) {
    switch (P.K) {
      case 1:  // a single state vector (transient simulation), complex128 rows
        if constexpr (sizeof(Z) == 16) return launch_bstage<Z, 1>(stage, P, st);
        break;
      case 2: return launch_bstage<Z, 2>(stage, P, st);
      case 4: return launch_bstage<Z, 4>(stage, P, st);
      case 6: return launch_bstage<Z, 6>(stage, P, st);
      case 8: return launch_bstage<Z, 8>(stage, P, st);
      case 10: return launch_bstage<Z, 10>(stage, P, st);
      case 16: return launch_bstage<Z, 16>(stage, P, st);
      default: break;
    }
  }
  const int th = 256;
  const int g = grid_for(P.N * P.K, th);
  switch (stage) {
    case 1: launch_pdl(k_stage<Z, 1>, g, th, 0, st, P); break;
    case 2: launch_pdl(k_stage<Z, 2>, g, th, 0, st, P); break;
    case 3: launch_pdl(k_stage<Z, 3>, g, th, 0, st, P); break;
    default: launch_pdl(k_stage<Z, 4>, g, th, 0, st, P); break;
  }
}

template <class Z>
static void enqueue_step(rsvdt_ctx *ctx, const StepArgs<Z> &P) {
  for (int s = 1; s <= 4; ++s) launch_stage(s, P, ctx->stream);
}

// Slabs of the state's Ks test vectors, k0 .. k0+Ks-1 of the working block.
rsvdt_status stage_forcing_coeffs(rsvdt_ctx *ctx, int prec) {
  const int64_t total = ctx->N * ctx->Nw_eff * ctx->Ks;
  const int th = 256;
  if (prec == RSVDT_PREC_C64)
    k_stage_slabs<z64><<<grid_for(total, th), th, 0, ctx->stream>>>(ctx->blk, ctx->N, (int)ctx->Nw_eff,
                                                                     (int)ctx->Ks, ctx->pair ? 1 : 0,
                                                                     (z64 *)ctx->Fh, (int)ctx->K, (int)ctx->k0);
  else
    k_stage_slabs<z128><<<grid_for(total, th), th, 0, ctx->stream>>>(ctx->blk, ctx->N, (int)ctx->Nw_eff,
                                                                      (int)ctx->Ks, ctx->pair ? 1 : 0,
                                                                      (z128 *)ctx->Fh, (int)ctx->K, (int)ctx->k0);
  ctx->launches += 1;
  return cuda_ok(ctx, cudaGetLastError(), "forcing slabs") ? RSVDT_OK : RSVDT_ERR_CUDA;
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
// Device memory a forcing block leaves free for everything else (dense-stage
// scratch, transfers) when it is allocated.
static const size_t kFbHeadroom = (size_t)4 << 30;

static void free_step_graphs(rsvdt_ctx *ctx) {
  for (auto &g : ctx->step_graph)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
}

// Turns on the forcing block for these stage arguments when it applies;
// *G = the block length, 0 when stage 1 synthesises the forcing (not an
// error: the stage kernels then synthesise it themselves). The buffer
// (2 G N k complex64 values) is, where it fits, the unused half of the slab
// buffer, which is sized for complex128 slabs while the complex64 slabs take
// half of it (automatic G halved down to what fits there: Nw_eff / 2 steps);
// otherwise its own allocation, made only with kFbHeadroom of device memory
// to spare.
static void prepare_forcing_block(rsvdt_ctx *ctx, StepArgs<z64> &P, int *G) {
  *G = 0;
  if (ctx->fb_steps == 0 || !forcing_block_applies(P)) return;
  int g = ctx->fb_steps < 0 ? kFbMaxSteps : ctx->fb_steps;
  const size_t per_step = sizeof(z64) * 2 * (size_t)P.N * (size_t)P.K;
  const size_t slabs = sizeof(z64) * (size_t)P.Nw * (size_t)P.N * (size_t)P.K;
  void *buf = nullptr;
  if (ctx->Fh && ctx->Fh_bytes >= slabs) {
    const size_t fit = (ctx->Fh_bytes - slabs) / per_step;
    int gi = g;
    if (ctx->fb_steps < 0)
      while (gi > 1 && (size_t)gi > fit) gi /= 2;
    if ((size_t)gi <= fit) {
      buf = (unsigned char *)ctx->Fh + slabs;  // slabs is a multiple of 16 bytes (Nw_eff even)
      g = gi;
    }
  }
  if (!buf) {
    const size_t need = per_step * (size_t)g;
    if (ctx->fb_bytes < need) {
      dfree(ctx, ctx->fblk);
      ctx->fblk = nullptr;
      ctx->fb_bytes = 0;
      size_t fr = 0, tot = 0;
      if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
        cudaGetLastError();
        return;
      }
      if (fr < need + kFbHeadroom) return;
      ctx->fblk = dalloc(ctx, need);
      if (!ctx->fblk) return;
      ctx->fb_bytes = need;
    }
    buf = ctx->fblk;
  }
  if (buf != ctx->fb_ptr) {
    free_step_graphs(ctx);  // captured with another buffer
    ctx->fb_ptr = buf;
  }
  if (!ctx->sm_count) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, ctx->device) != cudaSuccess) {
      cudaGetLastError();
      n = 1;
    }
    ctx->sm_count = n;
  }
  P.fblk = (z64 *)buf;
  *G = g;
}

// n steps as stage launches, preceded (G > 0) by one forcing-block launch
// per block of at most G steps; returns the kernels launched.
template <class Z>
static int64_t enqueue_steps(rsvdt_ctx *ctx, const StepArgs<Z> &P, int64_t n, int G) {
  if (G <= 0) {
    for (int64_t s = 0; s < n; ++s) enqueue_step(ctx, P);
    return 4 * n;
  }
  int64_t launches = 0;
  if constexpr (sizeof(Z) == 8) {
    for (int64_t done = 0; done < n;) {
      const int nb = (int)std::min<int64_t>(G, n - done);
      launch_forcing_block(P, nb, ctx->sm_count, ctx->stream);
      for (int s = 0; s < nb; ++s) enqueue_step(ctx, P);
      launches += 1 + 4 * nb;
      done += nb;
    }
  }
  return launches;
}

template <class Z>
static rsvdt_status run_steps_t(rsvdt_ctx *ctx, int dir, int64_t i0, int64_t nsteps) {
  auto P = make_args<Z>(ctx, dir, true);
  int G = 0;
  if constexpr (sizeof(Z) == 8) {
    prepare_forcing_block(ctx, P, &G);
    ctx->fb_last = G;
  }
  k_set_step<<<1, 1, 0, ctx->stream>>>(ctx->d_step, i0);
  ctx->launches += 1;
  int64_t full = nsteps / kGraphSteps, rest = nsteps % kGraphSteps;
  if (full > 0) {
    cudaGraphExec_t &ge = ctx->step_graph[dir ? 1 : 0];
    int &gprec = ctx->step_graph_prec[dir ? 1 : 0];
    int &gfb = ctx->step_graph_fb[dir ? 1 : 0];
    const int prec = sizeof(Z) == sizeof(z64) ? RSVDT_PREC_C64 : RSVDT_PREC_C128;
    if (ge && (gprec != prec || gfb != G)) {
      cudaGraphExecDestroy(ge);
      ge = nullptr;
    }
    int64_t per_graph = 0;
    if (!ge) {
      gprec = prec;
      gfb = G;
      cudaGraph_t g;
      if (!cuda_ok(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal),
                   "begin capture"))
        return RSVDT_ERR_CUDA;
      per_graph = enqueue_steps(ctx, P, kGraphSteps, G);
      if (!cuda_ok(ctx, cudaStreamEndCapture(ctx->stream, &g), "end capture")) return RSVDT_ERR_CUDA;
      if (!cuda_ok(ctx, cudaGraphInstantiate(&ge, g, 0), "graph instantiate")) return RSVDT_ERR_CUDA;
      cudaGraphDestroy(g);
    } else {
      per_graph = 4 * kGraphSteps + (G > 0 ? (kGraphSteps + G - 1) / G : 0);
    }
    for (int64_t c = 0; c < full; ++c)
      if (!cuda_ok(ctx, cudaGraphLaunch(ge, ctx->stream), "graph launch")) return RSVDT_ERR_CUDA;
    ctx->launches += full * per_graph;
  }
  ctx->launches += enqueue_steps(ctx, P, rest, G);
  if (!cuda_ok(ctx, cudaGetLastError(), "rk4 steps")) return RSVDT_ERR_CUDA;
  return RSVDT_OK;
}

// Step i as four stage launches with `after_stage1` recorded between stages
// 1 and 2 (F3, the forcing at the step's end, is final from there on):
// rsvdt_rk4_steps reads F3 back on a second stream meanwhile. Row kernels
// (one lane per row) only.
// Row slabs stage 4 of a step can run in: the one-thread-per-row complex128
// kernel takes a row range (k_rstage: 5x5 block rows, k in its list);
// other kernels run whole (1 slab).
template <class Z>
static int stage4_slabs(const StepArgs<Z> &P, int want) {
  if constexpr (sizeof(Z) != 16) return 1;
  if (P.bs != 5 || P.fblk) return 1;
  switch (P.K) {
    case 1: case 2: case 4: case 6: case 8: case 10: case 16: return want;
    default: return 1;
  }
}

// Stages 2-4 of a step, stage 4 in nslab row slabs with slab_done[s]
// recorded after slab s (rows N s / nslab .. N (s+1) / nslab).
template <class Z>
static int64_t launch_stages_234(rsvdt_ctx *ctx, StepArgs<Z> P, int nslab, cudaEvent_t *slab_done) {
  launch_stage(2, P, ctx->stream);
  launch_stage(3, P, ctx->stream);
  if (!slab_done) {
    launch_stage(4, P, ctx->stream);
    return 3;
  }
  const int64_t N = P.N;
  for (int s = 0; s < nslab; ++s) {
    P.row0 = N * s / nslab;
    P.row1 = N * (s + 1) / nslab;
    launch_stage(4, P, ctx->stream);
    cudaEventRecord(slab_done[s], ctx->stream);
  }
  return 2 + nslab;
}

int stage4_slab_count(rsvdt_ctx *ctx, int dir, int prec, int want) {
  if (prec == RSVDT_PREC_C64) return stage4_slabs(make_args<z64>(ctx, dir, true), want);
  return stage4_slabs(make_args<z128>(ctx, dir, true), want);
}

rsvdt_status run_last_step_split(rsvdt_ctx *ctx, int dir, int prec, int64_t i, cudaEvent_t after_stage1,
                                 int nslab, cudaEvent_t *slab_done) {
  k_set_step<<<1, 1, 0, ctx->stream>>>(ctx->d_step, i);
  int64_t n = 2;
  if (prec == RSVDT_PREC_C64) {
    auto P = make_args<z64>(ctx, dir, true);
    launch_stage(1, P, ctx->stream);
    cudaEventRecord(after_stage1, ctx->stream);
    n += launch_stages_234(ctx, P, 1, nullptr);
  } else {
    auto P = make_args<z128>(ctx, dir, true);
    launch_stage(1, P, ctx->stream);
    cudaEventRecord(after_stage1, ctx->stream);
    n += launch_stages_234(ctx, P, nslab, slab_done);
  }
  ctx->launches += n;
  return cuda_ok(ctx, cudaGetLastError(), "rk4 step") ? RSVDT_OK : RSVDT_ERR_CUDA;
}

// Lanes per (row, test vector) for a context's stepping: 1 runs the stage
// kernels above; 2, 4 or 8 runs the batched stage kernel (below) as a
// batch of one, whose FS lanes split a row's nonzeros and forcing slabs.
// A small problem (few rows x test vectors, e.g. the 500-node
// Ginzburg-Landau case) is bound by the dependent-load chain of one
// thread's forcing synthesis, which the split shortens FS times.
int step_lanes(const rsvdt_ctx *ctx) {
  if (ctx->lanes_override > 0) return ctx->lanes_override;
  // Measured on GB300, the 500-node Ginzburg-Landau step (5000 rows x test
  // vectors): 32 us with one lane, 25.7 with 8, 24.0 with 4; problems a few
  // times larger are faster with one lane per row.
  return ctx->N * ctx->Ks <= 8192 ? 4 : 1;
}

static const int kSmallThreads = 128;

static rsvdt_status run_steps_small(rsvdt_ctx *ctx, int dir, int prec, int64_t i0, int64_t nsteps, int fs) {
  const int d = dir ? 1 : 0;
  const size_t asz = step_args_size(RSVDT_PREC_C128);  // the larger of the two
  if (!ctx->small_args) {
    ctx->small_args = dalloc(ctx, 2 * asz);
    if (!ctx->small_args) return set_err(ctx, RSVDT_ERR_OOM, "argument block allocation failed");
  }
  const int64_t nk = ctx->N * ctx->Ks;
  const int tiles = (int)((nk * fs + kSmallThreads - 1) / kSmallThreads);
  if (ctx->small_nwork != tiles) {
    std::vector<int2> w((size_t)tiles);
    for (int t = 0; t < tiles; ++t) w[(size_t)t] = make_int2(0, t);
    dfree(ctx, ctx->small_work);
    ctx->small_work = (int2 *)dalloc(ctx, sizeof(int2) * (size_t)tiles);
    if (!ctx->small_work) return set_err(ctx, RSVDT_ERR_OOM, "work list allocation failed");
    if (!cuda_ok(ctx, cudaMemcpy(ctx->small_work, w.data(), sizeof(int2) * (size_t)tiles, cudaMemcpyHostToDevice),
                 "work list"))
      return RSVDT_ERR_CUDA;
    ctx->small_nwork = tiles;
    for (auto &g : ctx->small_graph)
      if (g) {
        cudaGraphExecDestroy(g);
        g = nullptr;
      }
  }
  // The argument block of this direction (the step counter is the
  // context's own; no last step).
  unsigned char host[sizeof(StepArgs<z128>)];
  fill_step_args(ctx, d, prec, INT64_MAX, ctx->d_step, host);
  void *dargs = (unsigned char *)ctx->small_args + d * asz;
  if (!cuda_ok(ctx, cudaMemcpyAsync(dargs, host, step_args_size(prec), cudaMemcpyHostToDevice, ctx->stream), "args"))
    return RSVDT_ERR_CUDA;
  launch_set_step(ctx->stream, ctx->d_step, i0);
  ctx->launches += 1;
  int64_t done = 0;
  if (nsteps >= kGraphSteps) {
    cudaGraphExec_t &ge = ctx->small_graph[d];
    const int key = prec * 16 + fs;
    if (ge && ctx->small_graph_key[d] != key) {
      cudaGraphExecDestroy(ge);
      ge = nullptr;
    }
    if (!ge) {
      cudaGraph_t g;
      if (!cuda_ok(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal), "begin capture"))
        return RSVDT_ERR_CUDA;
      for (int64_t s = 0; s < kGraphSteps; ++s)
        launch_batched_step(ctx->stream, prec, dargs, ctx->small_work, tiles, kSmallThreads, fs, ctx->d_step);
      if (!cuda_ok(ctx, cudaStreamEndCapture(ctx->stream, &g), "end capture")) return RSVDT_ERR_CUDA;
      const cudaError_t e = cudaGraphInstantiate(&ge, g, 0);
      cudaGraphDestroy(g);
      if (!cuda_ok(ctx, e, "graph instantiate")) return RSVDT_ERR_CUDA;
      ctx->small_graph_key[d] = key;
    }
    for (; done + kGraphSteps <= nsteps; done += kGraphSteps)
      if (!cuda_ok(ctx, cudaGraphLaunch(ge, ctx->stream), "graph launch")) return RSVDT_ERR_CUDA;
  }
  for (; done < nsteps; ++done)
    launch_batched_step(ctx->stream, prec, dargs, ctx->small_work, tiles, kSmallThreads, fs, ctx->d_step);
  ctx->launches += 4 * nsteps;
  if (!cuda_ok(ctx, cudaGetLastError(), "rk4 steps")) return RSVDT_ERR_CUDA;
  return RSVDT_OK;
}

// ------------------------------------------- the cluster engine (small problems)
//
// A small problem's step is four short dependent stages; launched one by
// one, each costs a launch (~5 us on GB300) for ~1 us of work. The cluster
// engine splits the step differently: the forcing synthesis, which does not
// depend on the state and is the FP64 bulk of a step, runs for G steps at
// once over the whole GPU (k_forcing_steps); then one thread-block cluster
// (up to 16 CTAs, one per SM of a GPC) runs the G steps' four stages back
// to back, one thread per (row, test vector), with a hardware cluster
// barrier between stages (k_cluster_steps). Each value is computed with the
// same operations in the same order as the one-lane stage kernels
// (k_stage): bit-identical results.

static const int kClusterSteps = 64;  // G: steps per forcing / cluster launch pair
static const int kClusterThreads = 512;         // most threads per CTA (one per value)
static const int64_t kClusterAutoMax = 8192;   // largest rows x test vectors AUTO hands to the engine

// A load through L2 only (a value another SM wrote in the same launch).
template <class Z>
__device__ __forceinline__ Z ld_l2(const Z *p) {
  if constexpr (sizeof(Z) == 16) {
    const double2 t = __ldcg(reinterpret_cast<const double2 *>(p));
    return zmake<Z>(t.x, t.y);
  } else {
    const float2 t = __ldcg(reinterpret_cast<const float2 *>(p));
    return zmake<Z>(t.x, t.y);
  }
}

template <class Z>
__global__ void __launch_bounds__(256) k_forcing_steps(const StepArgs<Z> P, int64_t i0, int G, Z *__restrict__ fbuf) {
  const int64_t NK = P.N * P.K;
  const int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (u >= NK * G) return;
  const int g = (int)(u / NK);
  const int64_t t = u - (int64_t)g * NK;
  const int64_t n = t / P.K;
  const int kc = (int)(t - n * P.K);
  Z f2 = zmake<Z>(0, 0), f3 = zmake<Z>(0, 0);
  if (P.Fh) {
    int64_t j2, j3;
    step_idx(P.dir, i0 + g, P.two_ns, j2, j3);
    forcing2(P, n, kc, P.tab + j2 * P.Nw, P.tab + j3 * P.Nw, 0, 1, f2, f3);
  }
  fbuf[(2 * (int64_t)g) * NK + t] = f2;
  fbuf[(2 * (int64_t)g + 1) * NK + t] = f3;
}

__device__ __forceinline__ void cluster_barrier() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// acc += sum_j A[n,j] x[j][kc] over the row (k_stage's row_product), the
// gathered values read through L2: other CTAs of the cluster wrote them
// in this launch.
template <class Z>
__device__ __forceinline__ void row_product_l2(const StepArgs<Z> &P, int64_t n, int kc, const Z *x, Z &acc) {
  const int K = P.K;
  if (P.bs == 0) {
    const int32_t b = __ldg(P.rowptr + n), e = __ldg(P.rowptr + n + 1);
    for (int32_t j = b; j < e; ++j) {
      const int32_t cj = __ldg(P.col + j);
      if (!RSVDT_CHECK_INDEX(cj >= 0 && cj < P.N, 0)) continue;
      zmac(acc, P.val[j], ld_l2<Z>(x + (int64_t)cj * K + kc));
    }
  } else {
    const int bs = P.bs;
    const int64_t br = n / bs;
    const int r = (int)(n - br * bs);
    const int32_t b = __ldg(P.rowptr + br), e = __ldg(P.rowptr + br + 1);
    for (int32_t j = b; j < e; ++j) {
      const int32_t cb = __ldg(P.col + j);
      if (!RSVDT_CHECK_INDEX(cb >= 0 && cb < P.N / bs, 1)) continue;
      const int64_t c0 = (int64_t)cb * bs;
      const Z *blkrow = P.val + (int64_t)j * P.bstride + r * bs;
      for (int c = 0; c < bs; ++c) zmac(acc, blkrow[c], ld_l2<Z>(x + (c0 + c) * K + kc));
    }
  }
}

// Steps i0 .. i0+G-1 of the whole problem on one cluster; fbuf holds each
// step's F2 and F3 (k_forcing_steps). Every thread of every CTA passes every
// barrier (no thread leaves early).
template <class Z>
__global__ void __launch_bounds__(kClusterThreads, 1) k_cluster_steps(const StepArgs<Z> P, int64_t i0, int G,
                                                        const Z *__restrict__ fbuf) {
  const int64_t NK = P.N * P.K;
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const bool valid = t < NK;
  const int64_t n = valid ? t / P.K : 0;
  const int kc = valid ? (int)(t - n * P.K) : 0;
  Z y = zmake<Z>(0, 0), f3old = zmake<Z>(0, 0), acc = zmake<Z>(0, 0);
  if (valid) {
    y = P.y[t];
    f3old = P.F3[t];
  }
  for (int g = 0; g < G; ++g) {
    const int64_t i = i0 + g;
    Z f2 = zmake<Z>(0, 0), f3 = zmake<Z>(0, 0);
    if (valid) {
      f2 = fbuf[(2 * (int64_t)g) * NK + t];
      f3 = fbuf[(2 * (int64_t)g + 1) * NK + t];
      Z k = f3old;  // stage 1: k1 = A y + F3 of the previous step
      row_product_l2(P, n, kc, P.y, k);
      P.zA[t] = zaxpy(P.dt_2, k, y);
      acc = zaxpy(P.dt_6, k, y);
      f3old = f3;
    }
    cluster_barrier();
    if (valid) {
      Z k = f2;  // stage 2
      row_product_l2(P, n, kc, P.zA, k);
      P.zB[t] = zaxpy(P.dt_2, k, y);
      acc = zaxpy(P.dt_62, k, acc);
    }
    cluster_barrier();
    if (valid) {
      Z k = f2;  // stage 3
      row_product_l2(P, n, kc, P.zB, k);
      P.zA[t] = zaxpy(P.dt, k, y);
      acc = zaxpy(P.dt_62, k, acc);
    }
    cluster_barrier();
    if (valid) {
      Z k = f3;  // stage 4
      row_product_l2(P, n, kc, P.zA, k);
      y = zaxpy(P.dt_6, k, acc);
      P.y[t] = y;
      const int64_t p = P.ring ? ring_slot(P.dir, i, P.Nt, P.R, P.Nstore) : -1;
      if (p >= 0 && RSVDT_CHECK_INDEX(p < P.Nstore, 2)) P.ring[p * NK + t] = y;
    }
    cluster_barrier();
  }
  if (valid) {
    P.F2[t] = fbuf[(2 * (int64_t)(G - 1)) * NK + t];
    P.F3[t] = f3old;
    P.acc[t] = acc;
  }
  if (t == 0) {
    P.step[0] = i0 + G;
    P.step[1] = i0 + G - 1;
  }
}

// Cluster size and threads per CTA for a problem of NK values (0: the
// engine does not apply).
template <class Z>
static int cluster_shape(int64_t NK, int *threads) {
  // Largest launchable cluster per device ordinal (devices may differ in
  // SM count or partitioning), stored plus one so that the zero-initialised
  // 0 means "not yet queried". Concurrent first queries from several host
  // threads compute and store the same value.
  constexpr int kMaxDevices = 64;
  static std::atomic<int> max_cluster_dev[kMaxDevices];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return 0;
  }
  int max_cluster = max_cluster_dev[dev].load(std::memory_order_acquire) - 1;
  if (max_cluster < 0) {
    max_cluster = 0;
    if (cudaFuncSetAttribute(k_cluster_steps<Z>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess) {
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(16);
      cfg.blockDim = dim3(kClusterThreads);
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeClusterDimension;
      at[0].val.clusterDim.x = 16;
      at[0].val.clusterDim.y = 1;
      at[0].val.clusterDim.z = 1;
      cfg.attrs = at;
      cfg.numAttrs = 1;
      int c = 0;
      if (cudaOccupancyMaxPotentialClusterSize(&c, k_cluster_steps<Z>, &cfg) == cudaSuccess) max_cluster = c;
    }
    cudaGetLastError();
    if (max_cluster > 16) max_cluster = 16;
    max_cluster_dev[dev].store(max_cluster + 1, std::memory_order_release);
  }
  // As many SMs as a cluster can have (the stages' FP64 work spreads over
  // them), one thread per value.
  if (max_cluster < 1) return 0;
  const int64_t per = (NK + max_cluster - 1) / max_cluster;
  if (per > kClusterThreads) return 0;
  *threads = (int)((per + 31) / 32 * 32);
  return max_cluster;
}

template <class Z>
static rsvdt_status run_steps_cluster_t(rsvdt_ctx *ctx, int dir, int64_t i0, int64_t nsteps, int C, int threads) {
  auto P = make_args<Z>(ctx, dir, true);
  const int64_t NK = P.N * P.K;
  const size_t need = sizeof(Z) * 2 * (size_t)NK * kClusterSteps;
  if (ctx->cl_bytes < need) {
    dfree(ctx, ctx->cl_fbuf);
    ctx->cl_fbuf = dalloc(ctx, need);
    ctx->cl_bytes = ctx->cl_fbuf ? need : 0;
    if (!ctx->cl_fbuf) return set_err(ctx, RSVDT_ERR_OOM, "forcing buffer allocation failed");
  }
  Z *fbuf = (Z *)ctx->cl_fbuf;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)C);
  cfg.blockDim = dim3((unsigned)threads);
  cfg.stream = ctx->stream;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = (unsigned)C;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  for (int64_t done = 0; done < nsteps;) {
    const int G = (int)std::min<int64_t>(kClusterSteps, nsteps - done);
    const int64_t i = i0 + done;
    k_forcing_steps<Z><<<grid_for(NK * G, 256), 256, 0, ctx->stream>>>(P, i, G, fbuf);
    if (!cuda_ok(ctx, cudaLaunchKernelEx(&cfg, k_cluster_steps<Z>, P, i, G, (const Z *)fbuf), "cluster steps"))
      return RSVDT_ERR_CUDA;
    ctx->launches += 2;
    done += G;
  }
  return cuda_ok(ctx, cudaGetLastError(), "cluster steps") ? RSVDT_OK : RSVDT_ERR_CUDA;
}

// ------------------------------- first step with its forcing synthesised ahead
//
// rsvdt_rk4_steps uploads the state from host memory before its first step.
// The step's forcing (F2, F3 from the slabs, the FP64 bulk of stage 1)
// needs no state, so k_forcing_steps computes it while the upload is in
// flight, and stage 1 then only adds the sparse product (k_stage1_pre):
// the same operations in the same order as k_stage<Z, 1> (bit-identical).

template <class Z>
__global__ void __launch_bounds__(256) k_stage1_pre(const StepArgs<Z> P, const Z *__restrict__ fbuf) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t NK = P.N * P.K;
  if (t >= NK) return;
  const int64_t i = P.step[0];
  if (t == 0) P.step[1] = i;
  const int64_t n = t / P.K;
  const int kc = (int)(t - n * P.K);
  Z k = P.F3[t];  // the previous step's F3
  row_product(P, n, kc, P.y, k);
  const Z yv = P.y[t];
  P.F2[t] = fbuf[t];
  P.F3[t] = fbuf[NK + t];
  P.zA[t] = zaxpy(P.dt_2, k, yv);
  P.acc[t] = zaxpy(P.dt_6, k, yv);
}

template <class Z>
static rsvdt_status forcing_ahead_t(rsvdt_ctx *ctx, int dir, int64_t i) {
  auto P = make_args<Z>(ctx, dir, true);
  const int64_t NK = P.N * P.K;
  const size_t need = sizeof(Z) * 2 * (size_t)NK;
  if (ctx->cl_bytes < need) {
    dfree(ctx, ctx->cl_fbuf);
    ctx->cl_fbuf = dalloc(ctx, need);
    ctx->cl_bytes = ctx->cl_fbuf ? need : 0;
    if (!ctx->cl_fbuf) return set_err(ctx, RSVDT_ERR_OOM, "forcing buffer allocation failed");
  }
  k_forcing_steps<Z><<<grid_for(NK, 256), 256, 0, ctx->stream>>>(P, i, 1, (Z *)ctx->cl_fbuf);
  ctx->launches += 1;
  return cuda_ok(ctx, cudaGetLastError(), "forcing") ? RSVDT_OK : RSVDT_ERR_CUDA;
}

template <class Z>
static rsvdt_status first_step_rest_t(rsvdt_ctx *ctx, int dir, int64_t i, cudaEvent_t after_stage1, int nslab,
                                      cudaEvent_t *slab_done) {
  auto P = make_args<Z>(ctx, dir, true);
  const int64_t NK = P.N * P.K;
  k_set_step<<<1, 1, 0, ctx->stream>>>(ctx->d_step, i);
  k_stage1_pre<Z><<<grid_for(NK, 256), 256, 0, ctx->stream>>>(P, (const Z *)ctx->cl_fbuf);
  if (after_stage1) cudaEventRecord(after_stage1, ctx->stream);
  ctx->launches += 2 + launch_stages_234(ctx, P, nslab, slab_done);
  return cuda_ok(ctx, cudaGetLastError(), "first step") ? RSVDT_OK : RSVDT_ERR_CUDA;
}

// Step i's forcing into the forcing buffer (stream of the context).
rsvdt_status launch_forcing_ahead(rsvdt_ctx *ctx, int dir, int prec, int64_t i) {
  return prec == RSVDT_PREC_C64 ? forcing_ahead_t<z64>(ctx, dir, i) : forcing_ahead_t<z128>(ctx, dir, i);
}

// The rest of step i once the state is on the device: stage 1 from the
// buffered forcing (after_stage1, if given, recorded after it), stages 2-4.
rsvdt_status launch_first_step_rest(rsvdt_ctx *ctx, int dir, int prec, int64_t i, cudaEvent_t after_stage1,
                                    int nslab, cudaEvent_t *slab_done) {
  return prec == RSVDT_PREC_C64 ? first_step_rest_t<z64>(ctx, dir, i, after_stage1, 1, nullptr)
                                : first_step_rest_t<z128>(ctx, dir, i, after_stage1, nslab, slab_done);
}

// Whether the cluster engine runs this context's steps (and its shape).
bool use_cluster_engine(const rsvdt_ctx *ctx, int prec, int *C, int *threads) {
  if (ctx->engine == RSVDT_ENGINE_STAGES) return false;
  const int64_t NK = ctx->N * ctx->Ks;
  if (ctx->engine == RSVDT_ENGINE_AUTO && NK > kClusterAutoMax) return false;
  *C = prec == RSVDT_PREC_C64 ? cluster_shape<z64>(NK, threads) : cluster_shape<z128>(NK, threads);
  return *C > 0;
}

rsvdt_status run_steps(rsvdt_ctx *ctx, int dir, int prec, int64_t i0, int64_t nsteps, bool) {
  int C = 0, threads = 0;
  if (nsteps > 0 && use_cluster_engine(ctx, prec, &C, &threads))
    return prec == RSVDT_PREC_C64 ? run_steps_cluster_t<z64>(ctx, dir, i0, nsteps, C, threads)
                                  : run_steps_cluster_t<z128>(ctx, dir, i0, nsteps, C, threads);
  const int fs = step_lanes(ctx);
  if (fs > 1) return run_steps_small(ctx, dir, prec, i0, nsteps, fs);
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
  int G = 0;
  if constexpr (sizeof(Z) == 8) {
    prepare_forcing_block(ctx, P, &G);
    ctx->fb_last = G;
  }
  cudaEvent_t ev[5], fb0 = nullptr, fb1 = nullptr;
  for (auto &e : ev)
    if (!cuda_ok(ctx, cudaEventCreate(&e), "event create")) return RSVDT_ERR_CUDA;
  if (G > 0 && (!cuda_ok(ctx, cudaEventCreate(&fb0), "event create") ||
                !cuda_ok(ctx, cudaEventCreate(&fb1), "event create")))
    return RSVDT_ERR_CUDA;
  k_set_step<<<1, 1, 0, ctx->stream>>>(ctx->d_step, i0);
  ctx->launches += 1;
  for (int s = 0; s < 5; ++s) stage_ms[s] = 0;
  rsvdt_status st = RSVDT_OK;
  for (int64_t n = 0; n < nsteps && st == RSVDT_OK; ++n) {
    if constexpr (sizeof(Z) == 8) {
      if (G > 0 && n % G == 0) {
        // The next block's forcing, timed on its own.
        cudaEventRecord(fb0, ctx->stream);
        launch_forcing_block(P, (int)std::min<int64_t>(G, nsteps - n), ctx->sm_count, ctx->stream);
        cudaEventRecord(fb1, ctx->stream);
        ctx->launches += 1;
        if (!cuda_ok(ctx, cudaEventSynchronize(fb1), "event sync")) {
          st = RSVDT_ERR_CUDA;
          break;
        }
        float ms = 0;
        cudaEventElapsedTime(&ms, fb0, fb1);
        stage_ms[4] += ms;
      }
    }
    cudaEventRecord(ev[0], ctx->stream);
    for (int s = 1; s <= 4; ++s) {
      launch_stage(s, P, ctx->stream);
      cudaEventRecord(ev[s], ctx->stream);
    }
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
  if (fb0) cudaEventDestroy(fb0);
  if (fb1) cudaEventDestroy(fb1);
  if (st == RSVDT_OK && !cuda_ok(ctx, cudaGetLastError(), "profile steps")) st = RSVDT_ERR_CUDA;
  return st;
}

rsvdt_status profile_steps(rsvdt_ctx *ctx, int dir, int prec, int64_t i0, int64_t nsteps,
                           double *stage_ms) {
  if (prec == RSVDT_PREC_C64) return profile_steps_t<z64>(ctx, dir, i0, nsteps, stage_ms);
  return profile_steps_t<z128>(ctx, dir, i0, nsteps, stage_ms);
}

// DFT of the sampled period (SourceCode/DFT.c:26-38), FP64 sums:
// out[n][iw][k0 + k] = ResRatio * sum_p ring[p][n][k] * dft[p][iw] for the
// ring's K test vectors (out holds Kb per frequency).
template <class Z>
__global__ void __launch_bounds__(256) k_dft(const Z *__restrict__ ring,
                                             const z128 *__restrict__ dft, int64_t N, int K,
                                             int Nw, int Nwe, double R, z128 *__restrict__ out,
                                             int32_t *flags, int Kb, int k0) {
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
  out[(n * Nwe + iw) * Kb + k0 + kc] = s;
}

// The same DFT by a radix-2 FFT when Nw is 8, 16, 32 (64: k_dft_fft64):
// one thread per (row, test vector) holds the NW samples in registers
// (loaded in bit-reversed order), NW/2 log2(NW) butterflies with the
// twiddles W^m = dft[1][m] of the reference's own table
// (SourceCode/CreateDFTiDFTMats.c:61-85), FP64 arithmetic: NW/2 log2(NW)
// complex products per output set instead of NW * Nw_eff. The first Nw_eff
// outputs are kept (all of them for a complex operator).
__device__ __forceinline__ constexpr int bit_reverse(int p, int bits) {
  int r = 0;
  for (int b = 0; b < bits; ++b) r |= ((p >> b) & 1) << (bits - 1 - b);
  return r;
}

template <class Z, int NW, int LOG>
__global__ void __launch_bounds__(128) k_dft_fft(const Z *__restrict__ ring, const z128 *__restrict__ dft,
                                                 int64_t N, int K, int Nwe, double R, z128 *__restrict__ out,
                                                 int32_t *flags, int Kb, int k0) {
  const int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (u >= N * K) return;
  const int64_t n = u / K;
  const int kc = (int)(u - n * K);
  const int64_t NK = N * K;
  double re[NW], im[NW];
#pragma unroll
  for (int p = 0; p < NW; ++p) {
    const Z v = ring[(int64_t)p * NK + u];
    re[bit_reverse(p, LOG)] = (double)v.re;
    im[bit_reverse(p, LOG)] = (double)v.im;
  }
#pragma unroll
  for (int half = 1; half < NW; half <<= 1) {
#pragma unroll
    for (int j = 0; j < half; ++j) {
      const double2 wt = __ldg(reinterpret_cast<const double2 *>(dft) + NW + j * (NW / (2 * half)));
      const z128 w = zmake<z128>(wt.x, wt.y);
#pragma unroll
      for (int i = j; i < NW; i += 2 * half) {
        const double xr = re[i + half], xi = im[i + half];
        const double tr = fma(w.re, xr, -w.im * xi), ti = fma(w.re, xi, w.im * xr);
        re[i + half] = re[i] - tr;
        im[i + half] = im[i] - ti;
        re[i] += tr;
        im[i] += ti;
      }
    }
  }
  bool ok = true;
#pragma unroll
  for (int iw = 0; iw < NW; ++iw) {
    if (iw < Nwe) {
      const z128 s = zmake<z128>(re[iw] * R, im[iw] * R);
      ok = ok && isfinite(s.re) && isfinite(s.im);
      out[(n * Nwe + iw) * Kb + k0 + kc] = s;
    }
  }
  if (!ok) atomicOr(flags, 1);
}

// Nw = 64: two lanes per (row, test vector). Lane h transforms the samples
// p = 2m + h (a 32-point FFT, twiddles W64^(2j)); the pair then exchanges
// one value per output through a shuffle: X[k] = E[k] + W64^k O[k] (lane 0),
// X[k + 32] = E[k] - W64^k O[k] (lane 1).
template <class Z>
__global__ void __launch_bounds__(128) k_dft_fft64(const Z *__restrict__ ring, const z128 *__restrict__ dft,
                                                   int64_t N, int K, int Nwe, double R, z128 *__restrict__ out,
                                                   int32_t *flags, int Kb, int k0) {
  constexpr int NW = 64, H = 32, LOG = 5;
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t u = t >> 1;
  const int h = (int)(t & 1);
  const bool valid = u < N * K;  // both lanes of a pair agree
  const int64_t uu = valid ? u : 0;
  const int64_t n = uu / K;
  const int kc = (int)(uu - n * K);
  const int64_t NK = N * K;
  double re[H], im[H];
#pragma unroll
  for (int m = 0; m < H; ++m) {
    double vr = 0, vi = 0;
    if (valid) {
      const Z v = ring[(int64_t)(2 * m + h) * NK + uu];
      vr = (double)v.re;
      vi = (double)v.im;
    }
    re[bit_reverse(m, LOG)] = vr;
    im[bit_reverse(m, LOG)] = vi;
  }
  const double2 *tw = reinterpret_cast<const double2 *>(dft) + NW;  // W64^m = dft[1][m]
#pragma unroll
  for (int half = 1; half < H; half <<= 1) {
#pragma unroll
    for (int j = 0; j < half; ++j) {
      const double2 w = __ldg(tw + 2 * j * (H / (2 * half)));
#pragma unroll
      for (int i = j; i < H; i += 2 * half) {
        const double xr = re[i + half], xi = im[i + half];
        const double tr = fma(w.x, xr, -w.y * xi), ti = fma(w.x, xi, w.y * xr);
        re[i + half] = re[i] - tr;
        im[i + half] = im[i] - ti;
        re[i] += tr;
        im[i] += ti;
      }
    }
  }
  bool ok = true;
#pragma unroll
  for (int k = 0; k < H; ++k) {
    const double pr = __shfl_xor_sync(0xffffffffu, re[k], 1), pi = __shfl_xor_sync(0xffffffffu, im[k], 1);
    // Lane 0 holds E[k] and receives O[k]; lane 1 holds O[k] and receives E[k].
    const double er = h ? pr : re[k], ei = h ? pi : im[k];
    const double orr = h ? re[k] : pr, oi = h ? im[k] : pi;
    const double2 w = __ldg(tw + k);
    const double tr = fma(w.x, orr, -w.y * oi), ti = fma(w.x, oi, w.y * orr);
    const int iw = k + h * H;
    if (valid && iw < Nwe) {
      const z128 s = zmake<z128>((h ? er - tr : er + tr) * R, (h ? ei - ti : ei + ti) * R);
      ok = ok && isfinite(s.re) && isfinite(s.im);
      out[(n * Nwe + iw) * Kb + k0 + kc] = s;
    }
  }
  if (!ok) atomicOr(flags, 1);
}

template <class Z>
static bool launch_dft_fft(rsvdt_ctx *ctx, const Z *ring, z128 *out) {
  const int64_t total = ctx->N * ctx->Ks;
  const int g = grid_for(total, 128);
  const int K = (int)ctx->Ks, Nwe = (int)ctx->Nw_eff, Kb = (int)ctx->K, k0 = (int)ctx->k0;
  const double R = (double)ctx->R;
  switch (ctx->Nw) {
    case 8: k_dft_fft<Z, 8, 3><<<g, 128, 0, ctx->stream>>>(ring, ctx->dft, ctx->N, K, Nwe, R, out, ctx->d_flags, Kb, k0); return true;
    case 16: k_dft_fft<Z, 16, 4><<<g, 128, 0, ctx->stream>>>(ring, ctx->dft, ctx->N, K, Nwe, R, out, ctx->d_flags, Kb, k0); return true;
    case 32: k_dft_fft<Z, 32, 5><<<g, 128, 0, ctx->stream>>>(ring, ctx->dft, ctx->N, K, Nwe, R, out, ctx->d_flags, Kb, k0); return true;
    case 64:
      k_dft_fft64<Z><<<grid_for(2 * total, 128), 128, 0, ctx->stream>>>(ring, ctx->dft, ctx->N, K, Nwe, R, out,
                                                                       ctx->d_flags, Kb, k0);
      return true;
    default: return false;
  }
}

// DFT of the ring (the state's Ks test vectors) into columns k0.. of `out`.
rsvdt_status launch_dft(rsvdt_ctx *ctx, int prec, z128 *out) {
  const int th = 256;
  const int64_t total = ctx->N * ctx->Nw_eff * ctx->Ks;
  const bool fft = prec == RSVDT_PREC_C64 ? launch_dft_fft<z64>(ctx, (const z64 *)ctx->ring, out)
                                          : launch_dft_fft<z128>(ctx, (const z128 *)ctx->ring, out);
  if (fft) {
  } else if (prec == RSVDT_PREC_C64)
    k_dft<z64><<<grid_for(total, th), th, 0, ctx->stream>>>(
        (const z64 *)ctx->ring, ctx->dft, ctx->N, (int)ctx->Ks, (int)ctx->Nw, (int)ctx->Nw_eff,
        (double)ctx->R, out, ctx->d_flags, (int)ctx->K, (int)ctx->k0);
  else
    k_dft<z128><<<grid_for(total, th), th, 0, ctx->stream>>>(
        (const z128 *)ctx->ring, ctx->dft, ctx->N, (int)ctx->Ks, (int)ctx->Nw, (int)ctx->Nw_eff,
        (double)ctx->R, out, ctx->d_flags, (int)ctx->K, (int)ctx->k0);
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

// Unforced RK4 (SourceCode/TSTransRK4.c:15-36) of one complex128 state
// vector y with time step dt, for the transient simulation
// (SourceCode/TransientRunRK4.c:128-130). work holds zA, zB, acc, F2, F3
// (5 N values); F2 and F3 must be zero (no forcing writes them). Full
// groups of kGraphSteps steps replay a CUDA graph cached in *graph, which
// the caller destroys.
rsvdt_status launch_trans_steps(rsvdt_ctx *ctx, double dt, z128 *y, z128 *work, int64_t nsteps,
                                cudaGraphExec_t *graph) {
  const int64_t N = ctx->N;
  auto P = make_args<z128>(ctx, 1, false);
  P.K = 1;
  P.y = y;
  P.zA = work;
  P.zB = work + N;
  P.acc = work + 2 * N;
  P.F2 = work + 3 * N;
  P.F3 = work + 4 * N;
  P.ring = nullptr;
  P.dt = dt;
  P.dt_2 = dt / 2;
  P.dt_6 = dt / 6;
  P.dt_62 = dt / 6 * 2;
  int64_t done = 0;
  if (nsteps >= kGraphSteps) {
    if (!*graph) {
      cudaGraph_t g;
      if (!cuda_ok(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal),
                   "begin capture"))
        return RSVDT_ERR_CUDA;
      for (int64_t s = 0; s < kGraphSteps; ++s) enqueue_step(ctx, P);
      if (!cuda_ok(ctx, cudaStreamEndCapture(ctx->stream, &g), "end capture")) return RSVDT_ERR_CUDA;
      const cudaError_t e = cudaGraphInstantiate(graph, g, 0);
      cudaGraphDestroy(g);
      if (!cuda_ok(ctx, e, "graph instantiate")) return RSVDT_ERR_CUDA;
    }
    for (; done + kGraphSteps <= nsteps; done += kGraphSteps)
      if (!cuda_ok(ctx, cudaGraphLaunch(*graph, ctx->stream), "graph launch")) return RSVDT_ERR_CUDA;
  }
  for (; done < nsteps; ++done) enqueue_step(ctx, P);
  ctx->launches += 4 * nsteps;
  if (!cuda_ok(ctx, cudaGetLastError(), "transient steps")) return RSVDT_ERR_CUDA;
  return RSVDT_OK;
}

// Reads and clears the debug build's index-check word (release build: OK).
rsvdt_status debug_index_status(rsvdt_ctx *ctx) {
#ifdef RSVDT_DEBUG
  unsigned int f = 0;
  if (!cuda_ok(ctx, cudaStreamSynchronize(ctx->stream), "sync") ||
      !cuda_ok(ctx, cudaMemcpyFromSymbol(&f, g_index_faults, sizeof f), "index check word"))
    return RSVDT_ERR_CUDA;
  if (f) {
    const unsigned int zero = 0;
    if (!cuda_ok(ctx, cudaMemcpyToSymbol(g_index_faults, &zero, sizeof zero), "index check word"))
      return RSVDT_ERR_CUDA;
    return set_err(ctx, RSVDT_ERR_ARG, "debug build: an index check failed in a stage kernel (sites 0x%x: "
                   "1 = CSR column, 2 = block column, 4 = ring slot)", f);
  }
#else
  (void)ctx;
#endif
  return RSVDT_OK;
}

}  // namespace rsvdt

// ------------------------------------------------------ batched stepping
//
// Many independent problems (own operator, k, Nw, time grid) advance in
// lockstep: one launch per RK4 stage covers the rows of every problem. A
// block works on one tile of one problem (work list entry (problem,
// tile)); a problem past the last step of its action (step > rend) skips.
// FS consecutive lanes share one (row, test vector): they split the
// nonzeros (and, in stage 1, the forcing slabs) and combine their partial
// sums with warp shuffles, which puts small problems on more lanes. The
// launch shape (threads per block, FS) is chosen by the batch's autotuner.

namespace rsvdt {

template <class Z>
__device__ __forceinline__ void row_product_split(const StepArgs<Z> &P, int64_t n, int kc, const Z *x, Z &acc,
                                                  int fsub, int FS) {
  const int K = P.K;
  if (P.bs == 0) {
    const int32_t b = __ldg(P.rowptr + n), e = __ldg(P.rowptr + n + 1);
    for (int32_t j = b + fsub; j < e; j += FS) {
      const int32_t cj = __ldg(P.col + j);
      if (!RSVDT_CHECK_INDEX(cj >= 0 && cj < P.N, 0)) continue;
      zmac(acc, P.val[j], x[(int64_t)cj * K + kc]);
    }
  } else {
    const int bs = P.bs;
    const int64_t br = n / bs;
    const int r = (int)(n - br * bs);
    const int32_t b = __ldg(P.rowptr + br), e = __ldg(P.rowptr + br + 1);
    for (int32_t j = b + fsub; j < e; j += FS) {
      const int32_t cb = __ldg(P.col + j);
      if (!RSVDT_CHECK_INDEX(cb >= 0 && cb < P.N / bs, 1)) continue;
      const int64_t c0 = (int64_t)cb * bs;
      const Z *blkrow = P.val + (int64_t)j * P.bstride + r * bs;
      for (int c = 0; c < bs; ++c) zmac(acc, blkrow[c], x[(c0 + c) * K + kc]);
    }
  }
}

template <class Z, int FS>
__device__ __forceinline__ void group_sum(Z &v) {
#pragma unroll
  for (int off = FS / 2; off > 0; off >>= 1) {
    v.re += __shfl_xor_sync(0xffffffffu, v.re, off);
    v.im += __shfl_xor_sync(0xffffffffu, v.im, off);
  }
}

template <class Z, int S, int FS>
__global__ void __launch_bounds__(256) k_stage_batched(const StepArgs<Z> *__restrict__ probs,
                                                       const int2 *__restrict__ work, int64_t *step) {
  pdl_wait_and_release();
  const int2 wk = work[blockIdx.x];
  const StepArgs<Z> &P = probs[wk.x];
  const int64_t i = (S == 1) ? step[0] : step[1];
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    if (S == 1) step[1] = i;
    if (S == 4) step[0] = i + 1;
  }
  if (i > P.rend) return;  // uniform over the block (one problem per block)
  // Stage 1: the step's two phasor rows in shared memory (read once per
  // slab by every thread of the block).
  constexpr int kMaxStagedNw = 128;
  __shared__ Z e_sm[S == 1 ? 2 * kMaxStagedNw : 1];
  const Z *e2 = nullptr, *e3 = nullptr;
  if (S == 1 && P.Fh) {
    int64_t j2, j3;
    step_idx(P.dir, i, P.two_ns, j2, j3);
    e2 = P.tab + j2 * P.Nw;
    e3 = P.tab + j3 * P.Nw;
    if (P.Nw <= kMaxStagedNw) {
      for (int s = threadIdx.x; s < P.Nw; s += blockDim.x) {
        e_sm[s] = e2[s];
        e_sm[kMaxStagedNw + s] = e3[s];
      }
      __syncthreads();
      e2 = e_sm;
      e3 = e_sm + kMaxStagedNw;
    }
  }
  const int64_t local = (int64_t)wk.y * blockDim.x + threadIdx.x;
  const int64_t u = local / FS;
  const int fsub = (int)(local - u * FS);
  const int64_t NK = P.N * P.K;
  const bool valid = u < NK;
  const int64_t n = valid ? u / P.K : 0;
  const int kc = valid ? (int)(u - n * P.K) : 0;
  const Z *x = (S == 1) ? P.y : (S == 2) ? P.zA : (S == 3) ? P.zB : P.zA;
  Z k = zmake<Z>(0, 0), f2 = zmake<Z>(0, 0), f3 = zmake<Z>(0, 0);
  if (valid) {
    row_product_split(P, n, kc, x, k, fsub, FS);
    if (S == 1 && P.Fh) forcing2(P, n, kc, e2, e3, fsub, FS, f2, f3);
  }
  if (FS > 1) {
    group_sum<Z, FS>(k);
    if (S == 1) {
      group_sum<Z, FS>(f2);
      group_sum<Z, FS>(f3);
    }
  }
  if (!valid || fsub != 0) return;
  const int64_t t = u;
  const Z addv = (S == 1 || S == 4) ? P.F3[t] : P.F2[t];
  k.re += addv.re;
  k.im += addv.im;
  const Z yv = P.y[t];
  if (S == 1) {
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
    if (p >= 0 && RSVDT_CHECK_INDEX(p < P.Nstore, 2)) P.ring[p * NK + t] = ynew;
  }
}

// complex64 batched stage with two test vectors per lane (every problem of
// the batch has an even k): a lane owns (row n, test vectors kc, kc+1), so
// every state, slab and gathered access is one 16-byte load or store
// instead of two 8-byte ones. Each of the two values is computed exactly as
// k_stage_batched<z64, S, 1> computes it (the same operations in the same
// order: bit-identical results).
template <int S>
__global__ void __launch_bounds__(256) k_stage_batched_pair(const StepArgs<z64> *__restrict__ probs,
                                                            const int2 *__restrict__ work, int64_t *step) {
  using Z = z64;
  pdl_wait_and_release();
  const int2 wk = work[blockIdx.x];
  const StepArgs<Z> &P = probs[wk.x];
  const int64_t i = (S == 1) ? step[0] : step[1];
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    if (S == 1) step[1] = i;
    if (S == 4) step[0] = i + 1;
  }
  if (i > P.rend) return;  // uniform over the block (one problem per block)
  constexpr int kMaxStagedNw = 128;
  __shared__ Z e_sm[S == 1 ? 2 * kMaxStagedNw : 1];
  const Z *e2 = nullptr, *e3 = nullptr;
  if (S == 1 && P.Fh) {
    int64_t j2, j3;
    step_idx(P.dir, i, P.two_ns, j2, j3);
    e2 = P.tab + j2 * P.Nw;
    e3 = P.tab + j3 * P.Nw;
    if (P.Nw <= kMaxStagedNw) {
      for (int s = threadIdx.x; s < P.Nw; s += blockDim.x) {
        e_sm[s] = e2[s];
        e_sm[kMaxStagedNw + s] = e3[s];
      }
      __syncthreads();
      e2 = e_sm;
      e3 = e_sm + kMaxStagedNw;
    }
  }
  const int64_t NK = P.N * P.K;
  const int64_t t = 2 * ((int64_t)wk.y * blockDim.x + threadIdx.x);  // first of the lane's two values
  if (t >= NK) return;
  const int K = P.K;
  const int64_t n = t / K;
  const int kc = (int)(t - n * K);
  const Z *x = (S == 1) ? P.y : (S == 2) ? P.zA : (S == 3) ? P.zB : P.zA;
  Z k[2] = {zmake<Z>(0, 0), zmake<Z>(0, 0)};
  if (P.bs == 0) {
    const int32_t b = __ldg(P.rowptr + n), e = __ldg(P.rowptr + n + 1);
    for (int32_t j = b; j < e; ++j) {
      const int32_t cj = __ldg(P.col + j);
      if (!RSVDT_CHECK_INDEX(cj >= 0 && cj < P.N, 0)) continue;
      const Z a = P.val[j];
      Z xv[2];
      ld_chunk<Z, 2>(x + (int64_t)cj * K + kc, xv);
      zmac(k[0], a, xv[0]);
      zmac(k[1], a, xv[1]);
    }
  } else {
    const int bs = P.bs;
    const int64_t br = n / bs;
    const int r = (int)(n - br * bs);
    const int32_t b = __ldg(P.rowptr + br), e = __ldg(P.rowptr + br + 1);
    for (int32_t j = b; j < e; ++j) {
      const int32_t cb = __ldg(P.col + j);
      if (!RSVDT_CHECK_INDEX(cb >= 0 && cb < P.N / bs, 1)) continue;
      const int64_t c0 = (int64_t)cb * bs;
      const Z *blkrow = P.val + (int64_t)j * P.bstride + r * bs;
      for (int c = 0; c < bs; ++c) {
        Z xv[2];
        ld_chunk<Z, 2>(x + (c0 + c) * K + kc, xv);
        zmac(k[0], blkrow[c], xv[0]);
        zmac(k[1], blkrow[c], xv[1]);
      }
    }
  }
  Z f2[2] = {zmake<Z>(0, 0), zmake<Z>(0, 0)}, f3[2] = {zmake<Z>(0, 0), zmake<Z>(0, 0)};
  if (S == 1 && P.Fh) {
    const Z *c = P.Fh + t;
    if (!P.pair) {
#pragma unroll 4
      for (int s = 0; s < P.Nw; ++s) {
        Z v[2];
        ldg_chunk<Z, 2>(c + (int64_t)s * NK, v);
        for (int q = 0; q < 2; ++q) {
          zmac(f2[q], v[q], e2[s]);
          zmac(f3[q], v[q], e3[s]);
        }
      }
    } else {
      const int H = P.Nw / 2, last = P.Nw - 1;
      Z v[2];
      ldg_chunk<Z, 2>(c, v);
      for (int q = 0; q < 2; ++q) {
        zmac(f2[q], v[q], e2[0]);
        zmac(f3[q], v[q], e3[0]);
      }
      int s = 1;
#pragma unroll 4
      for (; s < H; ++s) {
        ldg_chunk<Z, 2>(c + (int64_t)s * NK, v);
        const auto w2 = e2[s].re, w3 = e3[s].re;
        for (int q = 0; q < 2; ++q) {
          f2[q].re = fma(w2, v[q].re, f2[q].re);
          f2[q].im = fma(w2, v[q].im, f2[q].im);
          f3[q].re = fma(w3, v[q].re, f3[q].re);
          f3[q].im = fma(w3, v[q].im, f3[q].im);
        }
      }
#pragma unroll 4
      for (; s < last; ++s) {
        ldg_chunk<Z, 2>(c + (int64_t)s * NK, v);
        const auto w2 = e2[s - H + 1].im, w3 = e3[s - H + 1].im;
        for (int q = 0; q < 2; ++q) {
          f2[q].re = fma(w2, v[q].re, f2[q].re);
          f2[q].im = fma(w2, v[q].im, f2[q].im);
          f3[q].re = fma(w3, v[q].re, f3[q].re);
          f3[q].im = fma(w3, v[q].im, f3[q].im);
        }
      }
      ldg_chunk<Z, 2>(c + (int64_t)last * NK, v);
      for (int q = 0; q < 2; ++q) {
        zmac(f2[q], v[q], e2[H]);
        zmac(f3[q], v[q], e3[H]);
      }
    }
  }
  Z addv[2], yv[2], t2[2];
  ld_chunk<Z, 2>(((S == 1 || S == 4) ? P.F3 : P.F2) + t, addv);
  for (int q = 0; q < 2; ++q) {
    k[q].re += addv[q].re;
    k[q].im += addv[q].im;
  }
  ld_chunk<Z, 2>(P.y + t, yv);
  if (S == 1) {
    st_chunk<Z, 2>(P.F2 + t, f2);
    st_chunk<Z, 2>(P.F3 + t, f3);
    for (int q = 0; q < 2; ++q) t2[q] = zaxpy(P.dt_2, k[q], yv[q]);
    st_chunk<Z, 2>(P.zA + t, t2);
    for (int q = 0; q < 2; ++q) t2[q] = zaxpy(P.dt_6, k[q], yv[q]);
    st_chunk<Z, 2>(P.acc + t, t2);
  } else if (S == 2 || S == 3) {
    Z av[2];
    for (int q = 0; q < 2; ++q) t2[q] = zaxpy(S == 2 ? P.dt_2 : P.dt, k[q], yv[q]);
    st_chunk<Z, 2>((S == 2 ? P.zB : P.zA) + t, t2);
    ld_chunk<Z, 2>(P.acc + t, av);
    for (int q = 0; q < 2; ++q) t2[q] = zaxpy(P.dt_62, k[q], av[q]);
    st_chunk<Z, 2>(P.acc + t, t2);
  } else {
    Z av[2];
    ld_chunk<Z, 2>(P.acc + t, av);
    for (int q = 0; q < 2; ++q) t2[q] = zaxpy(P.dt_6, k[q], av[q]);
    st_chunk<Z, 2>(P.y + t, t2);
    const int64_t p = P.ring ? ring_slot(P.dir, i, P.Nt, P.R, P.Nstore) : -1;
    if (p >= 0 && RSVDT_CHECK_INDEX(p < P.Nstore, 2)) st_chunk<Z, 2>(P.ring + p * NK + t, t2);
  }
}

size_t step_args_size(int prec) { return prec == RSVDT_PREC_C64 ? sizeof(StepArgs<z64>) : sizeof(StepArgs<z128>); }

// Host copy of ctx's stage arguments for direction dir with the batch's
// shared step counter and the action's last step.
void fill_step_args(rsvdt_ctx *ctx, int dir, int prec, int64_t rend, int64_t *shared_step, void *out) {
  if (prec == RSVDT_PREC_C64) {
    auto P = make_args<z64>(ctx, dir, true);
    P.step = shared_step;
    P.rend = rend;
    memcpy(out, &P, sizeof P);
  } else {
    auto P = make_args<z128>(ctx, dir, true);
    P.step = shared_step;
    P.rend = rend;
    memcpy(out, &P, sizeof P);
  }
}

template <class Z, int FS>
static void launch_batched_fs(cudaStream_t st, const void *args, const int2 *work, int nwork, int threads,
                              int64_t *step) {
  const StepArgs<Z> *P = (const StepArgs<Z> *)args;
  launch_pdl(k_stage_batched<Z, 1, FS>, nwork, threads, 0, st, P, work, step);
  launch_pdl(k_stage_batched<Z, 2, FS>, nwork, threads, 0, st, P, work, step);
  launch_pdl(k_stage_batched<Z, 3, FS>, nwork, threads, 0, st, P, work, step);
  launch_pdl(k_stage_batched<Z, 4, FS>, nwork, threads, 0, st, P, work, step);
}

template <class Z>
static bool launch_batched_t(cudaStream_t st, const void *args, const int2 *work, int nwork, int threads, int fs,
                             int64_t *step) {
  switch (fs) {
    case 1: launch_batched_fs<Z, 1>(st, args, work, nwork, threads, step); return true;
    case 2: launch_batched_fs<Z, 2>(st, args, work, nwork, threads, step); return true;
    case 4: launch_batched_fs<Z, 4>(st, args, work, nwork, threads, step); return true;
    case 8: launch_batched_fs<Z, 8>(st, args, work, nwork, threads, step); return true;
    default: return false;
  }
}

// One batched RK4 step (four launches) on stream st. kv = 2 (complex64,
// fs = 1, every problem's k even): two test vectors per lane.
bool launch_batched_step(cudaStream_t st, int prec, const void *args, const int2 *work, int nwork, int threads,
                         int fs, int64_t *step, int kv) {
  if (kv == 2) {
    if (prec != RSVDT_PREC_C64 || fs != 1) return false;
    const StepArgs<z64> *P = (const StepArgs<z64> *)args;
    launch_pdl(k_stage_batched_pair<1>, nwork, threads, 0, st, P, work, step);
    launch_pdl(k_stage_batched_pair<2>, nwork, threads, 0, st, P, work, step);
    launch_pdl(k_stage_batched_pair<3>, nwork, threads, 0, st, P, work, step);
    launch_pdl(k_stage_batched_pair<4>, nwork, threads, 0, st, P, work, step);
    return true;
  }
  if (prec == RSVDT_PREC_C64) return launch_batched_t<z64>(st, args, work, nwork, threads, fs, step);
  return launch_batched_t<z128>(st, args, work, nwork, threads, fs, step);
}

void launch_set_step(cudaStream_t st, int64_t *step, int64_t i) { k_set_step<<<1, 1, 0, st>>>(step, i); }

}  // namespace rsvdt
