// Shared definitions of the GB300 RSVD-Delta-t library: complex arithmetic,
// device buffers, the context, launch helpers.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "rsvdt.h"

namespace rsvdt {

// ------------------------------------------------------------------ complex

template <class R>
struct cplx {
  R re, im;
};
template <class R>
struct alignas(2 * sizeof(R)) cplx_a {
  R re, im;
};
using z128 = cplx_a<double>;  // 16-byte aligned complex128
using z64 = cplx_a<float>;    // 8-byte aligned complex64

template <class Z>
struct real_of;
template <>
struct real_of<z128> {
  using type = double;
};
template <>
struct real_of<z64> {
  using type = float;
};

template <class Z>
__host__ __device__ __forceinline__ Z zmake(typename real_of<Z>::type r,
                                            typename real_of<Z>::type i) {
  Z z;
  z.re = r;
  z.im = i;
  return z;
}

// acc += a * x (complex multiply-accumulate, 4 FMA).
template <class Z>
__device__ __forceinline__ void zmac(Z &acc, const Z a, const Z x) {
  acc.re = fma(a.re, x.re, acc.re);
  acc.re = fma(-a.im, x.im, acc.re);
  acc.im = fma(a.re, x.im, acc.im);
  acc.im = fma(a.im, x.re, acc.im);
}
// acc += conj(a) * x
template <class Z>
__device__ __forceinline__ void zmacc(Z &acc, const Z a, const Z x) {
  acc.re = fma(a.re, x.re, acc.re);
  acc.re = fma(a.im, x.im, acc.re);
  acc.im = fma(a.re, x.im, acc.im);
  acc.im = fma(-a.im, x.re, acc.im);
}
// s * x + y with real s (VecWAXPY / VecAXPY with a real coefficient).
template <class Z>
__device__ __forceinline__ Z zaxpy(typename real_of<Z>::type s, const Z x, const Z y) {
  Z r;
  r.re = fma(s, x.re, y.re);
  r.im = fma(s, x.im, y.im);
  return r;
}
template <class Z>
__device__ __forceinline__ Z zmul(const Z a, const Z b) {
  Z r;
  r.re = a.re * b.re - a.im * b.im;
  r.im = a.re * b.im + a.im * b.re;
  return r;
}

// ---------------------------------------------------------------- buffers

struct DevBuf {
  void *p = nullptr;
  size_t bytes = 0;
};

// Device sparse matrix, CSR with int32 indices (rows, cols < 2^31).
struct DevCSR {
  bool present = false;
  bool diag = false;  // nonzeros are exactly the diagonal
  int64_t rows = 0, cols = 0, nnz = 0;
  int32_t *rowptr = nullptr;
  int32_t *col = nullptr;
  z128 *val = nullptr;
  z64 *val32 = nullptr;  // complex64 copy for the precision form
};

// Block-CSR operator with dense bs x bs blocks (row-major inside a block).
struct DevBCSR {
  bool present = false;
  int32_t bs = 0;
  int64_t nb = 0, nblocks = 0;
  int32_t *browptr = nullptr;
  int32_t *bcol = nullptr;
  z128 *val = nullptr;
  z64 *val32 = nullptr;
  // Complex64 values per block in val32: bs*bs, padded to 26 for 5x5
  // blocks so that every block starts on a 16-byte boundary.
  int32_t stride32 = 0;
};

}  // namespace rsvdt

struct rsvdt_ctx {
  rsvdt_params par{};
  // Derived grid (SourceCode/SetupTimeFreqGrid.c:16-21).
  double w = 0, dt = 0;
  int64_t Ns = 0, Nt = 0, R = 0, Nw = 0, Nw_eff = 0, K = 0;
  int64_t N = 0, Nb = 0, Nc = 0;
  bool real_op = false;
  bool pair = false;  // forcing slabs hold +-f pairs (complex operator, even Nw)
  bool have_operator = false;
  bool have_block = false;
  bool have_results = false;

  int device = 0;
  cudaStream_t stream = nullptr;
  bool owns_stream = true;  // false when the stream belongs to a batch
  // rsvdt_rk4_steps: a second stream and an event for reading F3 back while
  // the last step's stages 2-4 run (created on first use).
  cudaStream_t io_stream = nullptr;
  cudaEvent_t io_event = nullptr, up_event = nullptr;
  // ... and one event per row slab of the last stage 4 (y downloaded by slab).
  static constexpr int kIoSlabs = 4;
  cudaEvent_t slab_event[kIoSlabs] = {nullptr, nullptr, nullptr, nullptr};
  int64_t launches = 0;
  std::string err;

  // Operator and its conjugate transpose.
  rsvdt::DevCSR A, AH;
  rsvdt::DevBCSR BA, BAH;
  rsvdt::DevCSR W[5], WH[5];

  // Spectral blocks, layout [row][iw][k] (complex128).
  int64_t blk_rows = 0;  // rows of the working block
  rsvdt::z128 *blk = nullptr;
  rsvdt::z128 *blk2 = nullptr;
  rsvdt::z128 *Ublk = nullptr;
  int64_t U_rows = 0;
  rsvdt::z128 *Vblk = nullptr;
  double *S = nullptr;  // [iw][k] gains
  size_t blk_elems = 0; // capacity of blk/blk2 in complex values

  // Forcing coefficients of the running action as frequency slabs
  // [slab][n][k] (pair or plain, see step.cu).
  void *Fh = nullptr;
  // RK4 state, each N*K interleaved [n][k].
  void *y = nullptr, *zA = nullptr, *zB = nullptr, *acc = nullptr, *F2 = nullptr, *F3 = nullptr;
  void *ring = nullptr;  // [Nstore][n][k]
  int64_t Nstore = 0;
  // Phasor tables: idft^T [2Ns][Nw_eff] (complex128 and complex64 copies),
  // dft [Nw][Nw_eff].
  rsvdt::z128 *tab = nullptr;
  rsvdt::z64 *tab32 = nullptr;
  rsvdt::z128 *dft = nullptr;
  // Device step counters (see step.cu) and status flags.
  int64_t *d_step = nullptr;
  int32_t *d_flags = nullptr;
  // Scratch for the dense stages.
  void *scratch = nullptr;
  size_t scratch_bytes = 0;

  // Precision of the running action (rsvdt_precision's C128 or C64).
  int act_prec = 0;
  // Version of the working block's contents (bumped by every call that
  // writes it) and the version / precision the forcing slabs were staged
  // from, so that repeated rsvdt_rk4_steps calls restage only when needed.
  uint64_t blk_version = 1, staged_version = 0;
  int staged_prec = -1;
  // Wall time per phase (seconds; phases end at a stream synchronisation)
  // for rsvdt_get_timings.
  struct PhaseTimes {
    double prepare = 0, stepping = 0, finish = 0, qr = 0, svd = 0;
    int64_t actions[2] = {0, 0}, steps = 0;
  } tm;
  // Persistent host-transfer staging for rsvdt_rk4_steps.
  rsvdt::z128 *io_stage = nullptr;
  size_t io_bytes = 0;
  // Test vectors held by the RK4 state, ring and forcing slabs (Ks = K, or
  // the chunk size in capacity mode) and the first of them in the block.
  int64_t Ks = 0, k0 = 0;
  // Capacity mode: actions by chunks of cap_kc test vectors written in
  // place, no ping-pong block, U kept in host memory (per chunk, row layout
  // [row][iw][kc], complex128 or complex64).
  bool capacity = false, buf_capacity = false;
  int64_t cap_kc = 0;
  int cap_u_c64 = 0;
  std::vector<std::vector<unsigned char>> u_host;
  // Cached CUDA graphs of G RK4 steps per direction, and their precision.
  cudaGraphExec_t step_graph[2] = {nullptr, nullptr};
  int step_graph_prec[2] = {-1, -1};
  // Small-problem stepping on the batched stage kernel (step.cu:
  // step_lanes): lanes per row (0 = chosen from the size), the argument
  // blocks of both directions, the work list and the cached graphs.
  int lanes_override = 0;
  // Forcing blocks of the complex64 block-row stages (rsvdt_set_forcing_block:
  // -1 = automatic, 0 = synthesised in stage 1, else the block length),
  // their buffer, and the block length each cached step graph was captured
  // with.
  int fb_steps = -1;
  void *fblk = nullptr;
  size_t fb_bytes = 0;
  void *fb_ptr = nullptr;  // the block buffer the cached graphs use
  size_t Fh_bytes = 0;     // bytes allocated for the slabs (Fh)
  int step_graph_fb[2] = {-1, -1};
  int fb_last = 0;  // block length of the last complex64 stepping (0: none)
  int sm_count = 0;
  // rsvdt_step_engine, and the cluster engine's forcing buffer.
  int engine = RSVDT_ENGINE_AUTO;
  void *cl_fbuf = nullptr;
  size_t cl_bytes = 0;
  // rsvdt_set_checkpoint: called after the second QR of every power sweep.
  rsvdt_checkpoint_fn ckpt_fn = nullptr;
  void *ckpt_user = nullptr;
  void *small_args = nullptr;
  int2 *small_work = nullptr;
  int small_nwork = 0;
  cudaGraphExec_t small_graph[2] = {nullptr, nullptr};
  int small_graph_key[2] = {-1, -1};
  int64_t step_graph_len = 0;

  std::vector<void *> allocations;
};

namespace rsvdt {

// An NVTX range for the lifetime of the object (one per action, QR, SVD,
// transient run and batched action), so that profiles group the kernels by
// phase; costs nothing without a profiler attached.
struct NvtxRange {
  explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange &) = delete;
  NvtxRange &operator=(const NvtxRange &) = delete;
};

// Stage precision of an action under a params precision: complex128 for the
// plain form, complex64 for both precision forms.
inline int base_precision(int precision) {
  return precision == RSVDT_PREC_C128 ? RSVDT_PREC_C128 : RSVDT_PREC_C64;
}

// Returns false and records the message when a CUDA call failed.
bool cuda_ok(rsvdt_ctx *ctx, cudaError_t e, const char *what);
rsvdt_status set_err(rsvdt_ctx *ctx, rsvdt_status s, const char *fmt, ...);
// Allocates device memory tracked by the context (freed in rsvdt_destroy).
void *dalloc(rsvdt_ctx *ctx, size_t bytes);
void dfree(rsvdt_ctx *ctx, void *p);

inline int grid_for(int64_t n, int threads) {
  int64_t g = (n + threads - 1) / threads;
  return (int)(g < 1 ? 1 : g);
}

// ------------------------------------------------- kernels (launchers)
// api.cu (the two halves of an action around the RK4 steps)
rsvdt_status action_prepare(rsvdt_ctx *ctx, int dir, int64_t *rend);
rsvdt_status action_finish(rsvdt_ctx *ctx, int dir);
// step.cu
rsvdt_status stage_forcing_coeffs(rsvdt_ctx *ctx, int prec);
rsvdt_status launch_forcing_init(rsvdt_ctx *ctx, int dir, int prec);
rsvdt_status run_steps(rsvdt_ctx *ctx, int dir, int prec, int64_t i0, int64_t nsteps,
                       bool sample);
// stage_ms[0..3]: the four stages; stage_ms[4]: the forcing-block kernel
// (0 when stage 1 synthesises the forcing).
rsvdt_status profile_steps(rsvdt_ctx *ctx, int dir, int prec, int64_t i0, int64_t nsteps,
                           double *stage_ms);
rsvdt_status launch_dft(rsvdt_ctx *ctx, int prec, z128 *out);
// Batched stepping of many contexts (step.cu); the argument blocks are
// step_args_size(prec) bytes each.
size_t step_args_size(int prec);
void fill_step_args(rsvdt_ctx *ctx, int dir, int prec, int64_t rend, int64_t *shared_step, void *out);
bool launch_batched_step(cudaStream_t st, int prec, const void *args, const int2 *work, int nwork, int threads,
                         int fs, int64_t *step, int kv = 1);
void launch_set_step(cudaStream_t st, int64_t *step, int64_t i);
rsvdt_status launch_unforced_steps(rsvdt_ctx *ctx, int dir, z128 *cols, int64_t ncols,
                                   int64_t nsteps);
int step_lanes(const rsvdt_ctx *ctx);
bool use_cluster_engine(const rsvdt_ctx *ctx, int prec, int *C, int *threads);
// The last step of rsvdt_rk4_steps with events for the host transfers: after
// stage 1 (F3 final) and, with slab_done, after each of nslab row slabs of
// stage 4 (those rows of y final); stage4_slab_count says how many slabs
// the step's stage-4 kernel can take (1: slab_done[0] follows the whole).
int stage4_slab_count(rsvdt_ctx *ctx, int dir, int prec, int want);
rsvdt_status run_last_step_split(rsvdt_ctx *ctx, int dir, int prec, int64_t i, cudaEvent_t after_stage1,
                                 int nslab = 1, cudaEvent_t *slab_done = nullptr);
rsvdt_status launch_forcing_ahead(rsvdt_ctx *ctx, int dir, int prec, int64_t i);
rsvdt_status launch_first_step_rest(rsvdt_ctx *ctx, int dir, int prec, int64_t i, cudaEvent_t after_stage1,
                                    int nslab = 1, cudaEvent_t *slab_done = nullptr);
rsvdt_status debug_index_status(rsvdt_ctx *ctx);
rsvdt_status launch_trans_steps(rsvdt_ctx *ctx, double dt, z128 *y, z128 *work, int64_t nsteps,
                                cudaGraphExec_t *graph);
// dense.cu
rsvdt_status launch_colmajor_to_blk(rsvdt_ctx *ctx, const z128 *src, int64_t rows, int64_t ld,
                                    int64_t C, z128 *dst);
rsvdt_status launch_blk_to_colmajor(rsvdt_ctx *ctx, const z128 *src, int64_t rows, int64_t C,
                                    z128 *dst, int64_t ld, cudaStream_t st = nullptr);
// Complex64 state <-> complex128 host layout (rsvdt_rk4_steps in the
// precision form): the same transposes, rounding to / widening from
// complex64.
rsvdt_status launch_colmajor_to_blk64(rsvdt_ctx *ctx, const z128 *src, int64_t rows, int64_t ld,
                                      int64_t C, z64 *dst);
rsvdt_status launch_blk64_to_colmajor(rsvdt_ctx *ctx, const z64 *src, int64_t rows, int64_t C,
                                      z128 *dst, int64_t ld);
rsvdt_status apply_weight(rsvdt_ctx *ctx, const DevCSR &M, const z128 *in, z128 *out,
                          int64_t C);
rsvdt_status cholqr2(rsvdt_ctx *ctx, z128 *blk, int64_t rows, int64_t nw, int64_t K,
                     z128 *Rout);
rsvdt_status svd_all(rsvdt_ctx *ctx, z128 *blk, int64_t rows, int64_t nw, int64_t K,
                     z128 *Uout, double *S);
rsvdt_status launch_random(rsvdt_ctx *ctx, z128 *dst, int64_t n, uint64_t seed);
rsvdt_status launch_convert_to64(rsvdt_ctx *ctx, const z128 *src, z64 *dst, int64_t n);
rsvdt_status check_finite(rsvdt_ctx *ctx, const z128 *p, int64_t n, bool *ok);
rsvdt_status transient_removal(rsvdt_ctx *ctx, int dir, int prec, z128 *out);
rsvdt_status launch_chunk_copy(rsvdt_ctx *ctx, const z128 *src, z128 *dst, int64_t rows, int64_t Nwe, int64_t Kb,
                               int64_t k0, int64_t Kc, bool gather);

}  // namespace rsvdt
