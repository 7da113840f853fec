// Batching form: many independent resolvent problems of uneven size (own
// operator, k, Nw and time grid) solved together on one GPU.
//
// Each problem is an ordinary context (its own device buffers) whose work
// is issued on the batch's single stream. Every action of the RSVD-Delta-t
// sequence (SourceCode/main.c:134-144) runs for all problems at once: the
// per-problem halves before and after the time stepping (weights, forcing
// slabs, DFT) are issued problem by problem, and the RK4 steps of all
// problems advance in lockstep, one launch per RK4 stage covering every
// problem's rows (k_stage_batched), replayed from a CUDA graph of 16 steps.
// A problem whose action is shorter stops at its own last step. The launch
// shape (threads per block, lanes per row) is chosen once per batch by
// timing a few steps of each candidate on the actual problems.
#include <algorithm>
#include <cstdarg>
#include <cstring>
#include <string>
#include <vector>

#include "common.cuh"

using namespace rsvdt;

struct rsvdt_batch {
  int prec = RSVDT_PREC_C128;  // stage precision of the actions (C128 or C64)
  bool refine = false;         // the last adjoint action in complex128
  cudaStream_t stream = nullptr;
  std::vector<rsvdt_ctx *> probs;
  std::string err;
  int64_t *d_step = nullptr;
  void *d_args[2] = {nullptr, nullptr};  // per direction: nprob argument blocks
  void *d_args128[2] = {nullptr, nullptr};  // complex128 blocks of the refinement form's last action
  std::vector<unsigned char> h_args;
  int2 *d_work = nullptr;
  int nwork = 0;
  // With two values per lane, the one-value list of the same shape for the
  // refinement form's complex128 action.
  int2 *d_work1 = nullptr;
  int nwork1 = 0;
  int threads = 0, fs = 0, kv = 1;  // launch shape: threads, lanes per value, values per lane
  double tuned_ms = 0;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  cudaGraphExec_t graph128[2] = {nullptr, nullptr};
  bool ready = false;
  int64_t launches = 0;  // batched stage launches (shared by all problems)
};

static const int kBatchGraphSteps = 16;

static rsvdt_status bfail(rsvdt_batch *b, rsvdt_status st, const char *fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  b->err = buf;
  return st;
}

static rsvdt_status from_ctx(rsvdt_batch *b, size_t p, rsvdt_status st) {
  if (st != RSVDT_OK) b->err = "problem " + std::to_string(p) + ": " + rsvdt_last_error(b->probs[p]);
  return st;
}

static bool bcuda(rsvdt_batch *b, cudaError_t e, const char *what) {
  if (e == cudaSuccess) return true;
  b->err = std::string("CUDA error in ") + what + ": " + cudaGetErrorString(e);
  return false;
}

static void free_batch_graphs(rsvdt_batch *b) {
  for (auto *gs : {b->graph, b->graph128})
    for (int d = 0; d < 2; ++d)
      if (gs[d]) {
        cudaGraphExecDestroy(gs[d]);
        gs[d] = nullptr;
      }
}

// Argument blocks and graphs of the actions in precision `prec`.
static void **args_for(rsvdt_batch *b, int prec) { return prec == b->prec ? b->d_args : b->d_args128; }
static cudaGraphExec_t *graphs_for(rsvdt_batch *b, int prec) { return prec == b->prec ? b->graph : b->graph128; }

// Work list (problem, tile) for a launch shape into *dst / *n.
static rsvdt_status build_list(rsvdt_batch *b, int threads, int fs, int kv, int2 **dst, int *n) {
  std::vector<int2> w;
  for (size_t p = 0; p < b->probs.size(); ++p) {
    const int64_t nk = b->probs[p]->N * b->probs[p]->K * fs / kv;
    const int64_t tiles = (nk + threads - 1) / threads;
    for (int64_t t = 0; t < tiles; ++t) w.push_back(make_int2((int)p, (int)t));
  }
  if (*dst) cudaFree(*dst);
  *dst = nullptr;
  if (!bcuda(b, cudaMalloc(dst, sizeof(int2) * std::max<size_t>(w.size(), 1)), "work list")) return RSVDT_ERR_OOM;
  if (!bcuda(b, cudaMemcpy(*dst, w.data(), sizeof(int2) * w.size(), cudaMemcpyHostToDevice), "work list"))
    return RSVDT_ERR_CUDA;
  *n = (int)w.size();
  return RSVDT_OK;
}

static rsvdt_status build_work(rsvdt_batch *b, int threads, int fs, int kv) {
  rsvdt_status st = build_list(b, threads, fs, kv, &b->d_work, &b->nwork);
  if (st || kv == 1 || !b->refine) return st;
  return build_list(b, threads, fs, 1, &b->d_work1, &b->nwork1);
}

// Argument blocks of every problem for direction d; rend[p] = 0 leaves a
// problem out of this action.
static rsvdt_status upload_args(rsvdt_batch *b, int d, const std::vector<int64_t> &rend, int prec) {
  const size_t sz = step_args_size(prec);
  b->h_args.resize(sz * b->probs.size());
  for (size_t p = 0; p < b->probs.size(); ++p)
    fill_step_args(b->probs[p], d, prec, rend[p], b->d_step, b->h_args.data() + p * sz);
  if (!bcuda(b, cudaMemcpyAsync(args_for(b, prec)[d], b->h_args.data(), b->h_args.size(), cudaMemcpyHostToDevice,
                                b->stream),
             "arguments"))
    return RSVDT_ERR_CUDA;
  // The host buffer is reused at the next action: wait for the copy.
  return bcuda(b, cudaStreamSynchronize(b->stream), "sync") ? RSVDT_OK : RSVDT_ERR_CUDA;
}

static rsvdt_status capture(rsvdt_batch *b, int d, int prec) {
  cudaGraph_t g;
  if (!bcuda(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal), "begin capture"))
    return RSVDT_ERR_CUDA;
  // The refinement form's complex128 action takes one value per lane.
  const bool own = prec == b->prec || b->kv == 1;
  for (int s = 0; s < kBatchGraphSteps; ++s)
    launch_batched_step(b->stream, prec, args_for(b, prec)[d], own ? b->d_work : b->d_work1,
                        own ? b->nwork : b->nwork1, b->threads, b->fs, b->d_step, prec == b->prec ? b->kv : 1);
  if (!bcuda(b, cudaStreamEndCapture(b->stream, &g), "end capture")) return RSVDT_ERR_CUDA;
  const cudaError_t e = cudaGraphInstantiate(&graphs_for(b, prec)[d], g, 0);
  cudaGraphDestroy(g);
  if (!bcuda(b, e, "graph instantiate")) return RSVDT_ERR_CUDA;
  return RSVDT_OK;
}

// Times `steps` batched steps of direction d for each candidate launch
// shape; keeps the fastest. The problems' state is re-initialised by the
// caller afterwards.
static rsvdt_status autotune(rsvdt_batch *b, int d) {
  static const int cand_threads[] = {128, 256};
  // (lanes per value, values per lane); two values per lane only for
  // complex64 stages with every problem's k even.
  static const int cand_shape[][2] = {{1, 1}, {2, 1}, {4, 1}, {8, 1}, {1, 2}};
  bool even_k = true;
  for (auto *c : b->probs) even_k = even_k && c->K % 2 == 0;
  const int steps = 8;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  double best = 1e30;
  int bt = 0, bf = 0, bk = 1;
  for (int th : cand_threads)
    for (const auto &shape : cand_shape) {
      const int fs = shape[0], kv = shape[1];
      if (kv == 2 && (b->prec != RSVDT_PREC_C64 || !even_k)) continue;
      rsvdt_status st = build_work(b, th, fs, kv);
      if (st) return st;
      for (int rep = 0; rep < 2; ++rep) {  // first repetition warms up
        launch_set_step(b->stream, b->d_step, 1);
        cudaEventRecord(e0, b->stream);
        for (int s = 0; s < steps; ++s)
          launch_batched_step(b->stream, b->prec, b->d_args[d], b->d_work, b->nwork, th, fs, b->d_step, kv);
        cudaEventRecord(e1, b->stream);
        if (!bcuda(b, cudaEventSynchronize(e1), "autotune")) return RSVDT_ERR_CUDA;
      }
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      if (ms / steps < best) {
        best = ms / steps;
        bt = th;
        bf = fs;
        bk = kv;
      }
    }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  b->threads = bt;
  b->fs = bf;
  b->kv = bk;
  b->tuned_ms = best;
  return build_work(b, bt, bf, bk);
}

// One action (direct d = 1 or adjoint d = 0) of every problem in `mask`,
// stages in precision `prec`.
static rsvdt_status batch_action(rsvdt_batch *b, int d, const std::vector<char> &mask, int prec) {
  NvtxRange range(d ? "rsvdt batched direct action" : "rsvdt batched adjoint action");
  const size_t np = b->probs.size();
  std::vector<int64_t> rend(np, 0);
  int64_t maxrend = 0;
  for (size_t p = 0; p < np; ++p) {
    if (!mask[p]) continue;
    b->probs[p]->act_prec = prec;
    rsvdt_status st = from_ctx(b, p, action_prepare(b->probs[p], d, &rend[p]));
    if (st) return st;
    maxrend = std::max(maxrend, rend[p]);
  }
  rsvdt_status st = upload_args(b, d, rend, prec);
  if (st) return st;
  if (!b->threads) {
    st = autotune(b, d);
    if (st) return st;
    // Re-initialise y and the starting forcing after the timed steps.
    for (size_t p = 0; p < np; ++p)
      if (mask[p] && (st = from_ctx(b, p, launch_forcing_init(b->probs[p], d, prec)))) return st;
  }
  cudaGraphExec_t *gs = graphs_for(b, prec);
  if (!gs[d] && (st = capture(b, d, prec))) return st;
  launch_set_step(b->stream, b->d_step, 1);
  for (int64_t s = 0; s < maxrend; s += kBatchGraphSteps)
    if (!bcuda(b, cudaGraphLaunch(gs[d], b->stream), "graph launch")) return RSVDT_ERR_CUDA;
  if (!bcuda(b, cudaGetLastError(), "batched steps")) return RSVDT_ERR_CUDA;
  b->launches += 1 + (maxrend + kBatchGraphSteps - 1) / kBatchGraphSteps * kBatchGraphSteps * 4;
  for (size_t p = 0; p < np; ++p)
    if (mask[p] && (st = from_ctx(b, p, action_finish(b->probs[p], d)))) return st;
  for (size_t p = 0; p < np; ++p) b->probs[p]->act_prec = b->prec;
  return RSVDT_OK;
}

extern "C" {

rsvdt_status rsvdt_batch_create(int32_t precision, rsvdt_batch **out) {
  if (!out) return RSVDT_ERR_ARG;
  rsvdt_batch *b = new rsvdt_batch();
  *out = b;
  if (precision != RSVDT_PREC_C128 && precision != RSVDT_PREC_C64 && precision != RSVDT_PREC_C64_REFINE)
    return bfail(b, RSVDT_ERR_ARG, "unknown precision %d", (int)precision);
  b->prec = base_precision(precision);
  b->refine = precision == RSVDT_PREC_C64_REFINE;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return bfail(b, RSVDT_ERR_CUDA, "no CUDA device available");
  }
  if (!bcuda(b, cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking), "stream")) return RSVDT_ERR_CUDA;
  if (!bcuda(b, cudaMalloc(&b->d_step, sizeof(int64_t) * 2), "step counter")) return RSVDT_ERR_OOM;
  return RSVDT_OK;
}

void rsvdt_batch_destroy(rsvdt_batch *b) {
  if (!b) return;
  if (b->stream) cudaStreamSynchronize(b->stream);
  free_batch_graphs(b);
  for (auto *c : b->probs) rsvdt_destroy(c);
  for (auto p : b->d_args)
    if (p) cudaFree(p);
  for (auto p : b->d_args128)
    if (p) cudaFree(p);
  if (b->d_work) cudaFree(b->d_work);
  if (b->d_work1) cudaFree(b->d_work1);
  if (b->d_step) cudaFree(b->d_step);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

const char *rsvdt_batch_last_error(const rsvdt_batch *b) { return b ? b->err.c_str() : "null batch"; }

rsvdt_status rsvdt_batch_add(rsvdt_batch *b, const rsvdt_params *p, int64_t N, const int64_t *rowptr,
                             const int64_t *col, const double *val, int32_t *index) {
  if (!b || !p) return RSVDT_ERR_ARG;
  if (!b->stream) return bfail(b, RSVDT_ERR_STATE, "batch not created");
  rsvdt_params q = *p;
  q.precision = b->prec;
  rsvdt_ctx *c = nullptr;
  rsvdt_status st = rsvdt_create(&q, &c);
  if (st) {
    b->err = c ? rsvdt_last_error(c) : "context creation failed";
    rsvdt_destroy(c);
    return st;
  }
  // Issue everything of this problem on the batch's stream.
  cudaStreamDestroy(c->stream);
  c->stream = b->stream;
  c->owns_stream = false;
  st = rsvdt_set_operator(c, N, rowptr, col, val);
  if (st) {
    b->err = rsvdt_last_error(c);
    rsvdt_destroy(c);
    return st;
  }
  b->probs.push_back(c);
  if (index) *index = (int32_t)(b->probs.size() - 1);
  b->ready = false;
  return RSVDT_OK;
}

rsvdt_status rsvdt_batch_set_sketch(rsvdt_batch *b, int32_t index, const double *F, int64_t ld, int64_t ncols) {
  if (!b || index < 0 || (size_t)index >= b->probs.size()) return RSVDT_ERR_ARG;
  b->ready = false;
  return from_ctx(b, index, rsvdt_set_sketch(b->probs[index], F, ld, ncols));
}

rsvdt_status rsvdt_batch_random_sketch(rsvdt_batch *b, int32_t index, uint64_t seed) {
  if (!b || index < 0 || (size_t)index >= b->probs.size()) return RSVDT_ERR_ARG;
  b->ready = false;
  return from_ctx(b, index, rsvdt_random_sketch(b->probs[index], seed));
}

rsvdt_status rsvdt_batch_run(rsvdt_batch *b) {
  if (!b) return RSVDT_ERR_ARG;
  const size_t np = b->probs.size();
  if (np == 0) return bfail(b, RSVDT_ERR_STATE, "empty batch");
  if (!b->ready) {
    // Buffers are fixed once every problem has its sketch: argument arrays,
    // fresh graphs (the tuned launch shape is kept).
    free_batch_graphs(b);
    for (auto &p : b->d_args) {
      if (p) cudaFree(p);
      p = nullptr;
      if (!bcuda(b, cudaMalloc(&p, step_args_size(b->prec) * np), "arguments")) return RSVDT_ERR_OOM;
    }
    for (auto &p : b->d_args128) {
      if (p) cudaFree(p);
      p = nullptr;
      if (b->refine && !bcuda(b, cudaMalloc(&p, step_args_size(RSVDT_PREC_C128) * np), "arguments"))
        return RSVDT_ERR_OOM;
    }
    if (b->threads) {
      rsvdt_status st = build_work(b, b->threads, b->fs, b->kv);
      if (st) return st;
    }
    b->ready = true;
  }
  std::vector<char> all(np, 1);
  int64_t maxq = 0;
  for (auto *c : b->probs) maxq = std::max(maxq, c->par.q);
  rsvdt_status st;
  if ((st = batch_action(b, 1, all, b->prec))) return st;  // SourceCode/main.c:134
  for (int64_t iq = 0; iq < maxq; ++iq) {         // SourceCode/PowerIterationRK4.c:20-29
    std::vector<char> m(np);
    for (size_t p = 0; p < np; ++p) m[p] = b->probs[p]->par.q > iq;
    for (size_t p = 0; p < np; ++p)
      if (m[p] && (st = from_ctx(b, p, rsvdt_qr_all_freqs(b->probs[p])))) return st;
    if ((st = batch_action(b, 0, m, b->prec))) return st;
    for (size_t p = 0; p < np; ++p)
      if (m[p] && (st = from_ctx(b, p, rsvdt_qr_all_freqs(b->probs[p])))) return st;
    if ((st = batch_action(b, 1, m, b->prec))) return st;
  }
  for (size_t p = 0; p < np; ++p)
    if ((st = from_ctx(b, p, rsvdt_svd_all_freqs(b->probs[p], 1)))) return st;
  // SourceCode/main.c:142; the refinement form's FP64 sweep runs it in complex128.
  if ((st = batch_action(b, 0, all, b->refine ? RSVDT_PREC_C128 : b->prec))) return st;
  for (size_t p = 0; p < np; ++p)
    if ((st = from_ctx(b, p, rsvdt_svd_all_freqs(b->probs[p], 0)))) return st;
  return bcuda(b, cudaStreamSynchronize(b->stream), "sync") ? RSVDT_OK : RSVDT_ERR_CUDA;
}

rsvdt_status rsvdt_batch_get_results(rsvdt_batch *b, int32_t index, double *U, int64_t ldu, double *V, int64_t ldv,
                                     double *S) {
  if (!b || index < 0 || (size_t)index >= b->probs.size()) return RSVDT_ERR_ARG;
  return from_ctx(b, index, rsvdt_get_results(b->probs[index], U, ldu, V, ldv, S));
}

rsvdt_status rsvdt_batch_get_grid(const rsvdt_batch *b, int32_t index, rsvdt_grid *g) {
  if (!b || index < 0 || (size_t)index >= b->probs.size()) return RSVDT_ERR_ARG;
  return rsvdt_get_grid(b->probs[index], g);
}

rsvdt_status rsvdt_batch_get_tuning(const rsvdt_batch *b, int32_t *threads, int32_t *lanes_per_row,
                                    double *ms_per_step) {
  if (!b) return RSVDT_ERR_ARG;
  if (threads) *threads = b->threads;
  if (lanes_per_row) *lanes_per_row = b->fs;
  if (ms_per_step) *ms_per_step = b->tuned_ms;
  return RSVDT_OK;
}

int32_t rsvdt_batch_values_per_lane(const rsvdt_batch *b) { return b ? b->kv : 0; }

rsvdt_status rsvdt_batch_set_launch_shape(rsvdt_batch *b, int32_t threads, int32_t lanes_per_row,
                                          int32_t values_per_lane) {
  if (!b) return RSVDT_ERR_ARG;
  if (threads == 0) {  // back to the autotuner
    b->threads = 0;
    b->fs = 0;
    b->kv = 1;
    free_batch_graphs(b);
    return RSVDT_OK;
  }
  if ((threads != 128 && threads != 256) ||
      (lanes_per_row != 1 && lanes_per_row != 2 && lanes_per_row != 4 && lanes_per_row != 8) ||
      (values_per_lane != 1 && values_per_lane != 2))
    return bfail(b, RSVDT_ERR_ARG, "launch shape: threads 128 or 256, lanes per row 1, 2, 4 or 8, values per lane 1 or 2");
  if (values_per_lane == 2 && (b->prec != RSVDT_PREC_C64 || lanes_per_row != 1))
    return bfail(b, RSVDT_ERR_ARG, "two values per lane need complex64 stages and one lane per row");
  for (auto *c : b->probs)
    if (values_per_lane == 2 && c->K % 2)
      return bfail(b, RSVDT_ERR_ARG, "two values per lane need an even k in every problem");
  b->threads = threads;
  b->fs = lanes_per_row;
  b->kv = values_per_lane;
  free_batch_graphs(b);
  b->ready = false;  // rebuild the work lists
  return RSVDT_OK;
}

int64_t rsvdt_batch_launch_count(const rsvdt_batch *b) {
  if (!b) return 0;
  int64_t n = b->launches;
  for (auto *c : b->probs) n += c->launches;
  return n;
}

}  // extern "C"
