// Multilayer perceptron of the learned-sketch form: inference and training
// kernels written for this library.
//
// The network maps a problem's parameters to the coefficients of a
// warm-start test matrix in a POD basis: widths w0 -> w1 -> ... -> wL,
// GELU after every layer but the last. Weights are stored in bf16 (the
// operand of every matrix product), with FP32 master copies for the
// optimiser; activations, products and gradients are FP32 (FP32
// accumulation). Training minimises the mean squared error with Adam.
//
// Matrix products use one tiled kernel (32 x 32 output tile, K staged in
// shared memory 32 at a time) in the three shapes training needs:
//   forward    Z = X W^T + b     (X: B x in, W: out x in)
//   input grad dX = dZ W         (dZ: B x out)
//   weight grad dW = dZ^T X
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "rsvdt.h"

namespace {

constexpr int kT = 32;  // tile edge

__device__ __forceinline__ float ldv(const float *p) { return *p; }
__device__ __forceinline__ float ldv(const __nv_bfloat16 *p) { return __bfloat162float(*p); }

// C (M x N, row-major, ldc) = op(A) op(B) (+ bias[n]); op(A) is M x K,
// op(B) is K x N. TA: A stored K x M; TB: B stored N x K.
template <bool TA, bool TB, class TBv>
__global__ void __launch_bounds__(256) k_gemm(int M, int N, int K, const float *__restrict__ A, int lda,
                                              const TBv *__restrict__ B, int ldb, float *__restrict__ C, int ldc,
                                              const float *__restrict__ bias) {
  __shared__ float sa[kT][kT + 1];
  __shared__ float sb[kT][kT + 1];
  const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
  const int m0 = blockIdx.y * kT, n0 = blockIdx.x * kT;
  float acc[4] = {0, 0, 0, 0};
  for (int k0 = 0; k0 < K; k0 += kT) {
    for (int r = ty; r < kT; r += 8) {
      // sa[r][c] = op(A)[m0 + r][k0 + c], c = tx
      const int m = m0 + r, k = k0 + tx;
      float va = 0;
      if (m < M && k < K) va = TA ? A[(size_t)k * lda + m] : A[(size_t)m * lda + k];
      sa[r][tx] = va;
      // sb[r][c] = op(B)[k0 + r][n0 + c]
      const int kb = k0 + r, n = n0 + tx;
      float vb = 0;
      if (kb < K && n < N) vb = TB ? ldv(B + (size_t)n * ldb + kb) : ldv(B + (size_t)kb * ldb + n);
      sb[r][tx] = vb;
    }
    __syncthreads();
#pragma unroll 8
    for (int kk = 0; kk < kT; ++kk) {
      const float b = sb[kk][tx];
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[q] = fmaf(sa[ty + 8 * q][kk], b, acc[q]);
    }
    __syncthreads();
  }
  const int n = n0 + tx;
  if (n >= N) return;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int m = m0 + ty + 8 * q;
    if (m < M) C[(size_t)m * ldc + n] = acc[q] + (bias ? bias[n] : 0.f);
  }
}

__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float x) {
  const float cdf = 0.5f * (1.f + erff(x * 0.70710678118654752f));
  const float pdf = 0.39894228040143268f * expf(-0.5f * x * x);
  return cdf + x * pdf;
}

__global__ void k_gelu(const float *__restrict__ Z, float *__restrict__ Y, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) Y[i] = gelu(Z[i]);
}

// dZ = dA * gelu'(Z)
__global__ void k_gelu_back(const float *__restrict__ Z, const float *__restrict__ dA, float *__restrict__ dZ,
                            int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) dZ[i] = dA[i] * gelu_grad(Z[i]);
}

// dY = 2 (Y - T) / n and per-block partial sums of (Y - T)^2.
__global__ void k_mse(const float *__restrict__ Y, const float *__restrict__ T, float *__restrict__ dY, int64_t n,
                      float *__restrict__ part) {
  __shared__ float s[256];
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  float e = 0;
  if (i < n) {
    const float d = Y[i] - T[i];
    dY[i] = 2.f * d / (float)n;
    e = d * d;
  }
  s[threadIdx.x] = e;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = s[0];
}

// db[c] = sum over rows of dZ[:, c]
__global__ void k_colsum(const float *__restrict__ dZ, int rows, int cols, float *__restrict__ db) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cols) return;
  float s = 0;
  for (int r = 0; r < rows; ++r) s += dZ[(size_t)r * cols + c];
  db[c] = s;
}

__global__ void k_adam(float *__restrict__ w, const float *__restrict__ g, float *__restrict__ m, float *__restrict__ v,
                       int64_t n, float lr, float b1, float b2, float eps, float c1, float c2) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

__global__ void k_to_bf16(const float *__restrict__ s, __nv_bfloat16 *__restrict__ d, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) d[i] = __float2bfloat16(s[i]);
}

// out[r][c] = src[idx[r]][c]
__global__ void k_gather_rows(const float *__restrict__ src, const int32_t *__restrict__ idx, int rows, int cols,
                              float *__restrict__ out) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= (int64_t)rows * cols) return;
  const int r = (int)(i / cols), c = (int)(i - (int64_t)r * cols);
  out[i] = src[(size_t)idx[r] * cols + c];
}

inline int blocks(int64_t n, int t) { return (int)((n + t - 1) / t); }

}  // namespace

struct rsvdt_mlp {
  std::vector<int> w;  // widths, L+1 entries
  int L = 0;
  int64_t nparam = 0;
  std::vector<int64_t> woff, boff;  // offsets into the flat parameter vector
  float *p = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;  // FP32 master, grads, Adam moments
  __nv_bfloat16 *pb = nullptr;                                    // bf16 copy of the weights
  int64_t adam_t = 0;
  // Workspaces for a batch of up to cap rows.
  int cap = 0;
  std::vector<float *> Z, A;  // Z[l]: pre-activation of layer l (cap x w[l+1]); A[0] = input
  float *dA = nullptr, *dZ = nullptr, *loss_part = nullptr, *T = nullptr;
  int32_t *idx = nullptr;
  float *dataX = nullptr, *dataT = nullptr;
  int64_t data_n = 0;
  cudaStream_t stream = nullptr;
  std::string err;
};

static rsvdt_status mfail(rsvdt_mlp *n, rsvdt_status st, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (n) n->err = buf;
  return st;
}

static bool mok(rsvdt_mlp *n, cudaError_t e, const char *what) {
  if (e == cudaSuccess) return true;
  n->err = std::string("CUDA error in ") + what + ": " + cudaGetErrorString(e);
  return false;
}

static void free_work(rsvdt_mlp *n) {
  for (auto *q : n->Z) cudaFree(q);
  for (size_t i = 1; i < n->A.size(); ++i) cudaFree(n->A[i]);
  if (!n->A.empty()) cudaFree(n->A[0]);
  n->Z.clear();
  n->A.clear();
  cudaFree(n->dA);
  cudaFree(n->dZ);
  cudaFree(n->loss_part);
  cudaFree(n->T);
  cudaFree(n->idx);
  n->dA = n->dZ = n->loss_part = n->T = nullptr;
  n->idx = nullptr;
  n->cap = 0;
}

static rsvdt_status ensure_work(rsvdt_mlp *n, int rows) {
  if (rows <= n->cap) return RSVDT_OK;
  free_work(n);
  int wmax = 0;
  for (int x : n->w) wmax = std::max(wmax, x);
  n->A.assign(n->L + 1, nullptr);
  n->Z.assign(n->L, nullptr);
  bool ok = mok(n, cudaMalloc(&n->A[0], sizeof(float) * rows * n->w[0]), "alloc");
  for (int l = 0; l < n->L && ok; ++l) {
    ok = mok(n, cudaMalloc(&n->Z[l], sizeof(float) * rows * n->w[l + 1]), "alloc") &&
         mok(n, cudaMalloc(&n->A[l + 1], sizeof(float) * rows * n->w[l + 1]), "alloc");
  }
  ok = ok && mok(n, cudaMalloc(&n->dA, sizeof(float) * rows * wmax), "alloc") &&
       mok(n, cudaMalloc(&n->dZ, sizeof(float) * rows * wmax), "alloc") &&
       mok(n, cudaMalloc(&n->loss_part, sizeof(float) * (blocks((int64_t)rows * wmax, 256) + 1)), "alloc") &&
       mok(n, cudaMalloc(&n->T, sizeof(float) * rows * n->w[n->L]), "alloc") &&
       mok(n, cudaMalloc(&n->idx, sizeof(int32_t) * rows), "alloc");
  if (!ok) return RSVDT_ERR_OOM;
  n->cap = rows;
  return RSVDT_OK;
}

static void gemm(cudaStream_t s, bool ta, bool tb, int M, int N, int K, const float *A, int lda, const void *B,
                 bool b_bf16, int ldb, float *C, int ldc, const float *bias) {
  dim3 grid((N + kT - 1) / kT, (M + kT - 1) / kT), th(32, 8);
  if (b_bf16) {
    const __nv_bfloat16 *Bb = (const __nv_bfloat16 *)B;
    if (!ta && tb) k_gemm<false, true, __nv_bfloat16><<<grid, th, 0, s>>>(M, N, K, A, lda, Bb, ldb, C, ldc, bias);
    else k_gemm<false, false, __nv_bfloat16><<<grid, th, 0, s>>>(M, N, K, A, lda, Bb, ldb, C, ldc, bias);
  } else {
    const float *Bf = (const float *)B;
    k_gemm<true, false, float><<<grid, th, 0, s>>>(M, N, K, A, lda, Bf, ldb, C, ldc, bias);
  }
}

// Forward pass of `rows` rows already in A[0].
static void forward(rsvdt_mlp *n, int rows) {
  for (int l = 0; l < n->L; ++l) {
    const int in = n->w[l], out = n->w[l + 1];
    gemm(n->stream, false, true, rows, out, in, n->A[l], in, n->pb + n->woff[l], true, in, n->Z[l], out,
         n->p + n->boff[l]);
    const int64_t cnt = (int64_t)rows * out;
    if (l + 1 < n->L)
      k_gelu<<<blocks(cnt, 256), 256, 0, n->stream>>>(n->Z[l], n->A[l + 1], cnt);
    else
      cudaMemcpyAsync(n->A[l + 1], n->Z[l], sizeof(float) * cnt, cudaMemcpyDeviceToDevice, n->stream);
  }
}

// Loss and gradients into n->g for `rows` rows with targets in n->T.
static void backward(rsvdt_mlp *n, int rows) {
  const int L = n->L;
  const int64_t nout = (int64_t)rows * n->w[L];
  k_mse<<<blocks(nout, 256), 256, 0, n->stream>>>(n->A[L], n->T, n->dZ, nout, n->loss_part);
  for (int l = L - 1; l >= 0; --l) {
    const int in = n->w[l], out = n->w[l + 1];
    // dZ holds dL/dZ[l] (rows x out).
    gemm(n->stream, true, false, out, in, rows, n->dZ, out, n->A[l], false, in, n->g + n->woff[l], in, nullptr);
    k_colsum<<<blocks(out, 128), 128, 0, n->stream>>>(n->dZ, rows, out, n->g + n->boff[l]);
    if (l == 0) break;
    gemm(n->stream, false, false, rows, in, out, n->dZ, out, n->pb + n->woff[l], true, in, n->dA, in, nullptr);
    const int64_t cnt = (int64_t)rows * in;
    k_gelu_back<<<blocks(cnt, 256), 256, 0, n->stream>>>(n->Z[l - 1], n->dA, n->dZ, cnt);
  }
}

static float read_loss(rsvdt_mlp *n, int rows) {
  const int nb = blocks((int64_t)rows * n->w[n->L], 256);
  std::vector<float> part(nb);
  cudaMemcpyAsync(part.data(), n->loss_part, sizeof(float) * nb, cudaMemcpyDeviceToHost, n->stream);
  cudaStreamSynchronize(n->stream);
  double s = 0;
  for (float x : part) s += x;
  return (float)(s / ((double)rows * n->w[n->L]));
}

static void sync_bf16(rsvdt_mlp *n) {
  for (int l = 0; l < n->L; ++l) {
    const int64_t cnt = (int64_t)n->w[l] * n->w[l + 1];
    k_to_bf16<<<blocks(cnt, 256), 256, 0, n->stream>>>(n->p + n->woff[l], n->pb + n->woff[l], cnt);
  }
}

extern "C" {

rsvdt_status rsvdt_mlp_create(int32_t n_layers, const int32_t *widths, uint64_t seed, rsvdt_mlp **out) {
  if (!out) return RSVDT_ERR_ARG;
  rsvdt_mlp *n = new rsvdt_mlp();
  *out = n;
  if (n_layers < 1 || !widths) return mfail(n, RSVDT_ERR_ARG, "need at least one layer");
  for (int i = 0; i <= n_layers; ++i)
    if (widths[i] < 1 || widths[i] > 65536) return mfail(n, RSVDT_ERR_ARG, "invalid width %d", widths[i]);
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return mfail(n, RSVDT_ERR_CUDA, "no CUDA device available");
  }
  n->L = n_layers;
  n->w.assign(widths, widths + n_layers + 1);
  int64_t off = 0;
  for (int l = 0; l < n->L; ++l) {
    n->woff.push_back(off);
    off += (int64_t)n->w[l] * n->w[l + 1];
    n->boff.push_back(off);
    off += n->w[l + 1];
  }
  n->nparam = off;
  if (!mok(n, cudaStreamCreateWithFlags(&n->stream, cudaStreamNonBlocking), "stream") ||
      !mok(n, cudaMalloc(&n->p, sizeof(float) * off), "alloc") ||
      !mok(n, cudaMalloc(&n->g, sizeof(float) * off), "alloc") ||
      !mok(n, cudaMalloc(&n->m, sizeof(float) * off), "alloc") ||
      !mok(n, cudaMalloc(&n->v, sizeof(float) * off), "alloc") ||
      !mok(n, cudaMalloc(&n->pb, sizeof(__nv_bfloat16) * off), "alloc"))
    return RSVDT_ERR_OOM;
  // He-style initialisation (normal, std sqrt(2/in)), zero biases.
  std::vector<float> h(off, 0.f);
  std::mt19937_64 rng(seed);
  for (int l = 0; l < n->L; ++l) {
    std::normal_distribution<float> nd(0.f, std::sqrt(2.f / (float)n->w[l]));
    for (int64_t i = 0; i < (int64_t)n->w[l] * n->w[l + 1]; ++i) h[n->woff[l] + i] = nd(rng);
  }
  return rsvdt_mlp_set_params(n, h.data());
}

void rsvdt_mlp_destroy(rsvdt_mlp *n) {
  if (!n) return;
  if (n->stream) cudaStreamSynchronize(n->stream);
  free_work(n);
  cudaFree(n->p);
  cudaFree(n->g);
  cudaFree(n->m);
  cudaFree(n->v);
  cudaFree(n->pb);
  cudaFree(n->dataX);
  cudaFree(n->dataT);
  if (n->stream) cudaStreamDestroy(n->stream);
  delete n;
}

const char *rsvdt_mlp_last_error(const rsvdt_mlp *n) { return n ? n->err.c_str() : "null network"; }

int64_t rsvdt_mlp_param_count(const rsvdt_mlp *n) { return n ? n->nparam : 0; }

rsvdt_status rsvdt_mlp_set_params(rsvdt_mlp *n, const float *params) {
  if (!n || !params) return RSVDT_ERR_ARG;
  if (!mok(n, cudaMemcpyAsync(n->p, params, sizeof(float) * n->nparam, cudaMemcpyHostToDevice, n->stream), "copy") ||
      !mok(n, cudaMemsetAsync(n->m, 0, sizeof(float) * n->nparam, n->stream), "memset") ||
      !mok(n, cudaMemsetAsync(n->v, 0, sizeof(float) * n->nparam, n->stream), "memset"))
    return RSVDT_ERR_CUDA;
  n->adam_t = 0;
  sync_bf16(n);
  return mok(n, cudaStreamSynchronize(n->stream), "sync") ? RSVDT_OK : RSVDT_ERR_CUDA;
}

rsvdt_status rsvdt_mlp_get_params(rsvdt_mlp *n, float *params) {
  if (!n || !params) return RSVDT_ERR_ARG;
  if (!mok(n, cudaMemcpyAsync(params, n->p, sizeof(float) * n->nparam, cudaMemcpyDeviceToHost, n->stream), "copy") ||
      !mok(n, cudaStreamSynchronize(n->stream), "sync"))
    return RSVDT_ERR_CUDA;
  return RSVDT_OK;
}

rsvdt_status rsvdt_mlp_forward(rsvdt_mlp *n, const float *X, int64_t rows, float *Y) {
  if (!n || !X || !Y || rows < 1 || rows > (1 << 24)) return RSVDT_ERR_ARG;
  rsvdt_status st = ensure_work(n, (int)rows);
  if (st) return st;
  if (!mok(n, cudaMemcpyAsync(n->A[0], X, sizeof(float) * rows * n->w[0], cudaMemcpyHostToDevice, n->stream), "copy"))
    return RSVDT_ERR_CUDA;
  forward(n, (int)rows);
  if (!mok(n, cudaMemcpyAsync(Y, n->A[n->L], sizeof(float) * rows * n->w[n->L], cudaMemcpyDeviceToHost, n->stream),
           "copy") ||
      !mok(n, cudaStreamSynchronize(n->stream), "sync") || !mok(n, cudaGetLastError(), "forward"))
    return RSVDT_ERR_CUDA;
  return RSVDT_OK;
}

rsvdt_status rsvdt_mlp_gradients(rsvdt_mlp *n, const float *X, const float *T, int64_t rows, float *loss,
                                 float *grads) {
  if (!n || !X || !T || rows < 1 || rows > (1 << 24)) return RSVDT_ERR_ARG;
  rsvdt_status st = ensure_work(n, (int)rows);
  if (st) return st;
  if (!mok(n, cudaMemcpyAsync(n->A[0], X, sizeof(float) * rows * n->w[0], cudaMemcpyHostToDevice, n->stream), "copy") ||
      !mok(n, cudaMemcpyAsync(n->T, T, sizeof(float) * rows * n->w[n->L], cudaMemcpyHostToDevice, n->stream), "copy"))
    return RSVDT_ERR_CUDA;
  forward(n, (int)rows);
  backward(n, (int)rows);
  const float l = read_loss(n, (int)rows);
  if (loss) *loss = l;
  if (grads &&
      !mok(n, cudaMemcpyAsync(grads, n->g, sizeof(float) * n->nparam, cudaMemcpyDeviceToHost, n->stream), "copy"))
    return RSVDT_ERR_CUDA;
  return mok(n, cudaStreamSynchronize(n->stream), "sync") && mok(n, cudaGetLastError(), "gradients") ? RSVDT_OK
                                                                                                      : RSVDT_ERR_CUDA;
}

rsvdt_status rsvdt_mlp_train(rsvdt_mlp *n, const float *X, const float *T, int64_t samples, int64_t batch,
                             int64_t steps, float lr, uint64_t seed, float *final_loss) {
  if (!n || !X || !T || samples < 1 || batch < 1 || steps < 0 || samples > (1 << 24)) return RSVDT_ERR_ARG;
  if (batch > samples) batch = samples;
  rsvdt_status st = ensure_work(n, (int)batch);
  if (st) return st;
  cudaFree(n->dataX);
  cudaFree(n->dataT);
  n->dataX = n->dataT = nullptr;
  const int in = n->w[0], outw = n->w[n->L];
  if (!mok(n, cudaMalloc(&n->dataX, sizeof(float) * samples * in), "alloc") ||
      !mok(n, cudaMalloc(&n->dataT, sizeof(float) * samples * outw), "alloc"))
    return RSVDT_ERR_OOM;
  if (!mok(n, cudaMemcpyAsync(n->dataX, X, sizeof(float) * samples * in, cudaMemcpyHostToDevice, n->stream), "copy") ||
      !mok(n, cudaMemcpyAsync(n->dataT, T, sizeof(float) * samples * outw, cudaMemcpyHostToDevice, n->stream), "copy"))
    return RSVDT_ERR_CUDA;
  n->data_n = samples;
  // Minibatches: a fresh permutation of the samples each epoch.
  std::mt19937_64 rng(seed);
  std::vector<int32_t> perm(samples);
  for (int64_t i = 0; i < samples; ++i) perm[i] = (int32_t)i;
  std::vector<int32_t> idx_host((size_t)batch * steps);
  int64_t pos = samples;
  for (int64_t s = 0; s < steps; ++s)
    for (int64_t b = 0; b < batch; ++b) {
      if (pos == samples) {
        std::shuffle(perm.begin(), perm.end(), rng);
        pos = 0;
      }
      idx_host[s * batch + b] = perm[pos++];
    }
  int32_t *d_idx_all = nullptr;
  if (steps > 0 && !mok(n, cudaMalloc(&d_idx_all, sizeof(int32_t) * idx_host.size()), "alloc")) return RSVDT_ERR_OOM;
  if (steps > 0 && !mok(n, cudaMemcpyAsync(d_idx_all, idx_host.data(), sizeof(int32_t) * idx_host.size(),
                                           cudaMemcpyHostToDevice, n->stream), "copy")) {
    cudaFree(d_idx_all);
    return RSVDT_ERR_CUDA;
  }
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const int rows = (int)batch;
  for (int64_t s = 0; s < steps; ++s) {
    const int32_t *ix = d_idx_all + s * batch;
    k_gather_rows<<<blocks((int64_t)rows * in, 256), 256, 0, n->stream>>>(n->dataX, ix, rows, in, n->A[0]);
    k_gather_rows<<<blocks((int64_t)rows * outw, 256), 256, 0, n->stream>>>(n->dataT, ix, rows, outw, n->T);
    forward(n, rows);
    backward(n, rows);
    ++n->adam_t;
    const float c1 = 1.f - std::pow(b1, (float)n->adam_t), c2 = 1.f - std::pow(b2, (float)n->adam_t);
    k_adam<<<blocks(n->nparam, 256), 256, 0, n->stream>>>(n->p, n->g, n->m, n->v, n->nparam, lr, b1, b2, eps, c1, c2);
    sync_bf16(n);
  }
  float l = 0;
  if (steps > 0) l = read_loss(n, rows);
  cudaStreamSynchronize(n->stream);
  cudaFree(d_idx_all);
  if (final_loss) *final_loss = l;
  return mok(n, cudaGetLastError(), "train") ? RSVDT_OK : RSVDT_ERR_CUDA;
}

}  // extern "C"
