// The learned schedule cost model: a 3-layer FP32 MLP (n_in -> width -> width ->
// n_out, ReLU), trained and evaluated with these kernels only.  The network is
// tiny (width 64: ~7k parameters), so the kernels are latency-bound and kept
// simple: one thread per output element per layer, every reduction in a fixed
// order (runs are bit-reproducible), Adam updates (Kingma-Ba 2015).
#include <cmath>
#include <cstring>
#include <vector>

#include "tq_internal.h"

struct tq_mlp {
  int32_t n_in = 0, width = 0, n_out = 0;
  int64_t n_params = 0;
  // params | grads | adam m | adam v, each n_params floats
  tq::DevArray<float> buf;
  int64_t step = 0;
  // activations of the last forward pass (for backward), and scratch
  tq::DevArray<float> h1, h2, y, d2, d1, dy, loss;
  int64_t cap = 0;  // samples the activation buffers hold
  // offsets of W1 b1 W2 b2 W3 b3 inside params
  int64_t oW1, ob1, oW2, ob2, oW3, ob3;
  float *params() { return buf.p; }
  float *grads() { return buf.p + n_params; }
  float *m() { return buf.p + 2 * n_params; }
  float *v() { return buf.p + 3 * n_params; }
};

namespace tq {

// out[s][j] = act(b[j] + sum_i W[j][i] in[s][i]), W row-major [n_o][n_i]
__global__ void mlp_layer_fwd(const float *W, const float *b, const float *in, int n_i, int n_o,
                              int64_t n, int relu, float *out) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n * n_o) return;
  const int64_t s = g / n_o;
  const int j = (int)(g % n_o);
  float acc = b[j];
  const float *w = W + (int64_t)j * n_i, *x = in + s * n_i;
  for (int i = 0; i < n_i; i++) acc = fmaf(w[i], x[i], acc);
  out[g] = relu ? fmaxf(acc, 0.f) : acc;
}

// loss = mean over samples and outputs of mask * (y - t)^2; dy = d loss / d y
__global__ void mlp_mse(const float *y, const float *t, const float *mask, int64_t n, int n_o,
                        float *dy, float *loss_terms) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n * n_o) return;
  const float d = y[g] - t[g];
  const float w = mask ? mask[g] : 1.f;
  const float scale = 1.0f / (float)(n * n_o);
  dy[g] = 2.f * w * d * scale;
  loss_terms[g] = w * d * d * scale;
}

// fixed-order sum of n values by one block
__global__ void mlp_sum(const float *x, int64_t n, float *out) {
  __shared__ float red[256];
  float acc = 0.f;
  for (int64_t i = threadIdx.x; i < n; i += 256) acc += x[i];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0];
}

// dW[j][i] = sum_s dout[s][j] in[s][i]; db[j] = sum_s dout[s][j] (one thread each)
__global__ void mlp_wgrad(const float *dout, const float *in, int n_i, int n_o, int64_t n,
                          float *dW, float *db) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n_o * (n_i + 1)) return;
  const int j = g / (n_i + 1), i = g % (n_i + 1);
  float acc = 0.f;
  if (i < n_i) {
    for (int64_t s = 0; s < n; s++) acc = fmaf(dout[s * n_o + j], in[s * n_i + i], acc);
    dW[(int64_t)j * n_i + i] = acc;
  } else {
    for (int64_t s = 0; s < n; s++) acc += dout[s * n_o + j];
    db[j] = acc;
  }
}

// din[s][i] = (sum_j W[j][i] dout[s][j]) * relu'(act[s][i])
__global__ void mlp_dgrad(const float *W, const float *dout, const float *act, int n_i, int n_o,
                          int64_t n, float *din) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n * n_i) return;
  const int64_t s = g / n_i;
  const int i = (int)(g % n_i);
  float acc = 0.f;
  for (int j = 0; j < n_o; j++) acc = fmaf(W[(int64_t)j * n_i + i], dout[s * n_o + j], acc);
  din[g] = act[g] > 0.f ? acc : 0.f;
}

__global__ void mlp_adam(float *p, const float *g, float *m, float *v, int64_t n, float lr,
                         float b1, float b2, float eps, float c1, float c2) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  m[i] = b1 * m[i] + (1.f - b1) * gi;
  v[i] = b2 * v[i] + (1.f - b2) * gi * gi;
  p[i] -= lr * (m[i] / c1) / (sqrtf(v[i] / c2) + eps);
}

static inline unsigned grid_of(int64_t n) { return (unsigned)((n + 255) / 256); }

static tq_status ensure_cap(tq_mlp *M, int64_t n, cudaStream_t s) {
  if (n <= M->cap) return TQ_OK;
  TQ_CHECK(M->h1.alloc(n * M->width, s));
  TQ_CHECK(M->h2.alloc(n * M->width, s));
  TQ_CHECK(M->y.alloc(n * M->n_out, s));
  TQ_CHECK(M->d2.alloc(n * M->width, s));
  TQ_CHECK(M->d1.alloc(n * M->width, s));
  TQ_CHECK(M->dy.alloc(n * M->n_out, s));
  TQ_CHECK(M->loss.alloc(n * M->n_out + 1, s));
  M->cap = n;
  return TQ_OK;
}

static tq_status forward(tq_mlp *M, const float *X, int64_t n, cudaStream_t s) {
  TQ_CHECK(ensure_cap(M, n, s));
  const float *P = M->params();
  const int W = M->width;
  count_launch(), mlp_layer_fwd<<<grid_of(n * W), 256, 0, s>>>(P + M->oW1, P + M->ob1, X, M->n_in, W, n, 1, M->h1.p);
  count_launch(), mlp_layer_fwd<<<grid_of(n * W), 256, 0, s>>>(P + M->oW2, P + M->ob2, M->h1.p, W, W, n, 1, M->h2.p);
  count_launch(), mlp_layer_fwd<<<grid_of(n * M->n_out), 256, 0, s>>>(P + M->oW3, P + M->ob3, M->h2.p, W, M->n_out, n, 0, M->y.p);
  TQ_CUDA(cudaGetLastError());
  return TQ_OK;
}

// loss and gradients of the mean squared error against T (n x n_out)
static tq_status backward(tq_mlp *M, const float *X, const float *T, const float *mask, int64_t n,
                          cudaStream_t s) {
  TQ_CHECK(forward(M, X, n, s));
  const float *P = M->params();
  float *G = M->grads();
  const int W = M->width, O = M->n_out;
  count_launch(), mlp_mse<<<grid_of(n * O), 256, 0, s>>>(M->y.p, T, mask, n, O, M->dy.p, M->loss.p);
  count_launch(), mlp_sum<<<1, 256, 0, s>>>(M->loss.p, n * O, M->loss.p + n * O);
  count_launch(), mlp_wgrad<<<grid_of(O * (W + 1)), 256, 0, s>>>(M->dy.p, M->h2.p, W, O, n, G + M->oW3, G + M->ob3);
  count_launch(), mlp_dgrad<<<grid_of(n * W), 256, 0, s>>>(P + M->oW3, M->dy.p, M->h2.p, W, O, n, M->d2.p);
  count_launch(), mlp_wgrad<<<grid_of(W * (W + 1)), 256, 0, s>>>(M->d2.p, M->h1.p, W, W, n, G + M->oW2, G + M->ob2);
  count_launch(), mlp_dgrad<<<grid_of(n * W), 256, 0, s>>>(P + M->oW2, M->d2.p, M->h1.p, W, W, n, M->d1.p);
  count_launch(), mlp_wgrad<<<grid_of(W * (M->n_in + 1)), 256, 0, s>>>(M->d1.p, X, M->n_in, W, n, G + M->oW1, G + M->ob1);
  TQ_CUDA(cudaGetLastError());
  return TQ_OK;
}

}  // namespace tq

using namespace tq;

extern "C" {

tq_status tq_mlp_create(int32_t n_in, int32_t width, int32_t n_out, uint64_t seed, tq_mlp **out) {
  if (!out || n_in <= 0 || width <= 0 || n_out <= 0) return fail(TQ_ERR_INVALID, "bad MLP shape");
  std::unique_ptr<tq_mlp> M(new tq_mlp());
  M->n_in = n_in;
  M->width = width;
  M->n_out = n_out;
  M->oW1 = 0;
  M->ob1 = M->oW1 + (int64_t)width * n_in;
  M->oW2 = M->ob1 + width;
  M->ob2 = M->oW2 + (int64_t)width * width;
  M->oW3 = M->ob2 + width;
  M->ob3 = M->oW3 + (int64_t)n_out * width;
  M->n_params = M->ob3 + n_out;
  TQ_CHECK(M->buf.alloc(4 * M->n_params, nullptr));
  // He-uniform weights from a fixed 64-bit LCG (host), zero biases and moments
  std::vector<float> h(4 * M->n_params, 0.f);
  uint64_t x = seed * 6364136223846793005ull + 1442695040888963407ull;
  auto uni = [&]() {
    x = x * 6364136223846793005ull + 1442695040888963407ull;
    return ((x >> 40) & 0xffffff) / 16777216.0 * 2.0 - 1.0;
  };
  auto fill = [&](int64_t o, int64_t cnt, int fan_in) {
    const double a = std::sqrt(6.0 / fan_in);
    for (int64_t i = 0; i < cnt; i++) h[o + i] = (float)(a * uni());
  };
  fill(M->oW1, (int64_t)width * n_in, n_in);
  fill(M->oW2, (int64_t)width * width, width);
  fill(M->oW3, (int64_t)n_out * width, width);
  TQ_CUDA(cudaMemcpy(M->buf.p, h.data(), h.size() * 4, cudaMemcpyHostToDevice));
  *out = M.release();
  return TQ_OK;
}

tq_status tq_mlp_destroy(tq_mlp *M) {
  delete M;
  return TQ_OK;
}

tq_status tq_mlp_num_params(const tq_mlp *M, int64_t *n) {
  if (!M || !n) return fail(TQ_ERR_INVALID, "NULL argument");
  *n = M->n_params;
  return TQ_OK;
}

tq_status tq_mlp_get_params(tq_mlp *M, float *host) {
  if (!M || !host) return fail(TQ_ERR_INVALID, "NULL argument");
  TQ_CUDA(cudaMemcpy(host, M->params(), M->n_params * 4, cudaMemcpyDeviceToHost));
  return TQ_OK;
}

tq_status tq_mlp_set_params(tq_mlp *M, const float *host) {
  if (!M || !host) return fail(TQ_ERR_INVALID, "NULL argument");
  TQ_CUDA(cudaMemcpy(M->params(), host, M->n_params * 4, cudaMemcpyHostToDevice));
  return TQ_OK;
}

tq_status tq_mlp_forward(tq_mlp *M, const float *X, int64_t n, float *Y, tq_stream stream) {
  if (!M || (n > 0 && (!X || !Y))) return fail(TQ_ERR_INVALID, "NULL argument");
  if (n == 0) return TQ_OK;
  cudaStream_t s = (cudaStream_t)stream;
  TQ_CHECK(forward(M, X, n, s));
  TQ_CUDA(cudaMemcpyAsync(Y, M->y.p, n * M->n_out * 4, cudaMemcpyDeviceToDevice, s));
  return TQ_OK;
}

tq_status tq_mlp_gradients(tq_mlp *M, const float *X, const float *T, const float *mask, int64_t n,
                           float *grads_host, float *loss_host, tq_stream stream) {
  if (!M || !X || !T || n <= 0) return fail(TQ_ERR_INVALID, "bad argument");
  cudaStream_t s = (cudaStream_t)stream;
  TQ_CHECK(backward(M, X, T, mask, n, s));
  if (grads_host)
    TQ_CUDA(cudaMemcpyAsync(grads_host, M->grads(), M->n_params * 4, cudaMemcpyDeviceToHost, s));
  if (loss_host)
    TQ_CUDA(cudaMemcpyAsync(loss_host, M->loss.p + n * M->n_out, 4, cudaMemcpyDeviceToHost, s));
  TQ_CUDA(cudaStreamSynchronize(s));
  return TQ_OK;
}

tq_status tq_mlp_train_step(tq_mlp *M, const float *X, const float *T, const float *mask, int64_t n,
                            float lr, float *loss_dev, tq_stream stream) {
  if (!M || !X || !T || n <= 0) return fail(TQ_ERR_INVALID, "bad argument");
  cudaStream_t s = (cudaStream_t)stream;
  TQ_CHECK(backward(M, X, T, mask, n, s));
  M->step++;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - std::pow(b1, (float)M->step), c2 = 1.f - std::pow(b2, (float)M->step);
  count_launch(), mlp_adam<<<grid_of(M->n_params), 256, 0, s>>>(M->params(), M->grads(), M->m(), M->v(),
                                                   M->n_params, lr, b1, b2, 1e-8f, c1, c2);
  TQ_CUDA(cudaGetLastError());
  if (loss_dev)
    TQ_CUDA(cudaMemcpyAsync(loss_dev, M->loss.p + n * M->n_out, 4, cudaMemcpyDeviceToDevice, s));
  return TQ_OK;
}

}  // extern "C"
