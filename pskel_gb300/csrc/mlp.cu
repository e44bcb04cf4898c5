// A small multilayer perceptron cost model, trained and evaluated by this
// library's own CUDA kernels: dense layers with tanh activations and one
// linear output, full-batch mean-squared error, Adam.
//
// Layout: X is n x in (row-major), y is n. Parameters are one flat fp32 array:
// for each layer l (din -> dout): W_l (dout x din, row-major) then b_l (dout).
// Every reduction over samples or units is a loop owned by one thread in a
// fixed order, so training is deterministic for a given seed.
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/pskel_gb300.h"
#include "capi_internal.h"

namespace pskel {
namespace {

constexpr int kMaxLayers = 8;

// out[s][j] = act(sum_k W[j][k] * in[s][k] + b[j])
__global__ void dense_forward(const float* __restrict__ in, const float* __restrict__ W, const float* __restrict__ b,
                              float* __restrict__ out, int n, int din, int dout, int act_tanh) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n * dout) return;
  const int s = idx / dout, j = idx - s * dout;
  const float* x = in + static_cast<size_t>(s) * din;
  const float* w = W + static_cast<size_t>(j) * din;
  float acc = b[j];
  for (int k = 0; k < din; ++k) acc = fmaf(w[k], x[k], acc);
  out[idx] = act_tanh ? tanhf(acc) : acc;
}

// delta = dL/dyhat for L = mean((yhat - y)^2); loss_parts[s] = (yhat - y)^2
__global__ void mse_grad(const float* __restrict__ yhat, const float* __restrict__ y, float* __restrict__ delta,
                         float* __restrict__ sq, int n) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const float e = yhat[s] - y[s];
  delta[s] = 2.0f * e / static_cast<float>(n);
  sq[s] = e * e;
}

// delta_pre = delta_post * (1 - a^2) for tanh units, in place
__global__ void tanh_backward(float* __restrict__ delta, const float* __restrict__ act, int count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  delta[i] *= 1.0f - act[i] * act[i];
}

// gW[j][k] = sum_s delta[s][j] * in[s][k]; gb[j] = sum_s delta[s][j]
__global__ void dense_weight_grad(const float* __restrict__ in, const float* __restrict__ delta,
                                  float* __restrict__ gW, float* __restrict__ gb, int n, int din, int dout) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= dout * (din + 1)) return;
  const int j = idx / (din + 1), k = idx - j * (din + 1);
  float acc = 0.0f;
  if (k < din) {
    for (int s = 0; s < n; ++s) acc = fmaf(delta[static_cast<size_t>(s) * dout + j], in[static_cast<size_t>(s) * din + k], acc);
    gW[static_cast<size_t>(j) * din + k] = acc;
  } else {
    for (int s = 0; s < n; ++s) acc += delta[static_cast<size_t>(s) * dout + j];
    gb[j] = acc;
  }
}

// din_delta[s][k] = sum_j W[j][k] * delta[s][j]
__global__ void dense_input_grad(const float* __restrict__ W, const float* __restrict__ delta,
                                 float* __restrict__ din_delta, int n, int din, int dout) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n * din) return;
  const int s = idx / din, k = idx - s * din;
  float acc = 0.0f;
  for (int j = 0; j < dout; ++j) acc = fmaf(W[static_cast<size_t>(j) * din + k], delta[static_cast<size_t>(s) * dout + j], acc);
  din_delta[idx] = acc;
}

// sum of n values, one thread, fixed order
__global__ void sum_serial(const float* __restrict__ v, int n, float* __restrict__ out) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  double acc = 0.0;
  for (int i = 0; i < n; ++i) acc += v[i];
  *out = static_cast<float>(acc);
}

__global__ void adam_step(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                          float* __restrict__ v, int count, float lr, float b1, float b2, float eps, float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.0f - b1) * gi;
  const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

inline int blocks(int count) { return (count + 255) / 256; }

}  // namespace
}  // namespace pskel

using namespace pskel;

struct pskel_mlp {
  int in_dim = 0, hidden = 0, layers = 0;  // layers = number of dense layers (>= 2)
  std::vector<int> dims;                   // dims[0] = in, ..., dims[layers] = 1
  std::vector<size_t> w_off, b_off;        // offsets into the flat parameter array
  size_t nparams = 0;
  float* d_params = nullptr;
  float* d_grads = nullptr;
  float* d_m = nullptr;
  float* d_v = nullptr;
  int64_t step = 0;
  // per-batch scratch
  int cap = 0;
  float* d_x = nullptr;
  float* d_y = nullptr;
  std::vector<float*> d_act;    // activations per layer output
  std::vector<float*> d_delta;  // deltas per layer output
  float* d_sq = nullptr;
  float* d_loss = nullptr;
  cudaStream_t stream = nullptr;
};

static pskel_status mlp_reserve(pskel_mlp* m, int n) {
  if (n <= m->cap) return PSKEL_OK;
  cudaFree(m->d_x);
  cudaFree(m->d_y);
  for (float* p : m->d_act) cudaFree(p);
  for (float* p : m->d_delta) cudaFree(p);
  cudaFree(m->d_sq);
  m->d_act.assign(m->layers, nullptr);
  m->d_delta.assign(m->layers + 1, nullptr);
  cudaError_t e = cudaMalloc(&m->d_x, sizeof(float) * n * m->in_dim);
  if (e == cudaSuccess) e = cudaMalloc(&m->d_y, sizeof(float) * n);
  for (int l = 0; l < m->layers && e == cudaSuccess; ++l) e = cudaMalloc(&m->d_act[l], sizeof(float) * n * m->dims[l + 1]);
  for (int l = 0; l <= m->layers && e == cudaSuccess; ++l)
    e = cudaMalloc(&m->d_delta[l], sizeof(float) * n * m->dims[l]);
  if (e == cudaSuccess) e = cudaMalloc(&m->d_sq, sizeof(float) * n);
  if (e != cudaSuccess) return cuda_fail(e, "MLP scratch");
  m->cap = n;
  return PSKEL_OK;
}

static void mlp_forward(pskel_mlp* m, int n) {
  const float* in = m->d_x;
  for (int l = 0; l < m->layers; ++l) {
    const int din = m->dims[l], dout = m->dims[l + 1];
    const bool last = (l == m->layers - 1);
    dense_forward<<<blocks(n * dout), 256, 0, m->stream>>>(in, m->d_params + m->w_off[l], m->d_params + m->b_off[l],
                                                           m->d_act[l], n, din, dout, last ? 0 : 1);
    in = m->d_act[l];
  }
}

// gradients of the mean-squared error into d_grads, loss into d_loss
static void mlp_backward(pskel_mlp* m, int n) {
  const int L = m->layers;
  mse_grad<<<blocks(n), 256, 0, m->stream>>>(m->d_act[L - 1], m->d_y, m->d_delta[L], m->d_sq, n);
  sum_serial<<<1, 1, 0, m->stream>>>(m->d_sq, n, m->d_loss);
  for (int l = L - 1; l >= 0; --l) {
    const int din = m->dims[l], dout = m->dims[l + 1];
    float* delta = m->d_delta[l + 1];
    if (l < L - 1) tanh_backward<<<blocks(n * dout), 256, 0, m->stream>>>(delta, m->d_act[l], n * dout);
    const float* in = (l == 0) ? m->d_x : m->d_act[l - 1];
    dense_weight_grad<<<blocks(dout * (din + 1)), 256, 0, m->stream>>>(in, delta, m->d_grads + m->w_off[l],
                                                                      m->d_grads + m->b_off[l], n, din, dout);
    if (l > 0)
      dense_input_grad<<<blocks(n * din), 256, 0, m->stream>>>(m->d_params + m->w_off[l], delta, m->d_delta[l], n, din,
                                                               dout);
  }
}

extern "C" {

pskel_status pskel_mlp_create(int32_t in_dim, int32_t hidden, int32_t layers, uint64_t seed, pskel_mlp** out) {
  clear_error();
  if (!out || in_dim <= 0 || hidden <= 0 || layers < 2 || layers > kMaxLayers)
    return fail(PSKEL_ERR_INVALID, "MLP: bad shape (in %d, hidden %d, layers %d)", in_dim, hidden, layers);
  pskel_mlp* m = new pskel_mlp();
  m->in_dim = in_dim;
  m->hidden = hidden;
  m->layers = layers;
  m->dims.push_back(in_dim);
  for (int l = 0; l < layers - 1; ++l) m->dims.push_back(hidden);
  m->dims.push_back(1);
  for (int l = 0; l < layers; ++l) {
    m->w_off.push_back(m->nparams);
    m->nparams += static_cast<size_t>(m->dims[l]) * m->dims[l + 1];
    m->b_off.push_back(m->nparams);
    m->nparams += m->dims[l + 1];
  }
  // Glorot-uniform weights from a SplitMix64 stream, zero biases
  std::vector<float> init(m->nparams, 0.0f);
  uint64_t z = seed * 0x9E3779B97F4A7C15ull + 1;
  auto next = [&]() {
    z += 0x9E3779B97F4A7C15ull;
    uint64_t x = z;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    x ^= x >> 31;
    return static_cast<double>(x >> 11) * (1.0 / 9007199254740992.0);
  };
  for (int l = 0; l < layers; ++l) {
    const double lim = std::sqrt(6.0 / (m->dims[l] + m->dims[l + 1]));
    for (size_t i = 0; i < static_cast<size_t>(m->dims[l]) * m->dims[l + 1]; ++i)
      init[m->w_off[l] + i] = static_cast<float>((2.0 * next() - 1.0) * lim);
  }
  cudaError_t e = cudaMalloc(&m->d_params, sizeof(float) * m->nparams);
  if (e == cudaSuccess) e = cudaMalloc(&m->d_grads, sizeof(float) * m->nparams);
  if (e == cudaSuccess) e = cudaMalloc(&m->d_m, sizeof(float) * m->nparams);
  if (e == cudaSuccess) e = cudaMalloc(&m->d_v, sizeof(float) * m->nparams);
  if (e == cudaSuccess) e = cudaMalloc(&m->d_loss, sizeof(float));
  if (e == cudaSuccess) e = cudaMemcpy(m->d_params, init.data(), sizeof(float) * m->nparams, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(m->d_m, 0, sizeof(float) * m->nparams);
  if (e == cudaSuccess) e = cudaMemset(m->d_v, 0, sizeof(float) * m->nparams);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete m;
    return cuda_fail(e, "MLP create");
  }
  *out = m;
  return PSKEL_OK;
}

int64_t pskel_mlp_num_params(const pskel_mlp* m) { return m ? static_cast<int64_t>(m->nparams) : 0; }

void pskel_mlp_shape(const pskel_mlp* m, int32_t* in_dim, int32_t* hidden, int32_t* layers) {
  if (in_dim) *in_dim = m ? m->in_dim : 0;
  if (hidden) *hidden = m ? m->hidden : 0;
  if (layers) *layers = m ? m->layers : 0;
}

pskel_status pskel_mlp_get_params(const pskel_mlp* m, float* host) {
  clear_error();
  if (!m || !host) return fail(PSKEL_ERR_INVALID, "MLP: NULL argument");
  cudaError_t e = cudaMemcpy(host, m->d_params, sizeof(float) * m->nparams, cudaMemcpyDeviceToHost);
  return e == cudaSuccess ? PSKEL_OK : cuda_fail(e, "MLP get params");
}

pskel_status pskel_mlp_set_params(pskel_mlp* m, const float* host) {
  clear_error();
  if (!m || !host) return fail(PSKEL_ERR_INVALID, "MLP: NULL argument");
  cudaError_t e = cudaMemcpy(m->d_params, host, sizeof(float) * m->nparams, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(m->d_m, 0, sizeof(float) * m->nparams);
  if (e == cudaSuccess) e = cudaMemset(m->d_v, 0, sizeof(float) * m->nparams);
  m->step = 0;
  return e == cudaSuccess ? PSKEL_OK : cuda_fail(e, "MLP set params");
}

pskel_status pskel_mlp_predict(pskel_mlp* m, const float* x_host, int32_t n, float* y_host) {
  clear_error();
  if (!m || !x_host || !y_host || n <= 0) return fail(PSKEL_ERR_INVALID, "MLP predict: bad arguments");
  if (pskel_status s = mlp_reserve(m, n)) return s;
  cudaError_t e = cudaMemcpyAsync(m->d_x, x_host, sizeof(float) * n * m->in_dim, cudaMemcpyHostToDevice, m->stream);
  if (e != cudaSuccess) return cuda_fail(e, "MLP predict copy");
  mlp_forward(m, n);
  e = cudaMemcpyAsync(y_host, m->d_act[m->layers - 1], sizeof(float) * n, cudaMemcpyDeviceToHost, m->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
  return e == cudaSuccess ? PSKEL_OK : cuda_fail(e, "MLP predict");
}

pskel_status pskel_mlp_gradient(pskel_mlp* m, const float* x_host, const float* y_host, int32_t n, float* grads_host,
                                float* loss) {
  clear_error();
  if (!m || !x_host || !y_host || n <= 0) return fail(PSKEL_ERR_INVALID, "MLP gradient: bad arguments");
  if (pskel_status s = mlp_reserve(m, n)) return s;
  cudaError_t e = cudaMemcpyAsync(m->d_x, x_host, sizeof(float) * n * m->in_dim, cudaMemcpyHostToDevice, m->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(m->d_y, y_host, sizeof(float) * n, cudaMemcpyHostToDevice, m->stream);
  if (e != cudaSuccess) return cuda_fail(e, "MLP gradient copy");
  mlp_forward(m, n);
  mlp_backward(m, n);
  if (grads_host)
    e = cudaMemcpyAsync(grads_host, m->d_grads, sizeof(float) * m->nparams, cudaMemcpyDeviceToHost, m->stream);
  float sum = 0.0f;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&sum, m->d_loss, sizeof(float), cudaMemcpyDeviceToHost, m->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
  if (e != cudaSuccess) return cuda_fail(e, "MLP gradient");
  if (loss) *loss = sum / static_cast<float>(n);
  return PSKEL_OK;
}

pskel_status pskel_mlp_train(pskel_mlp* m, const float* x_host, const float* y_host, int32_t n, int32_t epochs,
                             float lr, float* final_loss) {
  clear_error();
  if (!m || !x_host || !y_host || n <= 0 || epochs < 0) return fail(PSKEL_ERR_INVALID, "MLP train: bad arguments");
  if (pskel_status s = mlp_reserve(m, n)) return s;
  cudaError_t e = cudaMemcpyAsync(m->d_x, x_host, sizeof(float) * n * m->in_dim, cudaMemcpyHostToDevice, m->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(m->d_y, y_host, sizeof(float) * n, cudaMemcpyHostToDevice, m->stream);
  if (e != cudaSuccess) return cuda_fail(e, "MLP train copy");
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  for (int ep = 0; ep < epochs; ++ep) {
    mlp_forward(m, n);
    mlp_backward(m, n);
    ++m->step;
    const float c1 = 1.0f - std::pow(b1, static_cast<float>(m->step));
    const float c2 = 1.0f - std::pow(b2, static_cast<float>(m->step));
    adam_step<<<blocks(static_cast<int>(m->nparams)), 256, 0, m->stream>>>(
        m->d_params, m->d_grads, m->d_m, m->d_v, static_cast<int>(m->nparams), lr, b1, b2, eps, c1, c2);
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "MLP train launch");
  // loss of the final parameters
  mlp_forward(m, n);
  mlp_backward(m, n);
  float sum = 0.0f;
  e = cudaMemcpyAsync(&sum, m->d_loss, sizeof(float), cudaMemcpyDeviceToHost, m->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
  if (e != cudaSuccess) return cuda_fail(e, "MLP train");
  if (final_loss) *final_loss = sum / static_cast<float>(n);
  return PSKEL_OK;
}

pskel_status pskel_mlp_destroy(pskel_mlp* m) {
  clear_error();
  if (!m) return PSKEL_OK;
  cudaFree(m->d_params);
  cudaFree(m->d_grads);
  cudaFree(m->d_m);
  cudaFree(m->d_v);
  cudaFree(m->d_loss);
  cudaFree(m->d_x);
  cudaFree(m->d_y);
  for (float* p : m->d_act) cudaFree(p);
  for (float* p : m->d_delta) cudaFree(p);
  cudaFree(m->d_sq);
  if (m->stream) cudaStreamDestroy(m->stream);
  delete m;
  return PSKEL_OK;
}

}  // extern "C"
