// Training and inference kernels of the learned cost model: a 3-layer
// perceptron  y = W3 relu(W2 relu(W1 x + b1) + b2) + b3  (FP32), trained on
// the engine's own per-op timings with mean-squared error and Adam.
//
// Parameters are one packed array: W1[h][d], b1[h], W2[h][h], b2[h],
// W3[h], b3 (row-major, h = hidden width, d = input width). Activations of
// a forward pass are kept in a caller-provided work array: H1[n][h] then
// H2[n][h] then the output y[n] then the backward buffers dH2[n][h],
// dH1[n][h], dy[n]. Every reduction over samples runs in a fixed order, so
// a training run is deterministic.
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <string>

#include "../../include/qflex_gb300.h"

namespace {

struct Layout {
  std::size_t w1, b1, w2, b2, w3, b3, count;
};

Layout layout(int d, int h) {
  Layout L{};
  L.w1 = 0;
  L.b1 = L.w1 + std::size_t(h) * d;
  L.w2 = L.b1 + h;
  L.b2 = L.w2 + std::size_t(h) * h;
  L.w3 = L.b2 + h;
  L.b3 = L.w3 + h;
  L.count = L.b3 + 1;
  return L;
}

// out[i][j] = act(sum_k in[i][k] W[j][k] + b[j]), one thread per (i, j).
__global__ void dense_kernel(const float* __restrict__ in, const float* __restrict__ W,
                             const float* __restrict__ b, float* __restrict__ out, std::size_t n, int din,
                             int dout, int relu) {
  const std::size_t t = std::size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= n * dout) return;
  const std::size_t i = t / dout;
  const int j = int(t % dout);
  float acc = b[j];
  for (int k = 0; k < din; ++k) acc = fmaf(in[i * din + k], W[std::size_t(j) * din + k], acc);
  out[t] = relu ? fmaxf(acc, 0.f) : acc;
}

// dy[i] = 2 (y[i] - target[i]) / n and the loss sum((y - target)^2) / n,
// summed by one block in index order.
__global__ void mse_kernel(const float* __restrict__ y, const float* __restrict__ target, float* __restrict__ dy,
                           float* __restrict__ loss, std::size_t n) {
  __shared__ double part[256];
  double s = 0;
  for (std::size_t i = threadIdx.x; i < n; i += blockDim.x) {
    const float e = y[i] - target[i];
    dy[i] = 2.f * e / float(n);
    s += double(e) * e;
  }
  part[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) part[threadIdx.x] += part[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *loss = float(part[0] / double(n));
}

// dIn[i][k] = (sum_j dOut[i][j] W[j][k]) * (mask ? in[i][k] > 0 : 1)
__global__ void back_input_kernel(const float* __restrict__ dout_, const float* __restrict__ W,
                                  const float* __restrict__ act, float* __restrict__ din_, std::size_t n, int din,
                                  int dout) {
  const std::size_t t = std::size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= n * din) return;
  const std::size_t i = t / din;
  const int k = int(t % din);
  float acc = 0.f;
  for (int j = 0; j < dout; ++j) acc = fmaf(dout_[i * dout + j], W[std::size_t(j) * din + k], acc);
  din_[t] = act[t] > 0.f ? acc : 0.f;
}

// gW[j][k] = sum_i dOut[i][j] in[i][k], gb[j] = sum_i dOut[i][j]; one block
// per (j, k) pair (k == din is the bias), a fixed-order tree reduction.
__global__ void back_weight_kernel(const float* __restrict__ dout_, const float* __restrict__ in,
                                   float* __restrict__ gW, float* __restrict__ gb, std::size_t n, int din,
                                   int dout) {
  __shared__ float part[128];
  const int j = blockIdx.x / (din + 1), k = blockIdx.x % (din + 1);
  float s = 0.f;
  for (std::size_t i = threadIdx.x; i < n; i += blockDim.x)
    s = fmaf(dout_[i * dout + j], k < din ? in[i * din + k] : 1.f, s);
  part[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) part[threadIdx.x] += part[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    if (k < din)
      gW[std::size_t(j) * din + k] = part[0];
    else
      gb[j] = part[0];
  }
}

__global__ void adam_kernel(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, std::size_t count, float lr, float b1, float b2, float eps,
                            float c1, float c2) {
  const std::size_t i = std::size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= count) return;
  m[i] = b1 * m[i] + (1.f - b1) * g[i];
  v[i] = b2 * v[i] + (1.f - b2) * g[i] * g[i];
  p[i] -= lr * (m[i] / c1) / (sqrtf(v[i] / c2) + eps);
}

unsigned blocks(std::size_t n, unsigned t) { return unsigned((n + t - 1) / t); }

int check(const char* what) {
  return cudaGetLastError() == cudaSuccess ? QFLEX_GB300_OK : QFLEX_GB300_ERR_CUDA;
}

void forward(cudaStream_t s, const float* P, const float* X, std::size_t n, int d, int h, float* work) {
  const Layout L = layout(d, h);
  float* H1 = work;
  float* H2 = H1 + n * h;
  float* Y = H2 + n * h;
  dense_kernel<<<blocks(n * h, 256), 256, 0, s>>>(X, P + L.w1, P + L.b1, H1, n, d, h, 1);
  dense_kernel<<<blocks(n * h, 256), 256, 0, s>>>(H1, P + L.w2, P + L.b2, H2, n, h, h, 1);
  dense_kernel<<<blocks(n, 256), 256, 0, s>>>(H2, P + L.w3, P + L.b3, Y, n, h, 1, 0);
}

}  // namespace

extern "C" {

size_t qflex_gb300_mlp_param_count(int d_in, int hidden) { return layout(d_in, hidden).count; }

size_t qflex_gb300_mlp_work_floats(size_t n, int hidden) { return n * (4 * size_t(hidden) + 2); }

int qflex_gb300_mlp_forward(void* stream, const float* params, const float* X, size_t n, int d_in, int hidden,
                            float* work, float* y) {
  if (!params || !X || !work || !y || d_in <= 0 || hidden <= 0) return QFLEX_GB300_ERR_ARG;
  if (n == 0) return QFLEX_GB300_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  forward(s, params, X, n, d_in, hidden, work);
  const float* Y = work + 2 * n * hidden;
  cudaMemcpyAsync(y, Y, n * sizeof(float), cudaMemcpyDeviceToDevice, s);
  return check("mlp_forward");
}

int qflex_gb300_mlp_loss_grad(void* stream, const float* params, const float* X, const float* target, size_t n,
                              int d_in, int hidden, float* work, float* grads, float* loss) {
  if (!params || !X || !target || !work || !grads || !loss || d_in <= 0 || hidden <= 0 || n == 0)
    return QFLEX_GB300_ERR_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int d = d_in, h = hidden;
  const Layout L = layout(d, h);
  forward(s, params, X, n, d, h, work);
  float* H1 = work;
  float* H2 = H1 + n * h;
  float* Y = H2 + n * h;
  float* dH2 = Y + n;
  float* dH1 = dH2 + n * h;
  float* dY = dH1 + n * h;
  mse_kernel<<<1, 256, 0, s>>>(Y, target, dY, loss, n);
  // Layer 3: y = W3 . H2 + b3.
  back_weight_kernel<<<unsigned(1 * (h + 1)), 128, 0, s>>>(dY, H2, grads + L.w3, grads + L.b3, n, h, 1);
  back_input_kernel<<<blocks(n * h, 256), 256, 0, s>>>(dY, params + L.w3, H2, dH2, n, h, 1);
  // Layer 2.
  back_weight_kernel<<<unsigned(h * (h + 1)), 128, 0, s>>>(dH2, H1, grads + L.w2, grads + L.b2, n, h, h);
  back_input_kernel<<<blocks(n * h, 256), 256, 0, s>>>(dH2, params + L.w2, H1, dH1, n, h, h);
  // Layer 1 (no input gradient needed).
  back_weight_kernel<<<unsigned(h * (d + 1)), 128, 0, s>>>(dH1, X, grads + L.w1, grads + L.b1, n, d, h);
  return check("mlp_loss_grad");
}

int qflex_gb300_mlp_adam(void* stream, float* params, const float* grads, float* m, float* v, size_t count,
                         int step, float lr) {
  if (!params || !grads || !m || !v || step < 1) return QFLEX_GB300_ERR_ARG;
  const float b1 = 0.9f, b2 = 0.999f;
  float c1 = 1.f, c2 = 1.f;
  for (int i = 0; i < step; ++i) {
    c1 *= b1;
    c2 *= b2;
  }
  adam_kernel<<<blocks(count, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      params, grads, m, v, count, lr, b1, b2, 1e-8f, 1.f - c1, 1.f - c2);
  return check("mlp_adam");
}

}  // extern "C"
