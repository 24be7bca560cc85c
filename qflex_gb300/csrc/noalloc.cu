// Skinny complex products (dot products and narrow matrix-vector products
// with a long contraction) for callers that must not allocate device
// memory: the split-k partial sums live in a fixed array inside this
// library instead of a buffer obtained from cudaMalloc.
//
// Who needs this: cudaMalloc and cudaFree can synchronize the whole device,
// so code that keeps the GPU busy with asynchronous work (or that reserved
// its whole memory budget up front and may not take more) cannot afford an
// allocation, or even the first-use allocation an engine context makes, in
// the middle of a call. This entry point needs no context and allocates
// nothing: the caller passes the inputs, the output and a stream.
//
// The array is a file-scope __device__ variable, so every GPU that loads the
// library holds kNoAllocPartials * 8 bytes (512 KiB) until the process exits.
// In host code the array's name is not a device address; its address is
// fetched once per device with cudaGetSymbolAddress (on the first call made
// with that device current) and passed to the kernels.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/qflex_gb300.h"
#include "kernels.h"

namespace {

constexpr std::size_t kNoAllocPartials = std::size_t(1) << 16;  // float2 slots
constexpr int kMaxDevices = 64;

static __device__ __align__(256) float2 g_noalloc_partials[kNoAllocPartials];

std::mutex g_setup_mutex;
float2* g_partials_of_device[kMaxDevices] = {};

void put_error(char* err, std::size_t err_len, const char* msg) {
  if (err && err_len) {
    std::strncpy(err, msg, err_len - 1);
    err[err_len - 1] = '\0';
  }
}

}  // namespace

extern "C" int qflex_gb300_multiply_skinny_noalloc(const void* A, const void* B, void* C, size_t m,
                                                   size_t n, size_t k, void* stream, char* err,
                                                   size_t err_len) {
  if (!A || !B || !C) {
    put_error(err, err_len, "A, B and C must be non-null device pointers.");
    return QFLEX_GB300_ERR_ARG;
  }
  // m and n are bounded before m * n is formed, so the product cannot wrap.
  if (m > 64 || n > 64 || m * n > 64) {
    put_error(err, err_len,
              "qflex_gb300_multiply_skinny_noalloc takes at most 64 outputs (m * n <= 64); use "
              "qflex_gb300_multiply for larger products.");
    return QFLEX_GB300_ERR_ARG;
  }
  const std::size_t outputs = m * n;
  if (outputs == 0) return QFLEX_GB300_OK;
  // One split per 4096 terms, capped so outputs * splits fits the array.
  std::size_t splits = (k + 4095) / 4096;
  if (splits < 1) splits = 1;
  const std::size_t max_splits = kNoAllocPartials / outputs;
  if (splits > max_splits) splits = max_splits;
  if (outputs * splits > kNoAllocPartials) {
    put_error(err, err_len, "product exceeds the fixed partial-sum array (65536 slots).");
    return QFLEX_GB300_ERR_ARG;
  }

  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    put_error(err, err_len, e != cudaSuccess ? cudaGetErrorString(e) : "device index out of range");
    return QFLEX_GB300_ERR_CUDA;
  }
  float2* partials = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_partials_of_device[dev]) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_noalloc_partials);  // `dev` is current here
      if (e != cudaSuccess) {
        put_error(err, err_len, cudaGetErrorString(e));
        return QFLEX_GB300_ERR_CUDA;
      }
      g_partials_of_device[dev] = static_cast<float2*>(p);
    }
    partials = g_partials_of_device[dev];
  }
  try {
    qfx::launch_skinny_split(static_cast<const float2*>(A), static_cast<const float2*>(B),
                             static_cast<float2*>(C), m, n, k, (int)splits, partials,
                             static_cast<cudaStream_t>(stream));
  } catch (const std::string& msg) {
    put_error(err, err_len, msg.c_str());
    return QFLEX_GB300_ERR_CUDA;
  } catch (...) {  // nothing may cross the C ABI
    put_error(err, err_len, "unknown exception");
    return QFLEX_GB300_ERR_CUDA;
  }
  return QFLEX_GB300_OK;
}
