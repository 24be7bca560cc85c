// Split-precision complex64 products on the tcgen05 tensor cores.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace qfx {

// Shapes the tensor-core kernel takes (k a multiple of 4 for the TMA row
// stride; smaller products stay on the CUDA-core kernels).
bool tc_eligible(std::size_t m, std::size_t n, std::size_t k);
// fp32 elements of split planes one batch entry needs (A and B, 4 planes).
std::size_t tc_workspace_elems(std::size_t m, std::size_t n, std::size_t k);

// Kernel choice of one product.
struct TcConfig {
  int chunk = 2;     // k-steps per TMEM accumulation chunk, 1..64 (QFLEX_TC_CHUNK)
  int variant = 0;   // 0: single CTA; 1: CTA pair; -1: CTA pair when m >= 256, else single;
                     // 2: 3xFP16 single CTA with five stages; 3: 3xFP16 single CTA with 16
                     // epilogue warps; 4: 3xFP16 single CTA with 64-column tiles and four
                     // TMEM chunk buffers (others: single CTA)
};
// Defaults: chunk from QFLEX_TC_CHUNK, variant -1 when QFLEX_TC_PAIR=1, 2 when
// QFLEX_TC_DEEP=1.
TcConfig tc_default_config();

// C[m,n] = A[m,k] * Bt[n,k]^T (complex64, both K-major), 3xTF32 split,
// FP32 accumulation. Batch entry b reads A + b * ac_stride,
// Bt + b * bt_stride and writes C + b * ac_stride. `workspace` holds
// batch * tc_workspace_elems fp32; `err` (device int) receives a nonzero
// code if a pipeline wait expired.
void launch_cgemm_tf32x3(const float2* A, const float2* Bt, float2* C, std::size_t m, std::size_t n,
                         std::size_t k, std::uint64_t ac_stride, std::uint64_t bt_stride, int batch,
                         float* workspace, int* err, const TcConfig& cfg, cudaStream_t s);

// Where the 3xFP16 product keeps its operands in `workspace` (batch entries
// after each other in every region): A planes, Bt planes, the row exponents
// of A and of Bt, and the block exponents of an A operand that arrives as
// planes (one per 32 values of a row).
struct Fp16Workspace {
  void* a_planes;
  void* b_planes;
  int* a_exps;
  int* b_exps;
  int* a_block_exps;
};
Fp16Workspace fp16_workspace(float* workspace, std::size_t m, std::size_t n, std::size_t k, int batch);

// The same product with 3xFP16 planes: every row of A and of Bt is scaled by
// a power of two so that its largest component lies in [2^14, 2^15), split
// into FP16 hi + lo, multiplied as hi*hi + hi*lo + lo*hi on kind::f16
// tensor cores (twice the TF32 rate) and unscaled in the epilogue. Always
// the single-CTA kernel; cfg.variant is ignored.
// With `a_in_planes` the A planes and block exponents are already in the
// workspace (written by launch_permute_fp16_planes; k a power of two >= 32,
// cfg.chunk <= 2 so that a TMEM chunk never spans two exponent blocks) and
// A is not read.
void launch_cgemm_fp16x3(const float2* A, const float2* Bt, float2* C, std::size_t m, std::size_t n,
                         std::size_t k, std::uint64_t ac_stride, std::uint64_t bt_stride, int batch,
                         float* workspace, int* err, const TcConfig& cfg, cudaStream_t s,
                         bool a_in_planes = false);

// The same product with BF16x3 planes: x = b0 + b1 + b2 in BF16 (no
// scaling: BF16 has the FP32 exponent range), six products per real
// product (x0y0, x0y1, x1y0, x0y2, x1y1, x2y0) on kind::f16 tensor cores.
// Single-CTA kernel; cfg.variant is ignored.
void launch_cgemm_bf16x3(const float2* A, const float2* Bt, float2* C, std::size_t m, std::size_t n,
                         std::size_t k, std::uint64_t ac_stride, std::uint64_t bt_stride, int batch,
                         float* workspace, int* err, const TcConfig& cfg, cudaStream_t s);

}  // namespace qfx
