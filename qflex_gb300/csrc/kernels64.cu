// sm_103a kernels of the complex128 (FP64) contraction path: the GPU oracle
// that the complex64 paths are measured against. Tensors are complex128 in
// HBM (double2, 16 bytes per element), gate tensors come from the
// double-precision gate constants, and amplitudes are summed in FP64.
//
// GB300's FP64 pipes run at about 1/64 of the FP32 rate (a cuBLAS ZGEMM
// measured 1.1 TFLOP/s on this GPU), so the tiled products have two
// arithmetic modes over the same complex128 operands:
//   * native: every multiply-add is an FP64 FMA;
//   * float-float: each operand is split into an unevaluated sum of two
//     floats (h + l, about 48 significant bits) when it is staged in shared
//     memory, products are formed exactly with FMA and accumulated with
//     Knuth's two-sum into a float-float accumulator (renormalized every 16
//     terms), and the result is rounded once to double. About 44 correct
//     bits for these sums, on the FP32 pipes.
// Everything else (flatten, permutations, skinny products, sums) is FP64.
#include <algorithm>
#include <string>

#include "kernels.h"

namespace qfx {

namespace {

void check_launch(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) throw std::string("ERROR (qflex_gb300: launch ") + what + ") --> " + cudaGetErrorString(e);
}

__device__ __forceinline__ double2 zfma(double2 a, double2 b, double2 c) {
  c.x = fma(a.x, b.x, c.x);
  c.x = fma(-a.y, b.y, c.x);
  c.y = fma(a.x, b.y, c.y);
  c.y = fma(a.y, b.x, c.y);
  return c;
}
__device__ __forceinline__ double2 zmul(double2 a, double2 b) {
  return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}

// ---------------------------------------------------------------------------
// Column flatten in FP64 (the chain of 2x2 gate matrices of one qubit, as in
// the complex64 flatten, from the double gate constants).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) flatten64_kernel(const ColumnDesc* __restrict__ cols,
                                                        const StepDesc* __restrict__ steps,
                                                        const double2* __restrict__ mats,
                                                        const std::uint8_t* __restrict__ init_bits,
                                                        const std::uint8_t* __restrict__ final_bits,
                                                        int n_cols, double2* __restrict__ arena,
                                                        std::uint64_t arena_stride) {
  const int c = blockIdx.y;
  const int b = blockIdx.z;
  const ColumnDesc cd = cols[c];
  const std::uint64_t e = std::uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= (std::uint64_t(1) << cd.size_log2)) return;
  const bool one = init_bits[std::size_t(b) * n_cols + c] != 0;
  double2 p0 = make_double2(one ? 0.0 : 1.0, 0.0), p1 = make_double2(one ? 1.0 : 0.0, 0.0);
  for (std::uint32_t s = cd.step_begin; s < cd.step_end; ++s) {
    const StepDesc sd = steps[s];
    std::uint32_t g = sd.mat;
    std::uint32_t row = 2;
    if (sd.kind == 2) {
      const std::uint32_t v = std::uint32_t(e >> sd.shift) & (sd.V - 1);
      g += 2 * v;
      row = 2 * sd.V;
    }
    const double2 q0 = zfma(p1, mats[g + row], zmul(p0, mats[g]));
    const double2 q1 = zfma(p1, mats[g + row + 1], zmul(p0, mats[g + 1]));
    p0 = q0;
    p1 = q1;
  }
  int bit;
  if (cd.o_shift >= 0)
    bit = int((e >> cd.o_shift) & 1);
  else
    bit = final_bits[std::size_t(b) * n_cols + c];
  arena[std::uint64_t(b) * arena_stride + cd.out_offset + e] = bit ? p1 : p0;
}

// ---------------------------------------------------------------------------
// Float-float arithmetic. The _rn intrinsics keep the compiler from fusing
// the product and the sum of two-sum into one FMA, which would break the
// error-free transformations.
// ---------------------------------------------------------------------------
struct ffc {  // complex float-float: re = rh + rl, im = ih + il
  float rh, rl, ih, il;
};

__device__ __forceinline__ ffc to_ff(double2 z) {
  const float rh = __double2float_rn(z.x), ih = __double2float_rn(z.y);
  return {rh, __double2float_rn(z.x - double(rh)), ih, __double2float_rn(z.y - double(ih))};
}

// (h, l) += (xh + xl) * (yh + yl), dropping xl * yl (below 2^-48 of the
// product).
__device__ __forceinline__ void ff_mac(float& h, float& l, float xh, float xl, float yh, float yl) {
  const float p = __fmul_rn(xh, yh);
  float e = fmaf(xh, yh, -p);  // exact: xh * yh - p
  e = fmaf(xh, yl, e);
  e = fmaf(xl, yh, e);
  const float s = __fadd_rn(h, p);
  const float bb = __fsub_rn(s, h);
  const float t = __fadd_rn(__fsub_rn(h, __fsub_rn(s, bb)), __fsub_rn(p, bb));  // exact: h + p - s
  h = s;
  l = __fadd_rn(l, __fadd_rn(t, e));
}

__device__ __forceinline__ void ff_renorm(float& h, float& l) {
  const float s = __fadd_rn(h, l);
  l = __fsub_rn(l, __fsub_rn(s, h));
  h = s;
}

__device__ __forceinline__ void ffc_mac(ffc& acc, const ffc& a, const ffc& b) {
  ff_mac(acc.rh, acc.rl, a.rh, a.rl, b.rh, b.rl);
  ff_mac(acc.rh, acc.rl, -a.ih, -a.il, b.ih, b.il);
  ff_mac(acc.ih, acc.il, a.rh, a.rl, b.ih, b.il);
  ff_mac(acc.ih, acc.il, a.ih, a.il, b.rh, b.rl);
}

// ---------------------------------------------------------------------------
// Tiled complex128 product C = A * B (row-major, batch entries at
// batch_stride elements). Block tile BM x BN, k-step BK, TM x TN outputs per
// thread; operands pass through shared memory (converted to float-float
// there in FF mode) with a register-staged prefetch of the next k-step.
// ---------------------------------------------------------------------------
template <int BM, int BN, int BK, int TM, int TN, bool FF>
__global__ void __launch_bounds__((BM / TM) * (BN / TN))
    zgemm_kernel(const double2* __restrict__ A, const double2* __restrict__ B, double2* __restrict__ C, int m,
                 int n, int k, std::uint64_t batch_stride) {
  constexpr int NT = (BM / TM) * (BN / TN);
  constexpr int TX = BN / TN;
  constexpr int LA = BM * BK / NT;
  constexpr int LB = BK * BN / NT;
  static_assert(LA * NT == BM * BK && LB * NT == BK * BN, "tile/threads mismatch");
  using S = typename std::conditional<FF, ffc, double2>::type;  // 16 bytes either way
  __shared__ __align__(16) S As[BK][BM + 1];
  __shared__ __align__(16) S Bs[BK][BN + 1];

  const std::uint64_t boff = std::uint64_t(blockIdx.z) * batch_stride;
  A += boff;
  B += boff;
  C += boff;
  const int tiles_m = (m + BM - 1) / BM;
  const int m0 = int(blockIdx.x % tiles_m) * BM;
  const int n0 = int(blockIdx.x / tiles_m) * BN;
  const int t = threadIdx.x;
  const int tx = t % TX, ty = t / TX;

  S acc[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) {
      if constexpr (FF)
        acc[i][j] = ffc{0.f, 0.f, 0.f, 0.f};
      else
        acc[i][j] = make_double2(0.0, 0.0);
    }

  double2 ra[LA], rb[LB];
  auto load = [&](int k0) {
#pragma unroll
    for (int i = 0; i < LA; ++i) {
      const int idx = t + i * NT;
      const int r = idx / BK, c = idx % BK;
      const int gr = m0 + r, gc = k0 + c;
      ra[i] = (gr < m && gc < k) ? A[std::size_t(gr) * k + gc] : make_double2(0.0, 0.0);
    }
#pragma unroll
    for (int i = 0; i < LB; ++i) {
      const int idx = t + i * NT;
      const int r = idx / BN, c = idx % BN;
      const int gr = k0 + r, gc = n0 + c;
      rb[i] = (gr < k && gc < n) ? B[std::size_t(gr) * n + gc] : make_double2(0.0, 0.0);
    }
  };
  auto store = [&]() {
#pragma unroll
    for (int i = 0; i < LA; ++i) {
      const int idx = t + i * NT;
      if constexpr (FF)
        As[idx % BK][idx / BK] = to_ff(ra[i]);
      else
        As[idx % BK][idx / BK] = ra[i];
    }
#pragma unroll
    for (int i = 0; i < LB; ++i) {
      const int idx = t + i * NT;
      if constexpr (FF)
        Bs[idx / BN][idx % BN] = to_ff(rb[i]);
      else
        Bs[idx / BN][idx % BN] = rb[i];
    }
  };

  const int ktiles = (k + BK - 1) / BK;
  load(0);
  store();
  __syncthreads();
  for (int kt = 0; kt < ktiles; ++kt) {
    const bool more = kt + 1 < ktiles;
    if (more) load((kt + 1) * BK);
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      S a[TM], b[TN];
#pragma unroll
      for (int i = 0; i < TM; ++i) a[i] = As[kk][ty * TM + i];
#pragma unroll
      for (int j = 0; j < TN; ++j) b[j] = Bs[kk][tx * TN + j];
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) {
          if constexpr (FF)
            ffc_mac(acc[i][j], a[i], b[j]);
          else
            acc[i][j] = zfma(a[i], b[j], acc[i][j]);
        }
    }
    if constexpr (FF) {
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) {
          ff_renorm(acc[i][j].rh, acc[i][j].rl);
          ff_renorm(acc[i][j].ih, acc[i][j].il);
        }
    }
    __syncthreads();
    if (more) {
      store();
      __syncthreads();
    }
  }
#pragma unroll
  for (int i = 0; i < TM; ++i) {
    const int gr = m0 + ty * TM + i;
    if (gr >= m) continue;
#pragma unroll
    for (int j = 0; j < TN; ++j) {
      const int gc = n0 + tx * TN + j;
      if (gc >= n) continue;
      if constexpr (FF)
        C[std::size_t(gr) * n + gc] = make_double2(double(acc[i][j].rh) + double(acc[i][j].rl),
                                                   double(acc[i][j].ih) + double(acc[i][j].il));
      else
        C[std::size_t(gr) * n + gc] = acc[i][j];
    }
  }
}

__device__ __forceinline__ double2 warp_sum64(double2 v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
    v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
  }
  return v;
}

// C[i] = sum_kk A[i, kk] * B[kk]; one warp per row.
__global__ void __launch_bounds__(256) zgemv_rows(const double2* __restrict__ A, const double2* __restrict__ B,
                                                  double2* __restrict__ C, std::uint64_t m, std::uint64_t k,
                                                  std::uint64_t batch_stride) {
  const std::uint64_t boff = std::uint64_t(blockIdx.y) * batch_stride;
  const std::uint64_t i = (std::uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) / 32;
  const int lane = threadIdx.x & 31;
  if (i >= m) return;
  const double2* a = A + boff + i * k;
  const double2* b = B + boff;
  double2 acc = make_double2(0.0, 0.0);
  for (std::uint64_t kk = lane; kk < k; kk += 32) acc = zfma(a[kk], b[kk], acc);
  acc = warp_sum64(acc);
  if (lane == 0) C[boff + i] = acc;
}

// C[j] = sum_kk A[kk] * B[kk, j]; one thread per column.
__global__ void __launch_bounds__(256) zgemv_cols(const double2* __restrict__ A, const double2* __restrict__ B,
                                                  double2* __restrict__ C, std::uint64_t n, std::uint64_t k,
                                                  std::uint64_t batch_stride) {
  const std::uint64_t boff = std::uint64_t(blockIdx.y) * batch_stride;
  const std::uint64_t j = std::uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const double2* a = A + boff;
  const double2* b = B + boff + j;
  double2 acc = make_double2(0.0, 0.0);
  for (std::uint64_t kk = 0; kk < k; ++kk) acc = zfma(a[kk], b[kk * n], acc);
  C[boff + j] = acc;
}

// Products with few outputs (m * n <= 256) and a long contraction: block
// (r, s) sums chunk s of output r's k range; zskinny_finish adds the
// chunks of each output in chunk order.
__global__ void __launch_bounds__(256) zskinny_partial(const double2* __restrict__ A,
                                                       const double2* __restrict__ B,
                                                       double2* __restrict__ partial, int n, std::uint64_t k,
                                                       int splits, std::uint64_t batch_stride) {
  __shared__ double2 part[8];
  const int r = blockIdx.x / splits, s = blockIdx.x % splits;
  const int i = r / n, j = r % n;
  const std::uint64_t boff = std::uint64_t(blockIdx.y) * batch_stride;
  const std::uint64_t chunk = (k + splits - 1) / splits;
  const std::uint64_t k0 = std::uint64_t(s) * chunk;
  const std::uint64_t k1 = k0 + chunk < k ? k0 + chunk : k;
  const double2* a = A + boff + std::uint64_t(i) * k;
  const double2* b = B + boff + j;
  double2 acc = make_double2(0.0, 0.0);
  for (std::uint64_t kk = k0 + threadIdx.x; kk < k1; kk += blockDim.x) acc = zfma(a[kk], b[kk * n], acc);
  acc = warp_sum64(acc);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x / 32] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    double2 v = threadIdx.x < 8 ? part[threadIdx.x] : make_double2(0.0, 0.0);
    v = warp_sum64(v);
    if (threadIdx.x == 0) partial[std::uint64_t(blockIdx.y) * gridDim.x + blockIdx.x] = v;
  }
}

__global__ void zskinny_finish(const double2* __restrict__ partial, double2* __restrict__ C, int outputs,
                               int splits, std::uint64_t batch_stride) {
  const int r = (blockIdx.x * blockDim.x + threadIdx.x) / 32;
  const int lane = threadIdx.x & 31;
  if (r >= outputs) return;
  const double2* p = partial + (std::uint64_t(blockIdx.y) * outputs + r) * splits;
  double2 acc = make_double2(0.0, 0.0);
  for (int s = lane; s < splits; s += 32) {
    acc.x += p[s].x;
    acc.y += p[s].y;
  }
  acc = warp_sum64(acc);
  if (lane == 0) C[std::uint64_t(blockIdx.y) * batch_stride + r] = acc;
}

__global__ void reduce_amplitudes64_kernel(const double2* __restrict__ results, std::uint64_t stride,
                                           const std::uint32_t* __restrict__ ptr,
                                           const std::uint32_t* __restrict__ leaves, int n_amps,
                                           double2* __restrict__ amps) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  const int b = blockIdx.y;
  if (a >= n_amps) return;
  double re = 0, im = 0;
  const double2* r = results + std::uint64_t(b) * stride;
  for (std::uint32_t p = ptr[a]; p < ptr[a + 1]; ++p) {
    const double2 v = r[leaves[p]];
    re += v.x;
    im += v.y;
  }
  double2& out = amps[std::size_t(b) * n_amps + a];
  out.x += re;
  out.y += im;
}

template <int BM, int BN, int BK, int TM, int TN>
void run_zgemm(const double2* A, const double2* B, double2* C, std::size_t m, std::size_t n, std::size_t k,
               std::uint64_t stride, int batch, bool ff, cudaStream_t s) {
  const std::size_t tiles = ((m + BM - 1) / BM) * ((n + BN - 1) / BN);
  dim3 grid((unsigned)tiles, 1, (unsigned)batch);
  constexpr int NT = (BM / TM) * (BN / TN);
  if (ff)
    zgemm_kernel<BM, BN, BK, TM, TN, true><<<grid, NT, 0, s>>>(A, B, C, (int)m, (int)n, (int)k, stride);
  else
    zgemm_kernel<BM, BN, BK, TM, TN, false><<<grid, NT, 0, s>>>(A, B, C, (int)m, (int)n, (int)k, stride);
  check_launch("zgemm");
}

}  // namespace

int zskinny_splits(std::size_t m, std::size_t n, std::size_t k, int batch) {
  if (m * n > 256 || k < 4096) return 0;
  std::size_t splits = std::min<std::size_t>(2048, (k + 2047) / 2048);
  while (splits > 1 && splits * m * n * (std::size_t)batch > kSkinnyScratchElems64) splits /= 2;
  return splits >= 2 ? (int)splits : 0;
}

void launch_flatten64(const ColumnDesc* cols, int n_cols, std::uint32_t max_size_log2, const StepDesc* steps,
                      const double2* mats, const std::uint8_t* init_bits, const std::uint8_t* final_bits,
                      double2* arena, std::uint64_t arena_stride, int batch, cudaStream_t s) {
  if (n_cols == 0) return;
  const std::uint64_t blocks = ((std::uint64_t(1) << max_size_log2) + 255) / 256;
  dim3 grid((unsigned)blocks, (unsigned)n_cols, (unsigned)batch);
  flatten64_kernel<<<grid, 256, 0, s>>>(cols, steps, mats, init_bits, final_bits, n_cols, arena, arena_stride);
  check_launch("flatten64");
}

void launch_zgemm(const double2* A, const double2* B, double2* C, std::size_t m, std::size_t n, std::size_t k,
                  std::uint64_t stride, int batch, cudaStream_t s, double2* scratch, bool ff) {
  if (const int splits = scratch ? zskinny_splits(m, n, k, batch) : 0) {
    const int outputs = (int)(m * n);
    dim3 g1((unsigned)(outputs * splits), (unsigned)batch);
    zskinny_partial<<<g1, 256, 0, s>>>(A, B, scratch, (int)n, k, splits, stride);
    check_launch("zskinny_partial");
    dim3 g2((unsigned)((outputs * 32 + 127) / 128), (unsigned)batch);
    zskinny_finish<<<g2, 128, 0, s>>>(scratch, C, outputs, splits, stride);
    check_launch("zskinny_finish");
    return;
  }
  if (n == 1) {
    dim3 grid((unsigned)((m * 32 + 255) / 256), (unsigned)batch);
    zgemv_rows<<<grid, 256, 0, s>>>(A, B, C, m, k, stride);
    check_launch("zgemv_rows");
    return;
  }
  if (m == 1 && n >= 256) {
    dim3 grid((unsigned)((n + 255) / 256), (unsigned)batch);
    zgemv_cols<<<grid, 256, 0, s>>>(A, B, C, n, k, stride);
    check_launch("zgemv_cols");
    return;
  }
  if (m > 0x7fffffffull || n > 0x7fffffffull || k > 0x7fffffffull)
    throw std::string("ERROR (qflex_gb300: zgemm) --> dimension exceeds 2^31");
  if (n <= 16)
    run_zgemm<128, 16, 16, 4, 2>(A, B, C, m, n, k, stride, batch, ff, s);
  else if (m <= 16)
    run_zgemm<16, 128, 16, 2, 4>(A, B, C, m, n, k, stride, batch, ff, s);
  else
    run_zgemm<64, 64, 16, 4, 4>(A, B, C, m, n, k, stride, batch, ff, s);
}

void launch_reduce_amplitudes64(const double2* results, std::uint64_t stride, const std::uint32_t* ptr,
                                const std::uint32_t* leaves, int n_amps, double2* amps, int batch,
                                cudaStream_t s) {
  if (n_amps == 0) return;
  dim3 grid((unsigned)((n_amps + 127) / 128), (unsigned)batch);
  reduce_amplitudes64_kernel<<<grid, 128, 0, s>>>(results, stride, ptr, leaves, n_amps, amps);
  check_launch("reduce_amplitudes64");
}

}  // namespace qfx
