// sm_103a kernels of the contraction path: column flatten, binary-digit
// permutation, complex64 products on CUDA cores, FP64 amplitude sums.
#include <algorithm>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_fp16.h>

#include "kernels.h"

namespace qfx {

namespace {

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ float2 cfma(float2 a, float2 b, float2 c) {
  c.x = fmaf(a.x, b.x, c.x);
  c.x = fmaf(-a.y, b.y, c.x);
  c.y = fmaf(a.x, b.y, c.y);
  c.y = fmaf(a.y, b.x, c.y);
  return c;
}

void check_launch(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) throw std::string("ERROR (qflex_gb300: launch ") + what + ") --> " + cudaGetErrorString(e);
}

// ---------------------------------------------------------------------------
// Column flatten.
// ---------------------------------------------------------------------------
// Float-float numbers (an unevaluated sum h + l of two floats, ~44
// significant bits) built from the classic error-free transformations:
// Knuth's two-sum and the FMA-based exact product.
struct ff {
  float h, l;
};
__device__ __forceinline__ ff ff_add(ff a, ff b) {
  const float s = a.h + b.h;
  const float bb = s - a.h;
  float e = (a.h - (s - bb)) + (b.h - bb);
  e += a.l + b.l;
  const float h = s + e;
  return {h, e - (h - s)};
}
__device__ __forceinline__ ff ff_mul(ff a, ff b) {
  const float p = a.h * b.h;
  float e = fmaf(a.h, b.h, -p);
  e = fmaf(a.h, b.l, e);
  e = fmaf(a.l, b.h, e);
  const float h = p + e;
  return {h, e - (h - p)};
}
__device__ __forceinline__ ff ff_neg(ff a) { return {-a.h, -a.l}; }
struct cff {
  ff re, im;
};
__device__ __forceinline__ cff cff_mul(cff a, cff b) {
  return {ff_add(ff_mul(a.re, b.re), ff_neg(ff_mul(a.im, b.im))),
          ff_add(ff_mul(a.re, b.im), ff_mul(a.im, b.re))};
}
__device__ __forceinline__ cff cff_add(cff a, cff b) { return {ff_add(a.re, b.re), ff_add(a.im, b.im)}; }
__device__ __forceinline__ cff cff_load(const float2* hi, const float2* lo, std::uint32_t i) {
  const float2 h = __ldg(hi + i), l = __ldg(lo + i);
  return {{h.x, l.x}, {h.y, l.y}};
}

// Element e of a column's 2D tensor: <final| G_K ... G_1 |init> with every
// two-qubit half reading its virtual digit of e. Plain FP32 repeats the
// reference's complex<float> arithmetic on its float gate constants; the
// compensated form carries float-float values and gate constants (hi + lo
// of the double-precision gate) and rounds once at the end.
template <bool kCompensated>
__global__ void __launch_bounds__(256) flatten_kernel(const ColumnDesc* __restrict__ cols,
                                                      const StepDesc* __restrict__ steps,
                                                      const float2* __restrict__ mats,
                                                      const float2* __restrict__ mats_lo,
                                                      const std::uint8_t* __restrict__ init_bits,
                                                      const std::uint8_t* __restrict__ final_bits,
                                                      int n_cols, float2* __restrict__ arena,
                                                      std::uint64_t arena_stride) {
  const int c = blockIdx.y;
  const int b = blockIdx.z;
  const ColumnDesc cd = cols[c];
  const std::uint64_t e = std::uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= (std::uint64_t(1) << cd.size_log2)) return;
  const bool one = init_bits[std::size_t(b) * n_cols + c] != 0;
  float2 p0 = make_float2(one ? 0.f : 1.f, 0.f), p1 = make_float2(one ? 1.f : 0.f, 0.f);
  cff f0 = {{p0.x, 0.f}, {0.f, 0.f}}, f1 = {{p1.x, 0.f}, {0.f, 0.f}};
  for (std::uint32_t s = cd.step_begin; s < cd.step_end; ++s) {
    const StepDesc sd = steps[s];
    std::uint32_t g = sd.mat;
    std::uint32_t row = 2;  // distance between input rows of the gate data
    if (sd.kind == 2) {
      const std::uint32_t v = std::uint32_t(e >> sd.shift) & (sd.V - 1);
      g += 2 * v;
      row = 2 * sd.V;
    }
    if constexpr (kCompensated) {
      const cff q0 = cff_add(cff_mul(f0, cff_load(mats, mats_lo, g)),
                             cff_mul(f1, cff_load(mats, mats_lo, g + row)));
      const cff q1 = cff_add(cff_mul(f0, cff_load(mats, mats_lo, g + 1)),
                             cff_mul(f1, cff_load(mats, mats_lo, g + row + 1)));
      f0 = q0;
      f1 = q1;
    } else {
      const float2 q0 = cfma(p1, __ldg(mats + g + row), cmul(p0, __ldg(mats + g)));
      const float2 q1 = cfma(p1, __ldg(mats + g + row + 1), cmul(p0, __ldg(mats + g + 1)));
      p0 = q0;
      p1 = q1;
    }
  }
  if constexpr (kCompensated) {
    p0 = make_float2(f0.re.h + f0.re.l, f0.im.h + f0.im.l);
    p1 = make_float2(f1.re.h + f1.re.l, f1.im.h + f1.im.l);
  }
  int bit;
  if (cd.o_shift >= 0)
    bit = int((e >> cd.o_shift) & 1);
  else
    bit = final_bits[std::size_t(b) * n_cols + c];
  arena[std::uint64_t(b) * arena_stride + cd.out_offset + e] = bit ? p1 : p0;
}

// ---------------------------------------------------------------------------
// Binary-digit permutation.
// ---------------------------------------------------------------------------
// Output of the FP16-plane form of the permutation (see
// launch_permute_fp16_planes).
struct PlaneOut {
  __half* planes;
  int* exps;
  std::uint64_t rows;
  std::uint32_t k_log2;
};

// E is the element: float2 (complex64) or double2 (complex128; no planes).
template <typename E, bool PLANES>
__global__ void __launch_bounds__(256, 8) permute_kernel(const __grid_constant__ PermPlan P,
                                                      const E* __restrict__ src,
                                                      E* __restrict__ dst,
                                                      std::uint64_t batch_stride, PlaneOut po) {
  __shared__ E tile[1024];
  __shared__ std::uint32_t tab[6 * 32];
  if (threadIdx.x < 6 * 32) tab[threadIdx.x] = P.tab[threadIdx.x / 32][threadIdx.x % 32];
  __syncthreads();
  const std::uint32_t T = 1u << P.tile_bits;
  const E* s = src + std::uint64_t(blockIdx.y) * batch_stride;
  E* d = dst + std::uint64_t(blockIdx.y) * batch_stride;
  // The next tile's loads are issued into registers before the current
  // tile is stored, so loads stay in flight through the store phase.
  E r[4];
  auto load = [&](std::uint64_t t) {
    std::uint64_t bi, bo;
    perm_tile_base(P, t, &bi, &bo);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const std::uint32_t j = threadIdx.x + 256u * i;
      if (j < T) r[i] = __ldcs(s + bi + tab[j & 31] + tab[32 + (j >> 5)]);
    }
  };
  std::uint64_t t = blockIdx.x;
  if (t < P.n_tiles) load(t);
  for (; t < P.n_tiles; t += gridDim.x) {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const std::uint32_t j = threadIdx.x + 256u * i;
      if (j < T) tile[perm_swizzle(j)] = r[i];
    }
    __syncthreads();
    if (t + gridDim.x < P.n_tiles) load(t + gridDim.x);
    std::uint64_t bi, bo;
    perm_tile_base(P, t, &bi, &bo);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const std::uint32_t j = threadIdx.x + 256u * i;
      if (j >= T) continue;  // T is a multiple of 32 here: whole warps
      const std::uint64_t o = bo + tab[64 + (j & 31)] + tab[96 + (j >> 5)];
      const E v = tile[perm_swizzle(tab[128 + (j & 31)] + tab[160 + (j >> 5)])];
      if constexpr (!PLANES) {
        d[o] = v;
        continue;
      } else {
      // The warp's 32 values are outputs o - lane .. o - lane + 31: one
      // 32-aligned run of a row (the tile holds the 5 lowest output digits).
      // Its largest |re| or |im|: bit patterns of non-negative floats order
      // like their values, so one integer warp reduction finds it.
      const std::uint32_t mb = __reduce_max_sync(
          0xffffffffu, max(__float_as_uint(fabsf(v.x)), __float_as_uint(fabsf(v.y))));
      // e with max * 2^e in [2^14, 2^15): a normal max of biased exponent be
      // lies in [2^(be-127), 2^(be-126)); infinities and NaN keep e = 0.
      const int be = int(mb >> 23);
      int e = 0;
      if (be > 0 && be < 255) {
        e = 141 - be;
      } else if (be == 0 && mb != 0) {
        int ex;
        frexpf(__uint_as_float(mb), &ex);  // subnormal
        e = 15 - ex;
      }
      const std::uint64_t k = std::uint64_t(1) << po.k_log2;
      const std::uint64_t row = o >> po.k_log2, kk = o & (k - 1);
      // Scaling by 2^e is exact: a multiply when 2^e is a normal float.
      const bool direct = e >= -126 && e <= 127;
      const float sc = __uint_as_float(std::uint32_t(direct ? e + 127 : 127) << 23);
      const float xr = direct ? v.x * sc : ldexpf(v.x, e), xi = direct ? v.y * sc : ldexpf(v.y, e);
      const __half2 hi = __floats2half2_rn(xr, xi);  // (re_hi, im_hi)
      const float2 hf = __half22float2(hi);
      const __half2 lo = __floats2half2_rn(xr - hf.x, xi - hf.y);
      __half* pl = po.planes + std::uint64_t(blockIdx.y) * 4 * po.rows * k + ((kk / 16) * po.rows + row) * 64 +
                   (kk % 16);
      pl[0] = __low2half(hi);
      pl[16] = __low2half(lo);
      pl[32] = __high2half(hi);
      pl[48] = __high2half(lo);
      if ((threadIdx.x & 31) == 0)
        po.exps[std::uint64_t(blockIdx.y) * po.rows * (k / 32) + row * (k / 32) + kk / 32] = e;
      }
    }
    __syncthreads();
  }
}

// Index decomposition shared by the general permutation kernel and its host
// mirror: the input offset of output element o.
__host__ __device__ inline std::uint64_t general_source(const GeneralPerm& g, std::uint64_t o) {
  std::uint64_t in = 0;
  for (int i = int(g.rank) - 1; i >= 0; --i) {
    const std::uint64_t d = g.out_dims[i];
    const std::uint64_t q = o / d;
    in += (o - q * d) * g.in_stride[i];
    o = q;
  }
  return in;
}

__global__ void __launch_bounds__(256) permute_general_kernel(const __grid_constant__ GeneralPerm g,
                                                              const float2* __restrict__ src,
                                                              float2* __restrict__ dst,
                                                              std::uint64_t batch_stride) {
  const float2* s = src + std::uint64_t(blockIdx.y) * batch_stride;
  float2* d = dst + std::uint64_t(blockIdx.y) * batch_stride;
  for (std::uint64_t o = std::uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; o < g.size;
       o += std::uint64_t(gridDim.x) * blockDim.x)
    d[o] = __ldg(s + general_source(g, o));
}

// ---------------------------------------------------------------------------
// Complex64 GEMM on CUDA cores (C = A * B, row-major).
// Block tile BM x BN, k-step BK; each thread owns a TM x TN sub-tile.
// Operands pass through shared memory with a register-staged prefetch of
// the next k-step.
// ---------------------------------------------------------------------------
template <int BM, int BN, int BK, int TM, int TN>
__global__ void __launch_bounds__((BM / TM) * (BN / TN))
    cgemm_kernel(const float2* __restrict__ A, const float2* __restrict__ B, float2* __restrict__ C,
                 int m, int n, int k, std::uint64_t batch_stride) {
  constexpr int NT = (BM / TM) * (BN / TN);
  constexpr int TX = BN / TN;
  constexpr int LA = BM * BK / NT;
  constexpr int LB = BK * BN / NT;
  static_assert(LA * NT == BM * BK && LB * NT == BK * BN, "tile/threads mismatch");
  __shared__ __align__(16) float2 As[BK][BM + 2];
  __shared__ __align__(16) float2 Bs[BK][BN + 2];

  const std::uint64_t boff = std::uint64_t(blockIdx.z) * batch_stride;
  A += boff;
  B += boff;
  C += boff;
  const int tiles_m = (m + BM - 1) / BM;
  const int m0 = int(blockIdx.x % tiles_m) * BM;
  const int n0 = int(blockIdx.x / tiles_m) * BN;
  const int t = threadIdx.x;
  const int tx = t % TX, ty = t / TX;

  float2 acc[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) acc[i][j] = make_float2(0.f, 0.f);

  float2 ra[LA], rb[LB];
  auto load = [&](int k0) {
#pragma unroll
    for (int i = 0; i < LA; ++i) {
      const int idx = t + i * NT;
      const int r = idx / BK, c = idx % BK;
      const int gr = m0 + r, gc = k0 + c;
      ra[i] = (gr < m && gc < k) ? A[std::size_t(gr) * k + gc] : make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int i = 0; i < LB; ++i) {
      const int idx = t + i * NT;
      const int r = idx / BN, c = idx % BN;
      const int gr = k0 + r, gc = n0 + c;
      rb[i] = (gr < k && gc < n) ? B[std::size_t(gr) * n + gc] : make_float2(0.f, 0.f);
    }
  };
  auto store = [&]() {
#pragma unroll
    for (int i = 0; i < LA; ++i) {
      const int idx = t + i * NT;
      As[idx % BK][idx / BK] = ra[i];
    }
#pragma unroll
    for (int i = 0; i < LB; ++i) {
      const int idx = t + i * NT;
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
      float2 a[TM], b[TN];
#pragma unroll
      for (int i = 0; i < TM; ++i) a[i] = As[kk][ty * TM + i];
#pragma unroll
      for (int j = 0; j < TN; ++j) b[j] = Bs[kk][tx * TN + j];
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) acc[i][j] = cfma(a[i], b[j], acc[i][j]);
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
      if (gc < n) C[std::size_t(gr) * n + gc] = acc[i][j];
    }
  }
}

__device__ __forceinline__ float2 warp_sum(float2 v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
    v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
  }
  return v;
}

// C[i] = sum_kk A[i, kk] * B[kk]; one thread per row (short rows).
__global__ void __launch_bounds__(256) gemv_rows_thread(const float2* __restrict__ A,
                                                        const float2* __restrict__ B,
                                                        float2* __restrict__ C, std::uint64_t m,
                                                        int k, std::uint64_t batch_stride) {
  const std::uint64_t boff = std::uint64_t(blockIdx.y) * batch_stride;
  const std::uint64_t i = std::uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= m) return;
  const float2* a = A + boff + i * k;
  const float2* b = B + boff;
  float2 acc = make_float2(0.f, 0.f);
  for (int kk = 0; kk < k; ++kk) acc = cfma(a[kk], b[kk], acc);
  C[boff + i] = acc;
}

// Same, one warp per row (long rows).
__global__ void __launch_bounds__(256) gemv_rows_warp(const float2* __restrict__ A,
                                                      const float2* __restrict__ B,
                                                      float2* __restrict__ C, std::uint64_t m,
                                                      std::uint64_t k, std::uint64_t batch_stride) {
  const std::uint64_t boff = std::uint64_t(blockIdx.y) * batch_stride;
  const std::uint64_t i = (std::uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) / 32;
  const int lane = threadIdx.x & 31;
  if (i >= m) return;
  const float2* a = A + boff + i * k;
  const float2* b = B + boff;
  float2 acc = make_float2(0.f, 0.f);
  for (std::uint64_t kk = lane; kk < k; kk += 32) acc = cfma(a[kk], b[kk], acc);
  acc = warp_sum(acc);
  if (lane == 0) C[boff + i] = acc;
}

// C[j] = sum_kk A[kk] * B[kk, j]; one thread per column (wide rows of B).
__global__ void __launch_bounds__(256) gemv_cols_thread(const float2* __restrict__ A,
                                                        const float2* __restrict__ B,
                                                        float2* __restrict__ C, std::uint64_t n,
                                                        std::uint64_t k, std::uint64_t batch_stride) {
  const std::uint64_t boff = std::uint64_t(blockIdx.y) * batch_stride;
  const std::uint64_t j = std::uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const float2* a = A + boff;
  const float2* b = B + boff + j;
  float2 acc = make_float2(0.f, 0.f);
  for (std::uint64_t kk = 0; kk < k; ++kk) acc = cfma(a[kk], b[kk * n], acc);
  C[boff + j] = acc;
}

// Same, one block per column with a block-wide reduction (narrow B).
__global__ void __launch_bounds__(256) gemv_cols_block(const float2* __restrict__ A,
                                                       const float2* __restrict__ B,
                                                       float2* __restrict__ C, std::uint64_t n,
                                                       std::uint64_t k, std::uint64_t batch_stride) {
  __shared__ float2 part[8];
  const std::uint64_t boff = std::uint64_t(blockIdx.y) * batch_stride;
  const std::uint64_t j = blockIdx.x;
  const float2* a = A + boff;
  const float2* b = B + boff + j;
  float2 acc = make_float2(0.f, 0.f);
  for (std::uint64_t kk = threadIdx.x; kk < k; kk += blockDim.x) acc = cfma(a[kk], b[kk * n], acc);
  acc = warp_sum(acc);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x / 32] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    float2 v = threadIdx.x < 8 ? part[threadIdx.x] : make_float2(0.f, 0.f);
    v = warp_sum(v);
    if (threadIdx.x == 0) C[boff + j] = v;
  }
}

// Skinny products with a long contraction (m * n small, k large): the k range
// is split over `splits` blocks per output; block (r, s) writes the FP32
// partial sum of chunk s of output r, and skinny_finish adds the partials of
// each output in chunk order (FP64), so the result does not depend on
// scheduling.
__global__ void __launch_bounds__(256) skinny_partial(const float2* __restrict__ A,
                                                      const float2* __restrict__ B,
                                                      float2* __restrict__ partial, int n,
                                                      std::uint64_t k, int splits,
                                                      std::uint64_t batch_stride) {
  __shared__ float2 part[8];
  const int r = blockIdx.x / splits, s = blockIdx.x % splits;
  const int i = r / n, j = r % n;
  const std::uint64_t boff = std::uint64_t(blockIdx.y) * batch_stride;
  const std::uint64_t chunk = (k + splits - 1) / splits;
  const std::uint64_t k0 = std::uint64_t(s) * chunk;
  const std::uint64_t k1 = k0 + chunk < k ? k0 + chunk : k;
  const float2* a = A + boff + std::uint64_t(i) * k;
  const float2* b = B + boff + j;
  float2 acc = make_float2(0.f, 0.f);
  for (std::uint64_t kk = k0 + threadIdx.x; kk < k1; kk += blockDim.x) acc = cfma(a[kk], b[kk * n], acc);
  acc = warp_sum(acc);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x / 32] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    float2 v = threadIdx.x < 8 ? part[threadIdx.x] : make_float2(0.f, 0.f);
    v = warp_sum(v);
    if (threadIdx.x == 0) partial[(std::uint64_t(blockIdx.y) * gridDim.x) + blockIdx.x] = v;
  }
}

// C[1][n] = A[1][k] * B[k][n] for 2 <= n <= 256 and long k (the vector
// times matrix products of multiply, src/tensor.cpp:1144-1150): block s sums
// rows [k0, k1) of B for all n columns at once. R = 256 / n rows per pass,
// thread t on column t % n of row t / n, so every pass reads R whole rows
// of B (coalesced) and A once; the R row partials of each column are added
// in row order into partial[(b * n + j) * splits + s], which skinny_finish
// adds up in FP64.
__global__ void __launch_bounds__(256) vm_partial(const float2* __restrict__ A, const float2* __restrict__ B,
                                                  float2* __restrict__ partial, int n, std::uint64_t k, int splits,
                                                  std::uint64_t batch_stride) {
  __shared__ float2 red[256];
  const int s = blockIdx.x;
  const std::uint64_t boff = std::uint64_t(blockIdx.y) * batch_stride;
  const std::uint64_t chunk = (k + splits - 1) / splits;
  const std::uint64_t k0 = std::uint64_t(s) * chunk;
  const std::uint64_t k1 = k0 + chunk < k ? k0 + chunk : k;
  const int R = 256 / n;
  const int t = threadIdx.x, r = t / n, j = t % n;
  float2 acc = make_float2(0.f, 0.f);
  if (r < R) {
    const float2* a = A + boff;
    const float2* b = B + boff + j;
#pragma unroll 4
    for (std::uint64_t kk = k0 + r; kk < k1; kk += R) acc = cfma(a[kk], b[kk * n], acc);
  }
  red[t] = acc;
  __syncthreads();
  if (t < n) {
    float2 v = red[t];
    for (int q = 1; q < R; ++q) {
      v.x += red[q * n + t].x;
      v.y += red[q * n + t].y;
    }
    partial[(std::uint64_t(blockIdx.y) * n + t) * splits + s] = v;
  }
}

// One warp per output: lane l adds partials l, l + 32, ... in FP64, then a
// fixed shuffle tree combines the lanes.
__global__ void skinny_finish(const float2* __restrict__ partial, float2* __restrict__ C, int outputs,
                              int splits, std::uint64_t batch_stride) {
  const int r = (blockIdx.x * blockDim.x + threadIdx.x) / 32;
  const int lane = threadIdx.x & 31;
  if (r >= outputs) return;
  const float2* p = partial + (std::uint64_t(blockIdx.y) * outputs + r) * splits;
  double re = 0, im = 0;
  for (int s = lane; s < splits; s += 32) {
    re += double(p[s].x);
    im += double(p[s].y);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    re += __shfl_xor_sync(0xffffffffu, re, o);
    im += __shfl_xor_sync(0xffffffffu, im, o);
  }
  if (lane == 0) C[std::uint64_t(blockIdx.y) * batch_stride + r] = make_float2(float(re), float(im));
}

__global__ void reduce_amplitudes_kernel(const float2* __restrict__ results, std::uint64_t stride,
                                         const std::uint32_t* __restrict__ ptr,
                                         const std::uint32_t* __restrict__ leaves, int n_amps,
                                         double2* __restrict__ amps) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  const int b = blockIdx.y;
  if (a >= n_amps) return;
  double re = 0, im = 0;
  const float2* r = results + std::uint64_t(b) * stride;
  for (std::uint32_t p = ptr[a]; p < ptr[a + 1]; ++p) {
    const float2 v = r[leaves[p]];
    re += double(v.x);
    im += double(v.y);
  }
  double2& out = amps[std::size_t(b) * n_amps + a];
  out.x += re;
  out.y += im;
}

template <int BM, int BN, int BK, int TM, int TN>
void run_cgemm(const float2* A, const float2* B, float2* C, std::size_t m, std::size_t n,
               std::size_t k, std::uint64_t stride, int batch, cudaStream_t s) {
  const std::size_t tiles = ((m + BM - 1) / BM) * ((n + BN - 1) / BN);
  dim3 grid((unsigned)tiles, 1, (unsigned)batch);
  cgemm_kernel<BM, BN, BK, TM, TN><<<grid, (BM / TM) * (BN / TN), 0, s>>>(A, B, C, (int)m, (int)n,
                                                                         (int)k, stride);
  check_launch("cgemm");
}

}  // namespace

void launch_flatten(const ColumnDesc* cols, int n_cols, std::uint32_t max_size_log2,
                    const StepDesc* steps, const float2* mats, const float2* mats_lo,
                    const std::uint8_t* init_bits, const std::uint8_t* final_bits, float2* arena,
                    std::uint64_t arena_stride, int batch, cudaStream_t s) {
  if (n_cols == 0) return;
  const std::uint64_t blocks = ((std::uint64_t(1) << max_size_log2) + 255) / 256;
  dim3 grid((unsigned)blocks, (unsigned)n_cols, (unsigned)batch);
  if (mats_lo)
    flatten_kernel<true><<<grid, 256, 0, s>>>(cols, steps, mats, mats_lo, init_bits, final_bits, n_cols,
                                              arena, arena_stride);
  else
    flatten_kernel<false><<<grid, 256, 0, s>>>(cols, steps, mats, mats, init_bits, final_bits, n_cols,
                                               arena, arena_stride);
  check_launch("flatten");
}

void make_perm_plan(int R, const std::uint8_t* perm, PermPlan* P) {
  if (R > 31) throw std::string("ERROR (qflex_gb300: permute) --> tensor exceeds 2^31 elements");
  std::memset(P, 0, sizeof(*P));
  bool in_tile[40] = {};
  const int want = std::min(10, R);
  int a = std::min(5, R), c = std::min(5, R), count = 0;
  auto recount = [&]() {
    count = 0;
    for (int p = 0; p < R; ++p) {
      in_tile[p] = (p < a) || (perm[p] < c);
      count += in_tile[p];
    }
  };
  recount();
  bool grow_in = true;
  while (count < want) {
    if ((grow_in && a < R) || c >= R)
      ++a;
    else
      ++c;
    grow_in = !grow_in;
    recount();
  }
  int t_in[40], t_out[40], rank_in[40] = {};
  int nt = 0;
  for (int p = 0; p < R; ++p)
    if (in_tile[p]) {
      rank_in[p] = nt;
      t_in[nt++] = p;
    }
  int no = 0;
  for (int q = 0; q < R; ++q)  // tile digits ordered by output position
    for (int p = 0; p < R; ++p)
      if (in_tile[p] && perm[p] == q) t_out[no++] = p;
  P->tile_bits = (std::uint32_t)nt;
  int n_outer = 0;
  std::uint8_t outer_in[40], outer_out[40];
  for (int p = 0; p < R; ++p)
    if (!in_tile[p]) {
      outer_in[n_outer] = (std::uint8_t)p;
      outer_out[n_outer] = perm[p];
      ++n_outer;
    }
  if (n_outer > 25) throw std::string("ERROR (qflex_gb300: permute) --> too many digits outside the tile");
  P->n_outer = (std::uint32_t)n_outer;
  P->n_tiles = std::uint64_t(1) << n_outer;
  for (int g = 0; g < 5; ++g)
    for (std::uint32_t x = 0; x < 32; ++x)
      for (int b = 0; b < 5; ++b) {
        const int q = 5 * g + b;
        if (q < n_outer && ((x >> b) & 1)) {
          P->otab[0][g][x] |= 1u << outer_in[q];
          P->otab[1][g][x] |= 1u << outer_out[q];
        }
      }
  for (std::uint32_t j = 0; j < 32; ++j) {
    for (int q = 0; q < 5; ++q) {
      if (!((j >> q) & 1)) continue;
      if (q < nt) {
        P->tab[0][j] |= 1u << t_in[q];
        P->tab[2][j] |= 1u << perm[t_out[q]];
        P->tab[4][j] |= 1u << rank_in[t_out[q]];
      }
      if (q + 5 < nt) {
        P->tab[1][j] |= 1u << t_in[q + 5];
        P->tab[3][j] |= 1u << perm[t_out[q + 5]];
        P->tab[5][j] |= 1u << rank_in[t_out[q + 5]];
      }
    }
  }
}

void permute_schedule_on_host(const PermPlan& P, const float2* src, float2* dst,
                              std::uint64_t size) {
  std::vector<float2> tile(1024);
  const std::uint32_t T = 1u << P.tile_bits;
  for (std::uint64_t t = 0; t < P.n_tiles; ++t) {
    std::uint64_t bi, bo;
    perm_tile_base(P, t, &bi, &bo);
    for (std::uint32_t j = 0; j < T; ++j) {
      const std::uint32_t slot = perm_swizzle(j);
      if (slot >= 1024) throw std::string("ERROR (qflex_gb300: permute) --> tile slot out of range");
      const std::uint64_t at = bi + P.tab[0][j & 31] + P.tab[1][j >> 5];
      if (at >= size) throw std::string("ERROR (qflex_gb300: permute) --> load out of range");
      tile[slot] = src[at];
    }
    for (std::uint32_t j = 0; j < T; ++j) {
      const std::uint32_t slot = perm_swizzle(P.tab[4][j & 31] + P.tab[5][j >> 5]);
      if (slot >= T) throw std::string("ERROR (qflex_gb300: permute) --> tile slot out of range");
      const std::uint64_t at = bo + P.tab[2][j & 31] + P.tab[3][j >> 5];
      if (at >= size) throw std::string("ERROR (qflex_gb300: permute) --> store out of range");
      dst[at] = tile[slot];
    }
  }
}

void launch_permute(const PermPlan& plan, const float2* src, float2* dst, std::uint64_t batch_stride,
                    int batch, cudaStream_t s) {
  const std::uint64_t tiles = plan.n_tiles;
  const unsigned gx = (unsigned)std::min<std::uint64_t>(tiles, 152ull * 16ull);
  dim3 grid(gx, (unsigned)batch, 1);
  permute_kernel<float2, false><<<grid, 256, 0, s>>>(plan, src, dst, batch_stride, PlaneOut{});
  check_launch("permute");
}

void make_general_perm(std::size_t rank, const std::size_t* dims, const std::size_t* new_order, GeneralPerm* g) {
  if (rank > (std::size_t)kGeneralPermMaxRank)
    throw std::string("ERROR (qflex_gb300: permute) --> at most 32 indices when a dimension is not a power of two");
  std::memset(g, 0, sizeof(*g));
  g->rank = (std::uint32_t)rank;
  std::uint64_t stride[kGeneralPermMaxRank];
  std::uint64_t size = 1;
  for (std::size_t i = rank; i-- > 0;) {
    if (dims[i] == 0) throw std::string("ERROR (qflex_gb300: permute) --> dimensions must be positive");
    stride[i] = size;
    if (dims[i] > (std::uint64_t(1) << 40) / size)
      throw std::string("ERROR (qflex_gb300: permute) --> tensor exceeds 2^40 elements");
    size *= dims[i];
  }
  bool seen[kGeneralPermMaxRank] = {};
  for (std::size_t i = 0; i < rank; ++i) {
    const std::size_t q = new_order[i];
    if (q >= rank || seen[q]) throw std::string("ERROR (qflex_gb300: permute) --> new_order is not a permutation");
    seen[q] = true;
    g->out_dims[i] = dims[q];
    g->in_stride[i] = stride[q];
  }
  g->size = size;
}

void permute_general_on_host(const GeneralPerm& g, const float2* src, float2* dst) {
  for (std::uint64_t o = 0; o < g.size; ++o) {
    const std::uint64_t at = general_source(g, o);
    if (at >= g.size) throw std::string("ERROR (qflex_gb300: permute) --> load out of range");
    dst[o] = src[at];
  }
}

void launch_permute_general(const GeneralPerm& g, const float2* src, float2* dst, std::uint64_t batch_stride,
                            int batch, cudaStream_t s) {
  if (g.size == 0 || batch == 0) return;
  const std::uint64_t blocks = std::min<std::uint64_t>((g.size + 255) / 256, 152ull * 64ull);
  dim3 grid((unsigned)blocks, (unsigned)batch, 1);
  permute_general_kernel<<<grid, 256, 0, s>>>(g, src, dst, batch_stride);
  check_launch("permute_general");
}

void launch_permute64(const PermPlan& plan, const double2* src, double2* dst, std::uint64_t batch_stride,
                      int batch, cudaStream_t s) {
  const std::uint64_t tiles = plan.n_tiles;
  const unsigned gx = (unsigned)std::min<std::uint64_t>(tiles, 152ull * 8ull);
  dim3 grid(gx, (unsigned)batch, 1);
  permute_kernel<double2, false><<<grid, 256, 0, s>>>(plan, src, dst, batch_stride, PlaneOut{});
  check_launch("permute64");
}

void launch_permute_fp16_planes(const PermPlan& plan, const float2* src, std::uint64_t src_batch_stride,
                                void* planes, int* exps, std::uint64_t rows, int k_log2, int batch,
                                cudaStream_t s) {
  if (k_log2 < 5 || plan.tile_bits < 5)
    throw std::string("ERROR (qflex_gb300: permute) --> plane output needs rows of at least 32 values");
  const std::uint64_t tiles = plan.n_tiles;
  const unsigned gx = (unsigned)std::min<std::uint64_t>(tiles, 152ull * 16ull);
  dim3 grid(gx, (unsigned)batch, 1);
  permute_kernel<float2, true><<<grid, 256, 0, s>>>(plan, src, nullptr, src_batch_stride,
                                            PlaneOut{static_cast<__half*>(planes), exps, rows, (std::uint32_t)k_log2});
  check_launch("permute_fp16_planes");
}

int vm_splits(std::size_t m, std::size_t n, std::size_t k, int batch) {
  if (m != 1 || n < 2 || n > 256 || k < 4096) return 0;
  std::size_t splits = std::min<std::size_t>(4096, k / 2048);
  while (splits > 1 && splits * n * (std::size_t)batch > kSkinnyScratchElems) splits /= 2;
  return splits >= 2 ? (int)splits : 0;
}

int skinny_splits(std::size_t m, std::size_t n, std::size_t k, int batch) {
  if (m * n > 64 || k < 8192) return 0;
  std::size_t splits = std::min<std::size_t>(2048, (k + 4095) / 4096);
  while (splits > 1 && splits * m * n * (std::size_t)batch > kSkinnyScratchElems) splits /= 2;
  return splits >= 2 ? (int)splits : 0;
}

void launch_skinny_split(const float2* A, const float2* B, float2* C, std::size_t m, std::size_t n,
                        std::size_t k, int splits, float2* partial, cudaStream_t s) {
  const int outputs = (int)(m * n);
  dim3 g1((unsigned)(outputs * splits), 1u);
  skinny_partial<<<g1, 256, 0, s>>>(A, B, partial, (int)n, k, splits, 0);
  check_launch("skinny_partial");
  dim3 g2((unsigned)((outputs * 32 + 127) / 128), 1u);
  skinny_finish<<<g2, 128, 0, s>>>(partial, C, outputs, splits, 0);
  check_launch("skinny_finish");
}

void launch_cgemm_fp32(const float2* A, const float2* B, float2* C, std::size_t m, std::size_t n,
                       std::size_t k, std::uint64_t stride, int batch, cudaStream_t s,
                       float2* scratch) {
  if (const int splits = scratch ? vm_splits(m, n, k, batch) : 0) {
    dim3 g1((unsigned)splits, (unsigned)batch);
    vm_partial<<<g1, 256, 0, s>>>(A, B, scratch, (int)n, k, splits, stride);
    check_launch("vm_partial");
    dim3 g2((unsigned)((n * 32 + 127) / 128), (unsigned)batch);
    skinny_finish<<<g2, 128, 0, s>>>(scratch, C, (int)n, splits, stride);
    check_launch("skinny_finish");
    return;
  }
  if (const int splits = scratch ? skinny_splits(m, n, k, batch) : 0) {
    const int outputs = (int)(m * n);
    dim3 g1((unsigned)(outputs * splits), (unsigned)batch);
    skinny_partial<<<g1, 256, 0, s>>>(A, B, scratch, (int)n, k, splits, stride);
    check_launch("skinny_partial");
    dim3 g2((unsigned)((outputs * 32 + 127) / 128), (unsigned)batch);
    skinny_finish<<<g2, 128, 0, s>>>(scratch, C, outputs, splits, stride);
    check_launch("skinny_finish");
    return;
  }
  if (n == 1) {
    if (k <= 32) {
      dim3 grid((unsigned)((m + 255) / 256), (unsigned)batch);
      gemv_rows_thread<<<grid, 256, 0, s>>>(A, B, C, m, (int)k, stride);
    } else {
      dim3 grid((unsigned)((m * 32 + 255) / 256), (unsigned)batch);
      gemv_rows_warp<<<grid, 256, 0, s>>>(A, B, C, m, k, stride);
    }
    check_launch("gemv_rows");
    return;
  }
  if (m == 1) {
    if (n >= 256) {
      dim3 grid((unsigned)((n + 255) / 256), (unsigned)batch);
      gemv_cols_thread<<<grid, 256, 0, s>>>(A, B, C, n, k, stride);
    } else {
      dim3 grid((unsigned)n, (unsigned)batch);
      gemv_cols_block<<<grid, 256, 0, s>>>(A, B, C, n, k, stride);
    }
    check_launch("gemv_cols");
    return;
  }
  if (m > 0x7fffffffull || n > 0x7fffffffull || k > 0x7fffffffull)
    throw std::string("ERROR (qflex_gb300: cgemm) --> dimension exceeds 2^31");
  if (n <= 32)
    run_cgemm<256, 16, 16, 8, 2>(A, B, C, m, n, k, stride, batch, s);
  else if (m <= 32)
    run_cgemm<16, 256, 16, 2, 8>(A, B, C, m, n, k, stride, batch, s);
  else
    run_cgemm<128, 64, 16, 8, 4>(A, B, C, m, n, k, stride, batch, s);
}

void launch_reduce_amplitudes(const float2* results, std::uint64_t stride, const std::uint32_t* ptr,
                              const std::uint32_t* leaves, int n_amps, double2* amps, int batch,
                              cudaStream_t s) {
  if (n_amps == 0) return;
  dim3 grid((unsigned)((n_amps + 127) / 128), (unsigned)batch);
  reduce_amplitudes_kernel<<<grid, 128, 0, s>>>(results, stride, ptr, leaves, n_amps, amps);
  check_launch("reduce_amplitudes");
}

}  // namespace qfx
