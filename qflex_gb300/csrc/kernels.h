// Device kernels of the contraction path and their launch helpers.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace qfx {

// ---- 3D -> 2D flatten -------------------------------------------------------
// One column = one active qubit's time column. Its 2D tensor element e is
// <final| G_K(v_K(e)) ... G_1(v_1(e)) |init>, where every two-qubit half
// reads its virtual digit v_t(e) = (e >> shift) & (V - 1) of its bond.
struct ColumnDesc {
  std::uint64_t out_offset;  // element offset of the 2D tensor in the arena
  std::uint32_t size_log2;   // log2 of the 2D tensor's element count
  std::uint32_t step_begin, step_end;
  std::int32_t o_shift;      // bit of the (o) index, -1 when not terminal
};

struct StepDesc {
  std::uint32_t kind;     // 1: 2x2 matrix; 2: two-qubit half (in, v, out)
  std::uint32_t V;        // virtual dimension of a two-qubit half
  std::uint32_t shift;    // bit position of the virtual digit
  std::uint32_t mat;      // offset of the gate data in the matrix pool
};

// `mats` holds the gate data as complex64; with `mats_lo` (the remainders
// of the double-precision gates) the chains run in float-float arithmetic,
// otherwise in plain FP32 like the reference.
void launch_flatten(const ColumnDesc* cols, int n_cols, std::uint32_t max_size_log2,
                    const StepDesc* steps, const float2* mats, const float2* mats_lo,
                    const std::uint8_t* init_bits, const std::uint8_t* final_bits, float2* arena,
                    std::uint64_t arena_stride, int batch, cudaStream_t s);

// ---- index permutation over binary digits --------------------------------------
// The tensor is viewed as nbits binary digits; input digit p moves to output
// digit perm[p]. A tile covers up to 10 digits: the low input digits (read
// coalesced) and the digits that become the low output digits (written
// coalesced); the remaining digits index the tiles.
struct PermPlan {
  std::uint32_t tile_bits;
  std::uint32_t n_outer;                 // number of digits outside the tile (<= 25)
  std::uint64_t n_tiles;                 // 2^n_outer
  // Lookup tables split by the low / high five bits of a tile index j:
  // [0],[1] input offset of tile element j (input order); [2],[3] output
  // offset of output-order element j; [4],[5] its tile slot.
  std::uint32_t tab[6][32];
  // Tile base offsets by five-bit groups g of the tile number t:
  // otab[0][g][x] / otab[1][g][x] = input / output offset contributed by
  // bits 5g .. 5g+4 of t having the value x.
  std::uint32_t otab[2][5][32];
};

void make_perm_plan(int nbits, const std::uint8_t* perm, PermPlan* plan);

// Index schedule of the permutation kernel, shared by the device kernel and
// the host-side schedule check.
__host__ __device__ inline std::uint32_t perm_swizzle(std::uint32_t j) { return j ^ ((j >> 5) & 31u); }
__host__ __device__ inline void perm_tile_base(const PermPlan& P, std::uint64_t t, std::uint64_t* bi,
                                               std::uint64_t* bo) {
  std::uint32_t i = 0, o = 0;
#pragma unroll
  for (int g = 0; g < 5; ++g) {
    const std::uint32_t x = std::uint32_t(t >> (5 * g)) & 31u;
    i += P.otab[0][g][x];
    o += P.otab[1][g][x];
  }
  *bi = i;
  *bo = o;
}

// Runs the kernel's schedule on host buffers (tile by tile, load phase then
// store phase, through a 1024-slot swizzled tile). Tests use it to check the
// plan and the index math without a GPU.
void permute_schedule_on_host(const PermPlan& plan, const float2* src, float2* dst,
                              std::uint64_t size);
void launch_permute(const PermPlan& plan, const float2* src, float2* dst, std::uint64_t batch_stride,
                    int batch, cudaStream_t s);
// The same permutation writing its output, a row-major [rows][k] operand
// (k a power of two >= 32), as the 3xFP16 tensor-core planes instead of
// complex64: [k / 16][rows][plane 4][16] fp16 per batch entry (the layout
// the product kernel loads), every 32 consecutive values of a row scaled by
// their own power of two 2^e (max in [2^14, 2^15)), e stored at
// exps[row * (k / 32) + kk / 32]. Planes of batch entry b start at
// planes + b * 4 * rows * k, exponents at exps + b * rows * (k / 32).
void launch_permute_fp16_planes(const PermPlan& plan, const float2* src, std::uint64_t src_batch_stride,
                                void* planes, int* exps, std::uint64_t rows, int k_log2, int batch,
                                cudaStream_t s);

// ---- permutation of indices of any dimension -------------------------------------
// Output element o (row-major over the permuted dimensions) reads input
// element sum_i digit_i(o) * in_stride[i], where in_stride[i] is the input
// stride of the index that goes to position i. One thread per output
// element: writes coalesced, reads gathered. For tensors whose dimensions
// are not all powers of two.
constexpr int kGeneralPermMaxRank = 32;
struct GeneralPerm {
  std::uint32_t rank;
  std::uint64_t size;
  std::uint64_t out_dims[kGeneralPermMaxRank];
  std::uint64_t in_stride[kGeneralPermMaxRank];
};
// Throws (std::string) for a rank above kGeneralPermMaxRank, a zero
// dimension, an element count above 2^40 or a new_order that is not a
// permutation.
void make_general_perm(std::size_t rank, const std::size_t* dims, const std::size_t* new_order, GeneralPerm* g);
void permute_general_on_host(const GeneralPerm& g, const float2* src, float2* dst);
void launch_permute_general(const GeneralPerm& g, const float2* src, float2* dst, std::uint64_t batch_stride,
                            int batch, cudaStream_t s);

// ---- complex64 products on CUDA cores -------------------------------------------
// C[m,n] = A[m,k] * B[k,n], row-major, all three advanced by batch_stride
// elements per batch entry. Products with m * n <= 64 and k >= 8192 split k
// over many blocks; their partial sums go to `scratch` (kSkinnyScratchElems
// float2, or nullptr to keep the one-block-per-output kernels).
constexpr std::size_t kSkinnyScratchElems = std::size_t(1) << 20;
int skinny_splits(std::size_t m, std::size_t n, std::size_t k, int batch);
// Vector-times-matrix products (m = 1, 2 <= n <= 256, long k) split k over
// blocks that each read whole rows of B; 0 when the shape does not qualify.
// Takes precedence over skinny_splits.
int vm_splits(std::size_t m, std::size_t n, std::size_t k, int batch);
void launch_cgemm_fp32(const float2* A, const float2* B, float2* C, std::size_t m, std::size_t n,
                       std::size_t k, std::uint64_t batch_stride, int batch, cudaStream_t s,
                       float2* scratch);

// One skinny product (m * n outputs) with k split over `splits` blocks per
// output; `partial` holds m * n * splits float2, every one of which is
// written before it is read.
void launch_skinny_split(const float2* A, const float2* B, float2* C, std::size_t m, std::size_t n,
                        std::size_t k, int splits, float2* partial, cudaStream_t s);

// ---- complex128 path (the FP64 GPU oracle, kernels64.cu) ----------------------
// Same layouts and index schedules as the complex64 kernels, with double2
// elements. Gate data are the double-precision gate constants.
void launch_flatten64(const ColumnDesc* cols, int n_cols, std::uint32_t max_size_log2, const StepDesc* steps,
                      const double2* mats, const std::uint8_t* init_bits, const std::uint8_t* final_bits,
                      double2* arena, std::uint64_t arena_stride, int batch, cudaStream_t s);
void launch_permute64(const PermPlan& plan, const double2* src, double2* dst, std::uint64_t batch_stride,
                      int batch, cudaStream_t s);
// Split-k partial sums of the complex128 skinny products share the skinny
// scratch buffer (kSkinnyScratchElems float2 = this many double2).
constexpr std::size_t kSkinnyScratchElems64 = kSkinnyScratchElems / 2;
int zskinny_splits(std::size_t m, std::size_t n, std::size_t k, int batch);
// C[m,n] = A[m,k] * B[k,n] in complex128. `ff` selects float-float
// arithmetic for the tiled products (FP64 FMA otherwise); skinny products
// and GEMVs always use FP64 FMA.
void launch_zgemm(const double2* A, const double2* B, double2* C, std::size_t m, std::size_t n, std::size_t k,
                  std::uint64_t batch_stride, int batch, cudaStream_t s, double2* scratch, bool ff);
void launch_reduce_amplitudes64(const double2* results, std::uint64_t stride, const std::uint32_t* ptr,
                                const std::uint32_t* leaves, int n_amps, double2* amps, int batch,
                                cudaStream_t s);

// ---- FP64 amplitude sums -------------------------------------------------------
// amps[b * n_amps + a] += sum of results[b * stride + leaf] over the leaves
// of amplitude a (CSR: leaves[ptr[a] .. ptr[a+1])), in leaf order.
void launch_reduce_amplitudes(const float2* results, std::uint64_t stride, const std::uint32_t* ptr,
                              const std::uint32_t* leaves, int n_amps, double2* amps, int batch,
                              cudaStream_t s);

}  // namespace qfx
