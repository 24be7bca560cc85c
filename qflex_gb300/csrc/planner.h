// Static device program for one contraction.
//
// The reference runs the EXPAND/CUT/MERGE ordering as a recursion that
// re-executes everything after a cut once per cut value, reordering tensors
// in place (src/contraction_utils.cpp:223-354). The planner performs that
// recursion once, on index metadata only, and records every data movement
// and product as a device op on arena buffers. The recorded program is then
// replayed on the GPU for any number of bitstrings at once.
#pragma once

#include <cstdint>
#include <functional>
#include <string>
#include <vector>

#include "qfx.h"

namespace qfx {

// One device op. Offsets are complex64 element offsets into one arena
// replica; the executor adds replica * arena_elems for batch entry `replica`.
struct DevOp {
  enum Kind : int { PERMUTE = 0, GEMM = 1 } kind;
  std::size_t a = 0, b = 0, c = 0;  // PERMUTE: a = source, c = destination
  std::size_t m = 1, n = 1, k = 1;  // GEMM: C[m,n] = A[m,k] * B[k,n]
  int nbits = 0;                    // PERMUTE: log2(size)
  std::uint8_t perm[40] = {};       // PERMUTE: output bit of each input bit
  int shape_id = -1;                // GEMM: index into Program::shapes
  bool b_nk = false;                // GEMM: B stored as [n][k] (K-major)
};

struct GemmShape {
  std::size_t m, n, k;
  std::size_t count;
};

// What one contraction computes and how it is laid out in HBM.
struct Program {
  std::vector<DevOp> ops;
  std::vector<GemmShape> shapes;       // distinct GEMM shapes and counts
  // Column (2D grid tensor) placement: element offset of each column's
  // tensor, in Network::columns order.
  std::vector<std::size_t> column_offset;
  std::size_t results_offset = 0;      // one complex64 per leaf
  std::size_t n_leaves = 0;
  std::vector<std::uint32_t> leaf_amp; // leaf -> amplitude index
  std::size_t n_amplitudes = 0;
  std::size_t arena_elems = 0;         // elements in one replica
  double reference_bytes = 0;          // the reference's planned allocation
  double gemm_flop = 0;                // 8*m*n*k summed over GEMMs
  double permute_bytes = 0;            // 16*size summed over permutes
};

// Plans the contraction of `net` by `ops` (the ordering IR). Throws the
// reference's errors (std::string) for orderings the reference rejects at
// contraction time, and the memory-limit error before anything is
// allocated.
// `b_kmajor(m, n, k)` tells whether the product of that shape runs on a
// kernel that reads B as [n][k] rows (the tensor-core path); by default
// every product reads the reference's [k][n] layout.
// With `open_terminals`, terminal cuts that take all their values (and are
// not followed by a two-qubit cut) stay open indices: the ops after them
// run once and the final tensor holds the terminal region's amplitudes.
Program plan_contraction(const Network& net, const std::vector<Op>& ops,
                         std::size_t n_amplitudes, double memory_limit,
                         std::function<bool(std::size_t, std::size_t, std::size_t)> b_kmajor = {},
                         bool open_terminals = false);

}  // namespace qfx
