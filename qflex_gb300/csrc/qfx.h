// Shared host-side declarations of the qflex_gb300 engine.
//
// The engine reproduces the qFlex grid tensor-network contraction
// (circuit + grid + ordering -> amplitudes). Host C++ parses the inputs,
// builds the network description and unrolls the EXPAND/CUT/MERGE recursion
// into a static device program; hand-written sm_103a kernels execute it.
#pragma once

#include <complex>
#include <cstddef>
#include <cstdint>
#include <map>
#include <sstream>
#include <string>
#include <utility>
#include <vector>

namespace qfx {

// Errors are thrown as std::string, like the reference (src/errors.h:7-9),
// so message substrings the reference's tests match on are preserved.
template <typename... T>
std::string cat(const T&... xs) {
  std::ostringstream ss;
  (ss << ... << xs);
  return ss.str();
}
#define QFX_ERR(...) ::qfx::cat("ERROR (qflex_gb300: ", __func__, ") --> ", __VA_ARGS__)
#define QFX_WRAP(fn, inner) \
  ::qfx::cat("ERROR (qflex_gb300: ", __func__, ") --> Failed to call " fn "(). Error:\n\t[", inner, "]")

using Coord = std::pair<int, int>;

// ---- input formats (src/circuit.h, src/grid.h, src/ordering.h) ----
struct Gate {
  std::string name;
  long cycle = 0;
  std::vector<long> qubits;
  std::vector<double> params;
  std::string raw;
};

struct Circuit {
  long num_active_qubits = 0;
  long depth = 0;
  std::vector<Gate> gates;
  void load(const std::string& text);
};

struct Grid {
  long I = 0, J = 0;
  std::vector<Coord> qubits_off;
  void load(const std::string& text);
  bool is_off(int i, int j) const;
};

struct Ordering {
  std::vector<std::string> instructions;
  void load(const std::string& text);
};

std::size_t parse_memory_string(std::string s);
std::string readable_memory_string(double bytes);

// ---- contraction ordering IR (src/contraction_utils.h:54-99) ----
struct Op {
  enum Kind { EXPAND, CUT, MERGE } kind;
  std::string patch;            // EXPAND
  Coord tensor{0, 0};           // EXPAND
  std::vector<Coord> tensors;   // CUT: 1 (terminal) or 2 positions
  std::vector<std::size_t> values;  // CUT: empty = all values
  std::string source, target;   // MERGE
};

std::string index_name(const Coord& a, const Coord& b);
std::string terminal_name(const Coord& a);
std::string cut_index_name(const Op& cut);
std::vector<Op> parse_ordering(const Ordering& ord, const Grid& grid);
void validate_ordering(const std::vector<Op>& ops);

// ---- network description ----
// One step of a qubit's time column: a single-qubit 2x2 matrix (in, out) or
// one half of a two-qubit gate (in, virtual[V], out), stored as complex64.
struct ColumnStep {
  int kind;          // 1 = single-qubit, 2 = two-qubit half
  int V;             // virtual dimension (2 for cz/cx, 4 for fsim)
  int link;          // index into Network::links for two-qubit halves
  int ordinal;       // 0-based position of this gate among the link's gates
  std::vector<std::complex<float>> data;  // 4 or 4*V entries, as the reference stores them
  std::vector<std::complex<double>> exact;  // the same gate evaluated in double
};

struct Link {
  Coord a, b;        // a < b in the reference's index_name order
  std::string name;  // "(i,j),(k,l)"
  int n_gates = 0;
  std::vector<int> V;  // per gate, in time order
  std::size_t dim() const {
    std::size_t d = 1;
    for (int v : V) d *= v;
    return d;
  }
};

struct QubitColumn {
  Coord pos;
  int init_bit = 0;
  int final_bit = 0;
  bool terminal = false;     // in the final region: last index is (o)
  std::vector<ColumnStep> steps;
  // Indices of the flattened 2D tensor in their final order, and dims.
  std::vector<std::string> indices;
  std::vector<std::size_t> dims;
};

struct Network {
  long I = 0, J = 0;
  std::vector<QubitColumn> columns;          // active qubits, row-major
  std::map<Coord, int> column_of;            // grid position -> column
  std::vector<Link> links;
  std::map<std::string, int> link_of;        // link name -> link
};

Network build_network(const Circuit& circuit, const Grid& grid,
                      const std::string& initial, const std::string& final_conf,
                      const std::vector<Coord>& final_region,
                      const std::vector<Op>& ops);

// Amplitude bookkeeping (src/evaluate_circuit.cpp:22-104).
std::size_t find_output_pos(const Grid& grid, const Coord& pos);
std::string get_output_states(const Grid& grid, const std::vector<Op>& ops,
                              const std::string& initial,
                              const std::string& final_state,
                              std::vector<Coord>* final_qubits,
                              std::vector<std::string>* output_states);

}  // namespace qfx
