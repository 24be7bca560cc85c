// Ordering IR, validation, gate tables and the description of the flattened
// 2D grid of tensors.
//
// The reference builds a 3D grid of gate tensors, contracts every qubit's
// time column with small GEMMs, bundles parallel bonds and permutes each 2D
// tensor into contraction order (src/read_circuit.cpp:296-689). This engine
// keeps only a *description* of each column (its gate matrices and which
// bond digit each two-qubit half reads) and lets one GPU kernel evaluate
// every element of every 2D tensor directly in its final layout.
#include <algorithm>
#include <cmath>
#include <functional>
#include <optional>
#include <set>
#include <unordered_map>
#include <unordered_set>

#include "qfx.h"

namespace qfx {

std::string index_name(const Coord& a, const Coord& b) {
  return cat("(", a.first, ",", a.second, "),(", b.first, ",", b.second, ")");
}

std::string terminal_name(const Coord& a) {
  return cat("(", a.first, ",", a.second, "),(o)");
}

std::string cut_index_name(const Op& cut) {
  if (cut.tensors.size() == 2) return index_name(cut.tensors[0], cut.tensors[1]);
  if (cut.tensors.size() == 1) return terminal_name(cut.tensors[0]);
  throw QFX_ERR("Failed to construct tensor name with input tensors size: ",
                cut.tensors.size(), ".");
}

// ordering_data_to_contraction_ordering (src/contraction_utils.cpp:358-475).
std::vector<Op> parse_ordering(const Ordering& ord, const Grid& grid) {
  std::vector<Op> ops;
  const long grid_size = grid.I * grid.J;
  for (const auto& line : ord.instructions) {
    if (line.empty() || line[0] == '#') continue;
    auto error = [&](const std::string& msg) {
      // The reference's message names an outer, never-assigned `line`
      // (src/contraction_utils.cpp:365-370), so the quoted line is always
      // empty; the text is kept identical.
      return QFX_ERR("Parsing failed on line: '' with error: ", msg);
    };
    auto check = [&](long idx) {
      if (idx < 0 || idx >= grid_size)
        throw error(cat("Index ", idx, " must be within grid boundaries."));
    };
    auto coords = [&](long q) { return Coord{int(q / grid.J), int(q % grid.J)}; };
    std::istringstream ss(line);
    std::string op;
    ss >> op;
    if (op == "expand") {
      Op e{Op::EXPAND};
      long idx = 0;
      ss >> e.patch >> std::ws;
      // A line that ends before the index leaves the reference's index
      // uninitialized (its extraction fails at end of stream and stores
      // nothing, src/contraction_utils.cpp:390-396): refused here. A token
      // that is not a number reads as 0 there (a failed conversion stores
      // 0) and reads as 0 here.
      if (ss.eof()) throw error("Expand needs a patch name and a qubit index.");
      ss >> idx;
      check(idx);
      e.tensor = coords(idx);
      if (grid.is_off(e.tensor.first, e.tensor.second))
        throw error("Index must specify an active qubit.");
      ops.push_back(e);
    } else if (op == "cut") {
      Op c{Op::CUT};
      std::string vs;
      ss >> vs;
      bool ok = vs.size() >= 2 && vs.front() == '(' && vs.back() == ')';
      for (std::size_t i = 1; ok && i + 1 < vs.size(); ++i)
        ok = std::isdigit((unsigned char)vs[i]) || vs[i] == ',';
      if (!ok) throw error("Cut values must be comma-separated ints, e.g. (0,1,3).");
      std::string inner = vs.substr(1, vs.size() - 2);
      if (!inner.empty()) {
        std::size_t start = 0;
        while (true) {
          std::size_t end = inner.find(',', start);
          c.values.push_back((std::size_t)std::atoi(
              inner.substr(start, end == std::string::npos ? std::string::npos : end - start)
                  .c_str()));
          if (end == std::string::npos) break;
          start = end + 1;
        }
      }
      long i1 = 0, i2 = 0;
      ss >> i1;
      check(i1);
      Coord p1 = coords(i1);
      if (grid.is_off(p1.first, p1.second)) throw error("Index 1 must specify an active qubit.");
      if (ss.eof()) {
        c.tensors = {p1};
      } else {
        ss >> i2;
        check(i2);
        Coord p2 = coords(i2);
        if (grid.is_off(p2.first, p2.second))
          throw error("Index 2 must specify an active qubit.");
        c.tensors = (i1 < i2) ? std::vector<Coord>{p1, p2} : std::vector<Coord>{p2, p1};
      }
      ops.push_back(c);
    } else if (op == "merge") {
      Op m{Op::MERGE};
      ss >> m.source >> m.target;
      ops.push_back(m);
    } else {
      throw error("Received an invalid operation in config.");
    }
  }
  validate_ordering(ops);
  return ops;
}

// ValidateOrdering (src/contraction_utils.cpp:534-610).
void validate_ordering(const std::vector<Op>& ops) {
  struct State {
    bool active = false, used = false, merged = false;
  };
  std::unordered_map<std::string, State> patches;
  std::unordered_set<std::string> cut_indices, used_tensors;
  std::string msg;
  for (const auto& op : ops) {
    if (op.kind == Op::EXPAND) {
      const auto& t = op.tensor;
      for (bool flag : {patches[op.patch].used, patches[op.patch].merged})
        if (flag)
          msg = cat(msg, "\nTensor at (", t.first, ",", t.second, ") is added to non-empty patch ",
                    op.patch, " after a cut.");
      std::string name = cat("(", t.first, ",", t.second, ")");
      if (used_tensors.count(name)) msg = cat(msg, "\nTensor ", name, " is contracted multiple times.");
      used_tensors.insert(name);
      patches[op.patch].active = true;
    } else if (op.kind == Op::CUT) {
      for (auto& [name, st] : patches)
        if (st.active) st.used = true;
      std::string index = cut_index_name(op);
      if (cut_indices.count(index)) msg = cat(msg, "\nIndex ", index, " is cut multiple times.");
      cut_indices.insert(index);
    } else {
      if (patches[op.source].merged)
        msg = cat(msg, "\nPatch ", op.source, " is merged multiple times.");
      if (patches[op.target].used)
        msg = cat(msg, "\nPatch ", op.source, " is merged into non-empty patch ", op.target,
                  " after a cut.");
      patches[op.source].merged = true;
      patches[op.target].active = true;
    }
  }
  if (!msg.empty()) throw msg;
}

namespace {

using cfloat = std::complex<float>;

// Gate constants of src/read_circuit.cpp:27-79. One-qubit gates are
// (input, output); two-qubit halves are (input, virtual, output). With
// T = float the values are exactly the reference's complex64 constants; with
// T = double they are the same constants in double (the split-precision path
// evaluates the time columns with these).
template <typename T>
std::vector<std::complex<T>> table_gate(const std::string& name) {
  using C = std::complex<T>;
  const T r = static_cast<T>(M_SQRT1_2), h = T(0.5);
  auto v = [](double x) { return C(static_cast<T>(x), T(0)); };
  if (name == "h") return {C(r), C(r), C(r), C(-r)};
  if (name == "hz_1_2") return {C(h, h), C(r, 0), C(0, -r), C(h, h)};
  if (name == "t") return {C(1), C(0), C(0), C(r, r)};
  if (name == "x_1_2") return {C(h, h), C(h, -h), C(h, -h), C(h, h)};
  if (name == "y_1_2") return {C(h, h), C(h, h), C(-h, -h), C(h, h)};
  if (name == "cz_q1")
    return {v(-0.3446133714352872), v(0), v(1.1381806476131544), v(0), v(0), v(-1.1381806476131544), v(0),
            v(-0.3446133714352872)};
  if (name == "cz_q2")
    return {v(-1.0484937059720079), v(0), v(0.5611368023131075), v(0), v(0), v(0.5611368023131075), v(0),
            v(1.0484937059720079)};
  if (name == "cx_q1")
    return {v(0.8408964152537143), v(0), v(0.8408964152537143), v(0), v(0), v(-0.8408964152537143), v(0),
            v(0.8408964152537143)};
  if (name == "cx_q2") {
    const T a = static_cast<T>(0.5946035575013604);
    return {C(a), C(-a), C(a), C(a), C(-a), C(a), C(a), C(a)};
  }
  return {};
}

template <typename T>
std::vector<std::complex<T>> one_qubit_gate(const Gate& g) {
  using C = std::complex<T>;
  if (g.name == "rz") {
    // rz(x) = diag(conj(p), p), p = exp(i * pi * x / 2); the reference
    // evaluates it in float (src/read_circuit.cpp:84-88).
    const double angle = M_PI * g.params.at(0);
    const C phase = std::exp(C(T(0), static_cast<T>(angle / 2)));
    return {std::conj(phase), C(0), C(0), phase};
  }
  auto t = table_gate<T>(g.name);
  if (t.size() == 4) return t;
  // The reference's gate table also holds the full cz and cx (16 entries,
  // src/read_circuit.cpp:61-79). Used on one qubit, they and the two-qubit
  // halves (8 entries) pass its name check, and the one-qubit tensor
  // (4 entries) refuses their data (src/read_circuit.cpp:419-427,
  // src/tensor.cpp:170-180).
  const std::size_t entries = (g.name == "cz" || g.name == "cx") ? 16 : t.size();
  if (entries == 0) throw QFX_ERR("Invalid gate name provided: ", g.name);
  throw QFX_ERR("Failed to call Tensor(). Error:\n\t[The vector data size: ", entries,
                ", has to match the size of the Tensor: 4]");
}

// fSim(theta, phi) split into two identical (input, virtual[4], output)
// halves, angles in units of pi (src/read_circuit.cpp:105-139,156-162);
// T = float repeats the reference's float arithmetic.
template <typename T>
std::vector<std::complex<T>> fsim_half(double theta_pi, double phi_pi) {
  using C = std::complex<T>;
  const T th = static_cast<T>(M_PI * theta_pi);
  const T ph = static_cast<T>(M_PI * phi_pi);
  const C e = std::exp(C(T(0), -1 * ph / 2));
  const C c1 = C(T(0.5)) * (e + C(std::cos(th), T(0)));
  const C c2 = C(T(0.5)) * (e - C(std::cos(th), T(0)));
  const C c3 = C(T(0), static_cast<T>(-1 / 2.)) * C(std::sin(th), T(0));
  const C s1 = std::sqrt(c1), s2 = std::sqrt(c2), s3 = std::sqrt(c3), s4 = std::sqrt(c3);
  const C d = std::exp(C(T(0), static_cast<T>(ph / 4.)));
  const C z(0, 0), I(0, 1);
  return {d * s1, z, d * s2, z, z, s3, z, I * s4,
          z, std::conj(d) * s1, z, -std::conj(d) * s2, s3, z, -I * s4, z};
}

// order_func (src/read_circuit.cpp:191-291): "lhs before rhs" for two
// neighbours of `local`: cut bonds first (in ordering order), then by the
// step at which the contraction reaches each neighbour.
bool neighbour_less(const std::vector<Op>& ops, const Coord& local, const Coord& lhs,
                    const Coord& rhs) {
  auto pair_of = [&](const Coord& n) {
    return (local.first < n.first || local.second < n.second) ? std::vector<Coord>{local, n}
                                                              : std::vector<Coord>{n, local};
  };
  const auto lp = pair_of(lhs), rp = pair_of(rhs);
  for (const auto& op : ops) {
    if (op.kind != Op::CUT) continue;
    if (op.tensors == lp) return true;
    if (op.tensors == rp) return false;
  }
  auto locate = [&](const Coord& n, std::string* patch) -> std::optional<std::size_t> {
    std::size_t k = 0;
    for (const auto& op : ops) {
      if (op.kind != Op::EXPAND) continue;
      if (op.tensor == n) {
        *patch = op.patch;
        return k;
      }
      ++k;
    }
    return std::nullopt;
  };
  std::string lpatch = "null", rpatch = "null";
  auto lpos = locate(lhs, &lpatch);
  if (!lpos)
    throw QFX_ERR("Left hand side of pair not found: (", local.first, ',', local.second, "),(",
                  lhs.first, ',', lhs.second, ").");
  auto rpos = locate(rhs, &rpatch);
  if (!rpos)
    throw QFX_ERR("Right hand side of pair not found: (", local.first, ',', local.second, "),(",
                  rhs.first, ',', rhs.second, ").");
  if (lpatch == rpatch) return *lpos < *rpos;
  std::string local_patch;
  for (const auto& op : ops)
    if (op.kind == Op::EXPAND && op.tensor == local) {
      local_patch = op.patch;
      break;
    }
  if (lpatch == local_patch) return true;
  if (rpatch == local_patch) return false;
  for (const auto& op : ops) {
    if (op.kind != Op::MERGE) continue;
    if (local_patch == op.source) {
      if (lpatch == op.target) return true;
      if (rpatch == op.target) return false;
      local_patch = op.target;
    } else if (local_patch == op.target) {
      if (lpatch == op.source) return true;
      if (rpatch == op.source) return false;
    } else if (lpatch == op.source) {
      lpatch = op.target;
    } else if (rpatch == op.source) {
      rpatch = op.target;
    }
  }
  throw QFX_ERR("Failed to compare (", lhs.first, ',', lhs.second, ") and (", rhs.first, ',',
                rhs.second, ") for local (", local.first, ',', local.second, ").");
}

}  // namespace

Network build_network(const Circuit& circuit, const Grid& grid, const std::string& initial,
                      const std::string& final_conf, const std::vector<Coord>& final_region,
                      const std::vector<Op>& ops) {
  Network net;
  net.I = grid.I;
  net.J = grid.J;
  const long grid_size = grid.I * grid.J;
  const long n_active = grid_size - (long)grid.qubits_off.size();
  if (circuit.num_active_qubits != n_active)
    throw QFX_ERR("The number of active qubits read from the file: ", circuit.num_active_qubits,
                  ", does not match the number of active qubits read from the grid: ", n_active,
                  ".");
  if ((long)initial.size() != n_active)
    throw QFX_ERR("Size of initial_conf: ", initial.size(),
                  ", must be equal to the number of qubits: ", n_active, ".");
  if (final_conf.size() != initial.size())
    throw QFX_ERR("Size of final_conf: ", final_conf.size(),
                  ", must be equal to size of initial_conf: ", initial.size(), ".");
  auto in_region = [&](const Coord& c) {
    return std::find(final_region.begin(), final_region.end(), c) != final_region.end();
  };
  long idx = 0;
  for (long q = 0; q < grid_size; ++q) {
    Coord c{int(q / grid.J), int(q % grid.J)};
    if (grid.is_off(c.first, c.second)) continue;
    QubitColumn col;
    col.pos = c;
    col.init_bit = initial[idx] == '0' ? 0 : 1;
    col.final_bit = final_conf[idx] == '0' ? 0 : 1;
    col.terminal = in_region(c);
    net.column_of[c] = (int)net.columns.size();
    net.columns.push_back(std::move(col));
    ++idx;
  }
  for (const auto& c : grid.qubits_off)
    if (c.first >= grid.I || c.second >= grid.J)
      throw QFX_ERR("Off qubit '(", c.first, ", ", c.second, ")' is outside the grid.");

  // Virtual-index counters are keyed by the pair as written in the circuit
  // (src/read_circuit.cpp:461-477); a pair written in both orders would give
  // two gates the same virtual index, which the reference silently
  // contracts together. That is rejected here instead.
  std::map<std::string, int> link_counters;
  std::set<std::string> virtual_names;
  std::unordered_set<long> used;
  long last_cycle = 0;
  for (const auto& g : circuit.gates) {
    if (g.cycle != last_cycle) {
      last_cycle = g.cycle;
      used.clear();
    }
    for (long q : g.qubits) {
      if (used.count(q))
        throw QFX_ERR("Qubit ", q, " has been used twice in the same cycle: ", g.cycle);
      used.insert(q);
    }
    auto coords = [&](long q) { return Coord{int(q / grid.J), int(q % grid.J)}; };
    auto column = [&](const Coord& c, long q) -> QubitColumn& {
      auto it = net.column_of.find(c);
      if (q < 0 || q >= grid_size || it == net.column_of.end())
        throw QFX_ERR("Qubit '", q, "' in gate '", g.raw, "' must correspond to an active qubit.");
      return net.columns[it->second];
    };
    if (g.qubits.size() == 1) {
      Coord c = coords(g.qubits[0]);
      QubitColumn& col = column(c, g.qubits[0]);
      ColumnStep s{1, 0, -1, 0, one_qubit_gate<float>(g), one_qubit_gate<double>(g)};
      col.steps.push_back(std::move(s));
    } else if (g.qubits.size() == 2) {
      Coord c1 = coords(g.qubits[0]), c2 = coords(g.qubits[1]);
      QubitColumn& col1 = column(c1, g.qubits[0]);
      QubitColumn& col2 = column(c2, g.qubits[1]);
      if (std::abs(c1.first - c2.first) + std::abs(c1.second - c2.second) != 1)
        throw QFX_ERR("Qubits ", g.qubits[0], " and ", g.qubits[1], " are not nearest neighbors.");
      std::vector<cfloat> d1, d2;
      std::vector<std::complex<double>> e1, e2;
      int V = 2;
      if (g.name == "cz" || g.name == "cx") {
        d1 = table_gate<float>(g.name + "_q1");
        d2 = table_gate<float>(g.name + "_q2");
        e1 = table_gate<double>(g.name + "_q1");
        e2 = table_gate<double>(g.name + "_q2");
      } else if (g.name == "fsim") {
        if (g.params.size() < 2) throw QFX_ERR("fsim needs two parameters: ", g.raw);
        d1 = d2 = fsim_half<float>(g.params[0], g.params[1]);
        e1 = e2 = fsim_half<double>(g.params[0], g.params[1]);
        V = 4;
      } else {
        throw QFX_ERR("Invalid gate name provided: ", g.name);
      }
      const int counter = ++link_counters[index_name(c1, c2)];
      const Coord lo{std::min(c1.first, c2.first), std::min(c1.second, c2.second)};
      const Coord hi{std::max(c1.first, c2.first), std::max(c1.second, c2.second)};
      const std::string vname =
          cat("(", lo.first, ",", lo.second, ",", counter, "),(", hi.first, ",", hi.second, ",",
              counter, ")");
      if (!virtual_names.insert(vname).second)
        throw QFX_ERR("Two gates on qubits ", g.qubits[0], " and ", g.qubits[1],
                      " share the virtual index ", vname,
                      "; list the pair in one order throughout the circuit.");
      const std::string lname = index_name(lo, hi);
      auto it = net.link_of.find(lname);
      int link;
      if (it == net.link_of.end()) {
        link = (int)net.links.size();
        net.links.push_back(Link{lo, hi, lname});
        net.link_of[lname] = link;
      } else {
        link = it->second;
      }
      const int ordinal = net.links[link].n_gates++;
      net.links[link].V.push_back(V);
      col1.steps.push_back(ColumnStep{2, V, link, ordinal, d1, e1});
      col2.steps.push_back(ColumnStep{2, V, link, ordinal, d2, e2});
    } else {
      throw QFX_ERR("k-qubit gates with k > 2 not yet implemented.");
    }
  }

  // Final index order of each 2D tensor (src/read_circuit.cpp:624-688):
  // the terminal index first, then bonds sorted by order_func. Every pair of
  // active neighbours has a bond; one without gates has dimension 1, as the
  // reference's empty bundle does.
  for (auto& col : net.columns) {
    const int i = col.pos.first, j = col.pos.second;
    std::vector<Coord> pairs;
    auto active = [&](int a, int b) {
      return a >= 0 && b >= 0 && a < grid.I && b < grid.J && !grid.is_off(a, b);
    };
    if (active(i - 1, j)) pairs.push_back({i - 1, j});
    if (active(i, j - 1)) pairs.push_back({i, j - 1});
    if (active(i + 1, j)) pairs.push_back({i + 1, j});
    if (active(i, j + 1)) pairs.push_back({i, j + 1});
    if (col.terminal) {
      col.indices.push_back(terminal_name(col.pos));
      col.dims.push_back(2);
    }
    std::sort(pairs.begin(), pairs.end(), [&](const Coord& a, const Coord& b) {
      return neighbour_less(ops, col.pos, a, b);
    });
    for (const auto& p : pairs) {
      const bool p_first = p.first < i || p.second < j;
      const std::string name = p_first ? index_name(p, col.pos) : index_name(col.pos, p);
      auto it = net.link_of.find(name);
      col.indices.push_back(name);
      col.dims.push_back(it == net.link_of.end() ? 1 : net.links[it->second].dim());
    }
  }
  return net;
}

std::size_t find_output_pos(const Grid& grid, const Coord& pos) {
  long p = pos.first * grid.J + pos.second;
  for (const auto& off : grid.qubits_off)
    if (off.first < pos.first || (off.first == pos.first && off.second < pos.second)) --p;
  return (std::size_t)p;
}

// get_output_states (src/evaluate_circuit.cpp:38-104): terminal cuts, in
// ordering order, are the digits of the amplitude index, the first one most
// significant.
std::string get_output_states(const Grid& grid, const std::vector<Op>& ops,
                              const std::string& initial, const std::string& final_state,
                              std::vector<Coord>* final_qubits,
                              std::vector<std::string>* output_states) {
  std::string base = final_state;
  const bool unspecified = final_state.empty();
  if (unspecified) base = std::string(initial.size(), '0');
  std::vector<std::size_t> pos_map;
  std::vector<std::vector<std::size_t>> val_map;
  for (const auto& op : ops) {
    if (op.kind != Op::CUT || op.tensors.size() != 1) continue;
    const std::size_t p = find_output_pos(grid, op.tensors[0]);
    if (p >= base.size())
      throw QFX_ERR("Terminal cut at qubit ", p, " is outside the final state of length ",
                    base.size(), ".");
    if (unspecified) base[p] = 'x';
    pos_map.push_back(p);
    val_map.push_back(op.values.empty() ? std::vector<std::size_t>{0, 1} : op.values);
    final_qubits->push_back(op.tensors[0]);
  }
  output_states->assign(1, base);
  for (std::size_t i = 0; i < pos_map.size(); ++i) {
    std::vector<std::string> next;
    for (const auto& s : *output_states)
      for (std::size_t v : val_map[i]) {
        std::string t = s;
        t[pos_map[i]] = std::to_string(v).at(0);
        next.push_back(t);
      }
    *output_states = std::move(next);
  }
  const std::string& first = output_states->at(0);
  for (std::size_t i = 0; i < first.size(); ++i)
    if (first[i] != '0' && first[i] != '1')
      throw QFX_ERR("Final state has non-binary character ", first[i], " at index ", i,
                    "despite having no terminal cut there.");
  return base;
}

}  // namespace qfx
