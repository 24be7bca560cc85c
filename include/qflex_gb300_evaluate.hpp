// C++ drop-in for the reference's public entry point
//   std::vector<std::pair<std::string, std::complex<double>>>
//   qflex::EvaluateCircuit(QflexInput* input)        (src/evaluate_circuit.h:81-82)
// and its input model QflexInput / QflexCircuit / QflexGrid / QflexOrdering
// (src/input.h:11-17, src/circuit.h, src/grid.h, src/ordering.h), implemented
// over the C ABI of libqflex_gb300.so (include/qflex_gb300.h).
//
// Header-only. Semantics kept from the reference:
//   * the input models expose the reference's members (QflexCircuit::
//     num_active_qubits / depth / gates, QflexGrid::I / J / qubits_off,
//     QflexOrdering::instructions); load(stream) / load(filename) parse the
//     text with the engine's parsers and throw the reference's std::string
//     errors at load time; clear() empties them;
//   * EvaluateCircuit reads the members (a caller may build or edit them
//     directly), so it evaluates exactly what they hold;
//   * errors are thrown as std::string;
//   * input->initial_state and input->final_state are mutated exactly as the
//     reference mutates them (src/evaluate_circuit.cpp:130-145);
//   * qflex::global::memory_limit caps the planned scratch (src/global.h:12).
// Each thread gets its own engine context on CUDA device
// qflex::global::device (default 0), created on first use.
#ifndef QFLEX_GB300_EVALUATE_HPP
#define QFLEX_GB300_EVALUATE_HPP

#include <complex>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <memory>
#include <sstream>
#include <string>
#include <utility>
#include <vector>

#include "qflex_gb300.h"

namespace qflex {

namespace global {
inline int verbose = 0;
inline std::size_t memory_limit = std::size_t(1) << 30;
inline int device = 0;
inline int precision = QFLEX_GB300_FP32;
}  // namespace global

namespace detail {
inline std::string read_all(std::istream& in) {
  std::stringstream ss;
  ss << in.rdbuf();
  return ss.str();
}
inline std::string format_double(double v) {
  char buf[64];
  std::snprintf(buf, sizeof(buf), "%.17g", v);
  return buf;
}
}  // namespace detail

// QflexGate (src/circuit.h).
struct QflexGate {
  std::string name;
  std::size_t cycle{0};
  std::vector<std::size_t> qubits;
  std::vector<double> params;
  std::string raw;
};

struct QflexCircuit {
  std::size_t num_active_qubits{0};
  std::size_t depth{0};
  std::vector<QflexGate> gates;
  void clear() {
    num_active_qubits = depth = 0;
    gates.clear();
  }
  void load(std::istream& in) { parse(detail::read_all(in)); }
  void load(std::istream&& in) { load(in); }
  void load(const std::string& filename) {
    std::ifstream in(filename);
    if (!in.good()) throw std::string("Cannot open circuit file ") + filename + ".";
    load(in);
  }
  // The circuit text format of the members (src/circuit.cpp:30-206).
  std::string text() const {
    std::string t = std::to_string(num_active_qubits) + "\n";
    for (const auto& g : gates) {
      t += std::to_string(g.cycle) + " " + g.name;
      if (!g.params.empty()) {
        t += "(";
        for (std::size_t i = 0; i < g.params.size(); ++i) t += (i ? "," : "") + detail::format_double(g.params[i]);
        t += ")";
      }
      for (std::size_t q : g.qubits) t += " " + std::to_string(q);
      t += "\n";
    }
    return t;
  }

 private:
  void parse(const std::string& text) {
    clear();
    char err[4096];
    qflex_gb300_circuit* raw_handle = nullptr;
    if (qflex_gb300_circuit_load(text.c_str(), &raw_handle, err, sizeof(err)) != QFLEX_GB300_OK)
      throw std::string(err);
    // Freed however this function is left.
    const std::unique_ptr<qflex_gb300_circuit, void (*)(qflex_gb300_circuit*)> handle(raw_handle,
                                                                                     qflex_gb300_circuit_free);
    const qflex_gb300_circuit* c = handle.get();
    num_active_qubits = qflex_gb300_circuit_num_active_qubits(c);
    depth = qflex_gb300_circuit_depth(c);
    const std::size_t n = qflex_gb300_circuit_gate_count(c);
    for (std::size_t i = 0; i < n; ++i) {
      const char *name = nullptr, *raw = nullptr;
      std::size_t cycle = 0, qubits[8], nq = 0, np = 0;
      double params[8];
      qflex_gb300_circuit_gate(c, i, &name, &raw, &cycle, qubits, 8, &nq, params, 8, &np);
      QflexGate g;
      g.name = name ? name : "";
      g.raw = raw ? raw : "";
      g.cycle = cycle;
      g.qubits.assign(qubits, qubits + (nq < 8 ? nq : 8));
      g.params.assign(params, params + (np < 8 ? np : 8));
      gates.push_back(std::move(g));
    }
  }
};

struct QflexGrid {
  std::size_t I{0}, J{0};
  std::vector<std::vector<std::size_t>> qubits_off;
  void clear() {
    I = J = 0;
    qubits_off.clear();
  }
  void load(std::istream& in) { parse(detail::read_all(in)); }
  void load(std::istream&& in) { load(in); }
  void load(const std::string& filename) {
    std::ifstream in(filename);
    if (!in.good()) throw std::string("Cannot open grid file: ") + filename + ".";
    load(in);
  }
  // The grid text format of the members (src/grid.cpp:11-45).
  std::string text() const {
    std::string t;
    for (std::size_t i = 0; i < I; ++i) {
      for (std::size_t j = 0; j < J; ++j) {
        bool off = false;
        for (const auto& q : qubits_off) off |= q.size() == 2 && q[0] == i && q[1] == j;
        t += j ? (off ? " 0" : " 1") : (off ? "0" : "1");
      }
      t += "\n";
    }
    return t;
  }

 private:
  void parse(const std::string& text) {
    clear();
    char err[4096];
    std::size_t n_off = 0;
    if (qflex_gb300_grid_load(text.c_str(), &I, &J, nullptr, 0, &n_off, err, sizeof(err)) != QFLEX_GB300_OK)
      throw std::string(err);
    std::vector<std::size_t> off(2 * n_off + 2);
    qflex_gb300_grid_load(text.c_str(), &I, &J, off.data(), n_off, &n_off, err, sizeof(err));
    for (std::size_t q = 0; q < n_off; ++q) qubits_off.push_back({off[2 * q], off[2 * q + 1]});
  }
};

struct QflexOrdering {
  std::vector<std::string> instructions;
  void clear() { instructions.clear(); }
  void load(std::istream& in) { parse(detail::read_all(in)); }
  void load(std::istream&& in) { load(in); }
  void load(const std::string& filename) {
    std::ifstream in(filename);
    if (!in.good()) throw std::string("Cannot open ordering file: ") + filename;
    load(in);
  }
  std::string text() const {
    std::string t;
    for (const auto& line : instructions) t += line + "\n";
    return t;
  }

 private:
  void parse(const std::string& text) {
    clear();
    char err[4096];
    std::size_t n = 0, needed = 0;
    if (qflex_gb300_ordering_load(text.c_str(), nullptr, 0, &n, &needed, err, sizeof(err)) != QFLEX_GB300_OK)
      throw std::string(err);
    std::string joined(needed, '\0');
    qflex_gb300_ordering_load(text.c_str(), &joined[0], needed, &n, &needed, err, sizeof(err));
    joined.resize(needed ? needed - 1 : 0);
    std::size_t start = 0;
    for (std::size_t i = 0; i < n; ++i) {
      const std::size_t end = joined.find('\n', start);
      instructions.push_back(joined.substr(start, end == std::string::npos ? std::string::npos : end - start));
      start = end == std::string::npos ? joined.size() : end + 1;
    }
  }
};

struct QflexInput {
  QflexOrdering ordering;
  QflexCircuit circuit;
  QflexGrid grid;
  std::string initial_state;
  std::string final_state;
};

namespace detail {
struct Context {
  qflex_gb300_context* ctx = nullptr;
  int device = -2;
  ~Context() { qflex_gb300_destroy(ctx); }
  qflex_gb300_context* get() {
    if (!ctx || device != global::device) {
      qflex_gb300_destroy(ctx);
      ctx = nullptr;
      const int rc = qflex_gb300_create(global::device, global::precision, &ctx);
      if (rc != QFLEX_GB300_OK) {
        std::string msg = qflex_gb300_last_error(ctx);
        qflex_gb300_destroy(ctx);
        ctx = nullptr;
        throw msg;
      }
      device = global::device;
    }
    if (qflex_gb300_set_precision(ctx, global::precision) != QFLEX_GB300_OK)
      throw std::string(qflex_gb300_last_error(ctx));
    return ctx;
  }
};
inline Context& thread_context() {
  thread_local Context c;
  return c;
}
}  // namespace detail

inline std::vector<std::pair<std::string, std::complex<double>>> EvaluateCircuit(QflexInput* input) {
  if (input == nullptr) throw std::string("ERROR (qflex_gb300: EvaluateCircuit) --> Input must be non-null.");
  qflex_gb300_context* ctx = detail::thread_context().get();
  const std::string circuit = input->circuit.text(), ordering = input->ordering.text(),
                    grid = input->grid.text();
  const int rc = qflex_gb300_evaluate(ctx, circuit.c_str(), ordering.c_str(), grid.c_str(),
                                      input->initial_state.c_str(), input->final_state.c_str(),
                                      double(global::memory_limit));
  if (rc != QFLEX_GB300_OK) throw std::string(qflex_gb300_last_error(ctx));
  input->initial_state = qflex_gb300_result_initial_state(ctx);
  input->final_state = qflex_gb300_result_final_state(ctx, 0);
  std::vector<std::pair<std::string, std::complex<double>>> out;
  const std::size_t n = qflex_gb300_result_count(ctx);
  for (std::size_t i = 0; i < n; ++i) {
    double re = 0, im = 0;
    qflex_gb300_result_amplitude(ctx, i, &re, &im);
    out.emplace_back(qflex_gb300_result_state(ctx, i), std::complex<double>(re, im));
  }
  return out;
}

}  // namespace qflex

#endif  // QFLEX_GB300_EVALUATE_HPP
