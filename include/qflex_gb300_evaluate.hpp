// C++ drop-in for the reference's public entry point
//   std::vector<std::pair<std::string, std::complex<double>>>
//   qflex::EvaluateCircuit(QflexInput* input)        (src/evaluate_circuit.h:81-82)
// and its input model QflexInput / QflexCircuit / QflexGrid / QflexOrdering
// (src/input.h:11-17, src/circuit.h, src/grid.h, src/ordering.h), implemented
// over the C ABI of libqflex_gb300.so (include/qflex_gb300.h).
//
// Header-only. Semantics kept from the reference:
//   * the input files are loaded with load(stream) / load(filename);
//     parsing and validation happen inside EvaluateCircuit, with the
//     reference's error texts;
//   * errors are thrown as std::string;
//   * input->initial_state and input->final_state are mutated exactly as the
//     reference mutates them (src/evaluate_circuit.cpp:130-145);
//   * qflex::global::memory_limit caps the planned scratch (src/global.h:12).
// Each thread gets its own engine context on CUDA device
// qflex::global::device (default 0), created on first use.
#ifndef QFLEX_GB300_EVALUATE_HPP
#define QFLEX_GB300_EVALUATE_HPP

#include <complex>
#include <fstream>
#include <iostream>
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
struct TextInput {
  std::string text;
  void load(std::istream& in) {
    std::stringstream ss;
    ss << in.rdbuf();
    text = ss.str();
  }
  void load(std::istream&& in) { load(in); }
};
}  // namespace detail

struct QflexCircuit : detail::TextInput {
  using detail::TextInput::load;
  void load(const std::string& filename) {
    std::ifstream in(filename);
    if (!in.good()) throw std::string("Cannot open circuit file ") + filename + ".";
    detail::TextInput::load(in);
  }
};

struct QflexGrid : detail::TextInput {
  using detail::TextInput::load;
  void load(const std::string& filename) {
    std::ifstream in(filename);
    if (!in.good()) throw std::string("Cannot open grid file: ") + filename + ".";
    detail::TextInput::load(in);
  }
};

struct QflexOrdering : detail::TextInput {
  using detail::TextInput::load;
  void load(const std::string& filename) {
    std::ifstream in(filename);
    if (!in.good()) throw std::string("Cannot open ordering file: ") + filename;
    detail::TextInput::load(in);
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
  const int rc = qflex_gb300_evaluate(ctx, input->circuit.text.c_str(), input->ordering.text.c_str(),
                                      input->grid.text.c_str(), input->initial_state.c_str(),
                                      input->final_state.c_str(), double(global::memory_limit));
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
