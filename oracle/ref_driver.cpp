// Command-line driver around the unmodified reference library (test
// infrastructure only; it links the reference sources compiled by
// oracle/Makefile and is used to pin the oracle and to generate golden
// fixtures). The reference's own CLI (src/main.cpp) needs the docopt
// submodule, which is empty, so this driver calls the same public entry point
// qflex::EvaluateCircuit (src/evaluate_circuit.h:81-82) directly.
//
// Usage:
//   qflex_ref eval <circuit> <ordering> <grid> <initial|-> <final|-> [mem]
//       prints "<state> <re> <im>" per amplitude (%.17g), exit 2 on a
//       reference error (message on stdout after "ERROR ").
//   qflex_ref reorder <n_binary> <perm...>
//       tensor of n binary indices named i0..i(n-1) with data[p] = p,
//       reordered to (i<perm[0]>, ...); prints the real parts.
//   qflex_ref reorder_dims <n> <dim...> <perm...>
//       the same with n indices of the given dimensions (any sizes; the
//       reference reorders those with its naive path).
//   qflex_ref threads <n> eval ...   (sets the OpenBLAS thread count first)
//   qflex_ref [threads <n>] time <reps> eval ...
//       runs EvaluateCircuit <reps> times on the loaded input and prints
//       "SECONDS <s>" for each run (wall time of the call alone, input
//       loading excluded), then the amplitudes of the last run.
#include <chrono>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "evaluate_circuit.h"
#include "global.h"
#include "input.h"
#include "tensor.h"
#include "utils.h"

extern "C" void scipy_openblas_set_num_threads(int);

static bool timed_mode = false;

static int do_eval(int argc, char** argv, int reps = 1) {
  if (argc < 7) {
    std::fprintf(stderr, "eval needs 5 arguments\n");
    return 64;
  }
  qflex::QflexInput input;
  try {
    input.circuit.load(std::string(argv[2]));
    input.ordering.load(std::string(argv[3]));
    input.grid.load(std::string(argv[4]));
    input.initial_state = std::strcmp(argv[5], "-") ? argv[5] : "";
    input.final_state = std::strcmp(argv[6], "-") ? argv[6] : "";
    if (argc > 7)
      qflex::global::memory_limit =
          qflex::utils::from_readable_memory_string(argv[7]);
    const std::string initial = input.initial_state, final_state = input.final_state;
    std::vector<std::pair<std::string, std::complex<double>>> amps;
    for (int r = 0; r < reps; ++r) {
      // EvaluateCircuit mutates the states; every run starts from the
      // caller's strings.
      input.initial_state = initial;
      input.final_state = final_state;
      const auto t0 = std::chrono::steady_clock::now();
      amps = qflex::EvaluateCircuit(&input);
      const auto t1 = std::chrono::steady_clock::now();
      if (reps > 1 || timed_mode)
        std::printf("SECONDS %.6f\n", std::chrono::duration<double>(t1 - t0).count());
    }
    std::printf("INITIAL %s\n", input.initial_state.c_str());
    std::printf("FINAL %s\n", input.final_state.c_str());
    for (auto& [state, a] : amps)
      std::printf("%s %.17g %.17g\n", state.c_str(), a.real(), a.imag());
  } catch (const std::string& msg) {
    std::string one = msg;
    for (auto& c : one)
      if (c == '\n') c = ' ';
    std::printf("ERROR %s\n", one.c_str());
    return 2;
  }
  return 0;
}

static int do_reorder(int argc, char** argv) {
  std::size_t n = std::strtoul(argv[2], nullptr, 10);
  std::vector<std::string> names(n), order;
  for (std::size_t i = 0; i < n; ++i) names[i] = "i" + std::to_string(i);
  for (int a = 3; a < argc; ++a) order.push_back(names[std::atoi(argv[a])]);
  std::vector<std::size_t> dims(n, 2);
  std::size_t size = std::size_t(1) << n;
  std::vector<qflex::s_type> data(size);
  for (std::size_t p = 0; p < size; ++p) data[p] = qflex::s_type(float(p), 0.f);
  qflex::Tensor t(names, dims, data);
  std::vector<qflex::s_type> scratch(size);
  t.reorder(order, scratch.data());
  for (std::size_t p = 0; p < size; ++p)
    std::printf("%ld\n", (long)t.data()[p].real());
  return 0;
}

static int do_reorder_dims(int argc, char** argv) {
  const std::size_t n = std::strtoul(argv[2], nullptr, 10);
  if (argc < int(3 + 2 * n)) {
    std::fprintf(stderr, "reorder_dims needs n dimensions and n positions\n");
    return 64;
  }
  std::vector<std::string> names(n), order;
  std::vector<std::size_t> dims(n);
  std::size_t size = 1;
  for (std::size_t i = 0; i < n; ++i) {
    names[i] = "i" + std::to_string(i);
    dims[i] = std::strtoul(argv[3 + i], nullptr, 10);
    size *= dims[i];
  }
  for (std::size_t i = 0; i < n; ++i) order.push_back(names[std::atoi(argv[3 + n + i])]);
  std::vector<qflex::s_type> data(size);
  for (std::size_t p = 0; p < size; ++p) data[p] = qflex::s_type(float(p), 0.f);
  qflex::Tensor t(names, dims, data);
  std::vector<qflex::s_type> scratch(size);
  t.reorder(order, scratch.data());
  for (std::size_t p = 0; p < size; ++p) std::printf("%ld\n", (long)t.data()[p].real());
  return 0;
}

int main(int argc, char** argv) {
  if (argc >= 3 && !std::strcmp(argv[1], "threads")) {
    scipy_openblas_set_num_threads(std::atoi(argv[2]));
    argv += 2;
    argc -= 2;
  }
  int reps = 1;
  if (argc >= 3 && !std::strcmp(argv[1], "time")) {
    reps = std::atoi(argv[2]);
    if (reps < 1) reps = 1;
    timed_mode = true;
    argv += 2;
    argc -= 2;
  }
  if (argc >= 2 && !std::strcmp(argv[1], "eval")) return do_eval(argc, argv, reps);
  if (argc >= 3 && !std::strcmp(argv[1], "reorder"))
    return do_reorder(argc, argv);
  if (argc >= 3 && !std::strcmp(argv[1], "reorder_dims")) return do_reorder_dims(argc, argv);
  std::fprintf(stderr, "usage: qflex_ref [threads N] eval|reorder ...\n");
  return 64;
}
