// The reference's EvaluateCircuit known-answer test and input-model checks,
// run through the C++ drop-in header (include/qflex_gb300_evaluate.hpp).
// The circuit, ordering and grid are those of the reference's
// tests/src/evaluate_circuit_test.cpp:134-207.
//
//   evaluate_circuit_dropin parse   input models only (no GPU)
//   evaluate_circuit_dropin eval    EvaluateCircuit on CUDA device 0
// Prints "OK <check>" per passed check; exits 1 at the first failure.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <sstream>
#include <string>

#include "qflex_gb300_evaluate.hpp"

namespace {

const char kCircuit[] = R"(5
0 h 0
0 h 1
0 h 2
0 h 3
0 h 5
1 t 0
1 t 1
1 t 2
1 t 3
1 t 5
2 cz 0 1
3 cx 0 2
4 cx 1 3
5 cz 2 3
6 cz 3 5
11 cz 0 1
12 cx 0 2
13 cx 1 3
14 cz 2 3
15 cx 3 5
17 h 0
17 h 1
17 h 2
17 h 3
17 h 5)";

const char kOrdering[] = R"(#
cut () 1 3
expand a 1
expand a 0
expand a 2
cut () 5
expand b 5
expand b 3
merge a b
)";

const char kGrid[] = R"(1 1
                        1 1
                        0 1)";

int failures = 0;
void check(bool ok, const char* what) {
  std::printf("%s %s\n", ok ? "OK" : "FAIL", what);
  if (!ok) ++failures;
}

template <typename F>
std::string thrown(F&& f) {
  try {
    f();
  } catch (const std::string& msg) {
    return msg;
  }
  return "";
}

void load(qflex::QflexInput& input) {
  std::stringstream circuit(kCircuit), ordering(kOrdering), grid(kGrid);
  input.circuit.load(circuit);
  input.ordering.load(ordering);
  input.grid.load(grid);
}

int parse_checks() {
  qflex::QflexInput input;
  load(input);
  check(input.circuit.num_active_qubits == 5, "circuit.num_active_qubits");
  check(input.circuit.gates.size() == 25, "circuit.gates.size()");
  check(input.circuit.gates[10].name == "cz" && input.circuit.gates[10].cycle == 2 &&
            input.circuit.gates[10].qubits == std::vector<std::size_t>{0, 1},
        "circuit.gates[10]");
  check(input.circuit.depth == 2, "circuit.depth");
  check(input.grid.I == 3 && input.grid.J == 2, "grid.I, grid.J");
  check(input.grid.qubits_off == std::vector<std::vector<std::size_t>>{{2, 0}}, "grid.qubits_off");
  check(input.ordering.instructions.size() == 8 && input.ordering.instructions[0] == "cut () 1 3" &&
            input.ordering.instructions[7] == "merge a b",
        "ordering.instructions");
  // The members serialize to text that parses back to the same members.
  qflex::QflexCircuit again;
  again.load(std::stringstream(input.circuit.text()));
  bool same = again.gates.size() == input.circuit.gates.size();
  for (std::size_t i = 0; same && i < again.gates.size(); ++i)
    same = again.gates[i].name == input.circuit.gates[i].name &&
           again.gates[i].qubits == input.circuit.gates[i].qubits &&
           again.gates[i].cycle == input.circuit.gates[i].cycle;
  check(same, "circuit text round trip");
  qflex::QflexGate f;
  f.name = "fsim";
  f.cycle = 1;
  f.qubits = {0, 1};
  f.params = {0.5, 1.0 / 6.0};
  qflex::QflexCircuit fc;
  fc.num_active_qubits = 2;
  fc.gates = {f};
  qflex::QflexCircuit fc2;
  fc2.load(std::stringstream(fc.text()));
  check(fc2.gates.size() == 1 && fc2.gates[0].params == f.params && fc2.depth == 2, "fsim parameters round trip");
  // Parse errors are thrown by load(), as the reference's load() throws them.
  const std::string bad = thrown([] {
    qflex::QflexCircuit c;
    c.load(std::stringstream("2\n1 cz 0 1\n0 h 0\n"));
  });
  check(bad.find("Cycle number can only increase.") != std::string::npos, "circuit load error");
  const std::string bad_grid = thrown([] {
    qflex::QflexGrid g;
    g.load(std::stringstream("1 1\n1 1 1\n"));
  });
  check(bad_grid.find("is inconsistent with a width of") != std::string::npos, "grid load error");
  const std::string missing = thrown([] {
    qflex::QflexCircuit c;
    c.load(std::string("/nonexistent/circuit.txt"));
  });
  check(missing.find("Cannot open circuit file") != std::string::npos, "missing file");
  const std::string null_input = thrown([] { qflex::EvaluateCircuit(nullptr); });
  check(null_input.find("Input must be non-null.") != std::string::npos, "null input");
  return failures ? 1 : 0;
}

int eval_checks() {
  qflex::QflexInput input;
  load(input);
  input.initial_state = "00000";
  input.final_state = "1100x";
  const auto amplitudes = qflex::EvaluateCircuit(&input);
  check(amplitudes.size() == 2, "two amplitudes");
  check(amplitudes[0].first == "11000" && amplitudes[1].first == "11001", "output states");
  // EXPECT_NEAR(..., 1e-5) of evaluate_circuit_test.cpp:203-206.
  check(std::abs(amplitudes[0].second.real() - 0.10669) < 1e-5 &&
            std::abs(amplitudes[0].second.imag() - 0.04419) < 1e-5,
        "amplitude 0");
  check(std::abs(amplitudes[1].second.real() + 0.01831) < 1e-5 &&
            std::abs(amplitudes[1].second.imag() + 0.25758) < 1e-5,
        "amplitude 1");
  check(input.final_state == "1100x" && input.initial_state == "00000", "mutated states");
  // Members edited by the caller are what gets evaluated: dropping the last
  // Hadamard layer from the model changes the amplitudes.
  qflex::QflexInput edited;
  load(edited);
  edited.circuit.gates.resize(20);
  edited.initial_state = "00000";
  edited.final_state = "1100x";
  const auto other = qflex::EvaluateCircuit(&edited);
  check(other.size() == 2 && std::abs(other[0].second - amplitudes[0].second) > 1e-3, "edited members evaluated");
  // The reference's memory-limit error, as a thrown std::string.
  const std::size_t saved = qflex::global::memory_limit;
  qflex::global::memory_limit = 512;
  const std::string mem = thrown([&] {
    qflex::QflexInput in;
    load(in);
    in.initial_state = "00000";
    in.final_state = "1100x";
    qflex::EvaluateCircuit(&in);
  });
  qflex::global::memory_limit = saved;
  check(mem.find("exceeds memory limit") != std::string::npos, "memory limit error");
  return failures ? 1 : 0;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc > 1 && !std::strcmp(argv[1], "parse")) return parse_checks();
  if (argc > 1 && !std::strcmp(argv[1], "eval")) return eval_checks();
  std::fprintf(stderr, "usage: evaluate_circuit_dropin parse|eval\n");
  return 64;
}
