// Command-line front end with the reference CLI's arguments and output
// (src/main.cpp:14-38 usage, :140-146 output lines, :148-155 exit codes),
// running the GB300 engine through the C++ drop-in header.
//
//   qflex <circuit> <ordering> <grid> [<initial_conf> <final_conf> <verbosity> <memory_limit>]
//   qflex -c <circuit> -o <ordering> -g <grid> [--initial-conf=S] [--final-conf=S]
//         [--verbosity=N] [--memory=M] [--device=N] [--precision=fp32|tf32x3|fp16x3|bf16x3|fp64|fp64ff]
//
// Output: one line "<initial> --> <state>: <re> <im>" per amplitude.
// Exit codes: 0 ok, 1 std::exception, 2 error message (thrown string).
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <map>
#include <string>
#include <vector>

#include "qflex_gb300_evaluate.hpp"

namespace {

std::size_t parse_memory(std::string s) {
  std::string digits, suffix;
  for (char c : s) {
    if (c == ' ' || c == '\t') continue;
    if (suffix.empty() && c >= '0' && c <= '9')
      digits += c;
    else
      suffix += (char)std::toupper((unsigned char)c);
  }
  if (digits.empty()) throw std::string("Memory limit '") + s + "' must start with a number.";
  std::size_t m = std::stoull(digits);
  if (suffix == "GB") return m << 30;
  if (suffix == "MB") return m << 20;
  if (suffix == "KB") return m << 10;
  if (suffix.empty() || suffix == "B") return m;
  throw std::string("Suffix ") + suffix + " not recognized.";
}

const char* kUsage =
    "Usage:\n"
    "  qflex <circuit_filename> <ordering_filename> <grid_filename> [<initial_conf> <final_conf> "
    "<verbosity_level> <memory_limit>]\n"
    "  qflex -c <circuit_filename> -o <ordering_filename> -g <grid_filename> [--initial-conf=S "
    "--final-conf=S --verbosity=N --memory=M --device=N --precision=fp32|tf32x3|fp16x3|bf16x3|fp64|fp64ff]\n";

}  // namespace

int main(int argc, char** argv) {
  try {
    std::vector<std::string> pos;
    std::map<std::string, std::string> opt;
    for (int i = 1; i < argc; ++i) {
      std::string a = argv[i];
      if (a == "-h" || a == "--help") {
        std::cout << kUsage;
        return 0;
      }
      if (a == "-c" || a == "-o" || a == "-g") {
        if (i + 1 >= argc) throw std::string("Missing value after ") + a;
        opt[a] = argv[++i];
      } else if (a.rfind("--", 0) == 0) {
        const auto eq = a.find('=');
        if (eq == std::string::npos) throw std::string("Options take the form --name=value: ") + a;
        opt[a.substr(0, eq)] = a.substr(eq + 1);
      } else {
        pos.push_back(a);
      }
    }
    auto pick = [&](const char* flag, std::size_t p) -> std::string {
      if (opt.count(flag)) return opt[flag];
      return p < pos.size() ? pos[p] : std::string();
    };
    const std::string circuit = pick("-c", 0), ordering = pick("-o", 1), grid = pick("-g", 2);
    if (circuit.empty() || ordering.empty() || grid.empty()) {
      std::cerr << kUsage;
      return 1;
    }
    qflex::QflexInput input;
    input.initial_state = pick("--initial-conf", 3);
    input.final_state = pick("--final-conf", 4);
    const std::string verbosity = pick("--verbosity", 5), memory = pick("--memory", 6);
    if (!verbosity.empty()) qflex::global::verbose = std::atoi(verbosity.c_str());
    if (!memory.empty()) qflex::global::memory_limit = parse_memory(memory);
    if (opt.count("--device")) qflex::global::device = std::atoi(opt["--device"].c_str());
    if (opt.count("--precision")) {
      const std::string p = opt["--precision"];
      if (p == "fp32")
        qflex::global::precision = QFLEX_GB300_FP32;
      else if (p == "tf32x3")
        qflex::global::precision = QFLEX_GB300_TF32X3;
      else if (p == "fp16x3")
        qflex::global::precision = QFLEX_GB300_FP16X3;
      else if (p == "bf16x3")
        qflex::global::precision = QFLEX_GB300_BF16X3;
      else if (p == "fp64")
        qflex::global::precision = QFLEX_GB300_FP64;
      else if (p == "fp64ff")
        qflex::global::precision = QFLEX_GB300_FP64_FF;
      else
        throw std::string("Unknown precision ") + p;
    }
    input.circuit.load(circuit);
    input.ordering.load(ordering);
    input.grid.load(grid);
    std::vector<std::pair<std::string, std::complex<double>>> amplitudes;
    try {
      amplitudes = qflex::EvaluateCircuit(&input);
    } catch (const std::string& msg) {
      throw std::string("ERROR (qflex_gb300: main) --> Failed to call EvaluateCircuit(). Error:\n\t[") + msg + "]";
    }
    std::cout.precision(17);
    for (const auto& [state, amp] : amplitudes)
      std::cout << input.initial_state << " --> " << state << ": " << amp.real() << " " << amp.imag() << "\n";
  } catch (const std::exception& e) {
    std::cerr << e.what() << std::endl;
    return 1;
  } catch (const std::string& msg) {
    std::cerr << msg << std::endl;
    return 2;
  }
  return 0;
}
