// Parsers for the three text inputs of the contraction path. The accepted
// syntax and the error texts follow the reference's formats:
//   circuit  : src/circuit.cpp:30-206   ("<cycle> <gate>[(p,..)] q1 [q2]")
//   grid     : src/grid.cpp:11-45       (0/1 matrix, 0 = qubit off)
//   ordering : src/ordering.cpp:10-45   (expand / cut / merge lines)
//   memory   : src/utils.cpp:19-68      ("16GB", "512MB", ...)
#include <algorithm>
#include <cmath>
#include <regex>
#include <set>
#include <unordered_map>

#include "qfx.h"

namespace qfx {
namespace {

std::vector<std::string> split_lines(const std::string& text) {
  std::vector<std::string> out;
  std::string cur;
  std::istringstream in(text);
  while (std::getline(in, cur)) out.push_back(cur);
  return out;
}

// Line clean-up shared by the circuit and ordering formats.
std::string strip_common(std::string line) {
  static const std::regex comment("#.*"), special("[^)(\\s\\ta-zA-Z0-9_.,-]"),
      tab("[\\t]"), spaces("[\\s]{2,}"), trailing("\\s+$");
  line = std::regex_replace(line, comment, "");
  line = std::regex_replace(line, special, "");
  line = std::regex_replace(line, tab, " ");
  line = std::regex_replace(line, spaces, " ");
  line = std::regex_replace(line, trailing, "");
  return line;
}

std::string strip_inside_parens(std::string line) {
  static const std::regex in_parens("\\s+(?=[^()]*\\))");
  return std::regex_replace(line, in_parens, "");
}

bool is_number(const std::string& tok) {
  try {
    (void)std::stol(tok);
  } catch (...) {
    return false;
  }
  return true;
}

bool is_integer(const std::string& tok) {
  return is_number(tok) && double(std::stol(tok)) == std::stod(tok);
}

std::vector<std::string> tokens_of(const std::string& line, char sep = ' ') {
  std::vector<std::string> out;
  std::string cur;
  for (char c : line) {
    bool is_sep = sep == ' ' ? std::isspace((unsigned char)c) != 0 : c == sep;
    if (is_sep) {
      if (!cur.empty()) out.push_back(cur);
      cur.clear();
    } else {
      cur.push_back(c);
    }
  }
  if (!cur.empty()) out.push_back(cur);
  return out;
}

}  // namespace

void Circuit::load(const std::string& text) {
  num_active_qubits = 0;
  depth = 0;
  gates.clear();
  static const std::regex before_paren("[\\s]+[(]");
  long last_cycle = 0;
  std::set<long> used;
  std::size_t counter = 0;
  std::string line;
  auto error = [&](const std::string& msg) {
    return QFX_ERR("[", counter + 1, ": ", line, "] ", msg);
  };
  for (const std::string& raw : split_lines(text)) {
    line = strip_common(raw);
    line = std::regex_replace(line, before_paren, "(");
    line = strip_inside_parens(line);
    if (!line.empty()) {
      auto n_open = std::count(line.begin(), line.end(), '(');
      auto n_close = std::count(line.begin(), line.end(), ')');
      if (n_open != n_close || n_open > 1) throw error("Not-matching parentheses.");
      auto tok = tokens_of(line);
      if (counter == 0) {
        if (tok.size() != 1 || !is_number(tok[0]) || std::stol(tok[0]) <= 0)
          throw error("First line in circuit must be the number of active qubits.");
        num_active_qubits = std::stol(tok[0]);
      } else {
        if (tok.size() < 3)
          throw error(
              "Gate must be specified as: cycle gate_name[(p1[,p2,...])] q1 "
              "[q2, ...]");
        Gate g;
        g.raw = line;
        if (!is_integer(tok[0])) throw error("First token must be a valid cycle number.");
        g.cycle = std::stol(tok[0]);
        if (g.cycle < last_cycle) throw error("Cycle number can only increase.");
        if (g.cycle != last_cycle) {
          used.clear();
          last_cycle = g.cycle;
        }
        auto beg = tok[1].find('(');
        if (beg != std::string::npos) {
          g.name = tok[1].substr(0, beg);
          std::string params = tok[1].substr(beg + 1, tok[1].find(')') - beg - 1);
          for (const auto& p : tokens_of(params, ',')) {
            if (!is_number(p)) throw QFX_ERR("Params must be valid numbers.");
            g.params.push_back(std::stod(p));
          }
        } else {
          g.name = tok[1];
        }
        for (std::size_t i = 2; i < tok.size(); ++i) {
          if (!is_integer(tok[i])) throw error("Qubit must be a valid number.");
          g.qubits.push_back(std::stol(tok[i]));
        }
        for (long q : g.qubits) {
          if (used.count(q)) throw error("Qubits can only used once per cycle.");
          used.insert(q);
        }
        gates.push_back(std::move(g));
      }
    }
    ++counter;
  }
  // Depth: the largest number of two-qubit interactions on one pair
  // (fsim counts twice), src/circuit.cpp:182-205.
  std::map<std::pair<long, long>, long> layers;
  for (const auto& g : gates) {
    if (g.qubits.size() > 2)
      throw error("Depth calculation does not handle k-qubit gates with k > 2.");
    if (g.qubits.size() == 2) {
      long a = g.qubits[0], b = g.qubits[1];
      if (b > a) std::swap(a, b);
      long& d = layers[{a, b}];
      d += (g.name == "fsim") ? 2 : 1;
      depth = std::max(depth, d);
    }
  }
}

void Grid::load(const std::string& text) {
  I = J = 0;
  qubits_off.clear();
  std::size_t counter = 0;
  for (std::string line : split_lines(text)) {
    if (line.empty() || line[0] == '#') continue;
    ++counter;
    line.erase(std::remove_if(line.begin(), line.end(),
                              [](char c) { return !(c == '0' || c == '1'); }),
               line.end());
    if (line.empty()) continue;
    if (J != 0 && J != (long)line.size())
      throw QFX_ERR("Grid size at line ", counter, " is inconsistent with a width of ",
                    line.size(), " instead of ", J, ".");
    J = (long)line.size();
    for (long q = 0; q < J; ++q)
      if (line[q] == '0') qubits_off.push_back({(int)I, (int)q});
    ++I;
  }
}

bool Grid::is_off(int i, int j) const {
  return std::find(qubits_off.begin(), qubits_off.end(), Coord{i, j}) != qubits_off.end();
}

void Ordering::load(const std::string& text) {
  instructions.clear();
  for (const std::string& raw : split_lines(text)) {
    std::string line = strip_inside_parens(strip_common(raw));
    if (!line.empty()) instructions.push_back(line);
  }
}

std::size_t parse_memory_string(std::string s) {
  static const std::regex special("[^)(\\s\\ta-zA-Z0-9_.,-]");
  s = std::regex_replace(s, special, "");
  s.erase(std::remove_if(s.begin(), s.end(), [](char c) { return c == ' ' || c == '\t'; }),
          s.end());
  for (auto& c : s) c = (char)std::toupper((unsigned char)c);
  std::size_t cut = std::min(s.find_first_not_of("0123456789"), s.size());
  if (cut == 0) throw QFX_ERR("Memory string '", s, "' must start with a number.");
  std::size_t m = std::stoull(s.substr(0, cut));
  std::string suffix = s.substr(cut);
  if (suffix == "GB")
    m <<= 30;
  else if (suffix == "MB")
    m <<= 20;
  else if (suffix == "KB")
    m <<= 10;
  else if (!(suffix == "B" || suffix.empty()))
    throw QFX_ERR("Suffix ", suffix, " not recognized.");
  return m;
}

std::string readable_memory_string(double bytes) {
  const char* suffix[] = {" B", " kB", " MB", " GB"};
  int scale = 0;
  while (bytes >= 1024 && scale < 3) {
    ++scale;
    bytes /= 1024;
  }
  return cat(double(static_cast<std::size_t>(bytes * 100)) / 100., suffix[scale]);
}

}  // namespace qfx
