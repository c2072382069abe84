// toml_config.hpp — the reference's TOML configuration, read natively.
//
// A reader for the subset of TOML the reference's configuration files use
// (tables and dotted sub-tables, `key = value` with strings, booleans,
// integers, floats and one-line or multi-line arrays, `#` comments), and
// DqmcInitializer::parse_toml_config's rules on top of it
// (src/dqmc_initializer.cpp:27-338): the same tables, keys and defaults, and an
// error (ConfigError) wherever the reference prints a message and exits.  The
// Python reader dqmc_gb300.io.parse_config applies the same rules.
#pragma once
#include <cctype>
#include <cmath>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

namespace dqmc_app {

struct ConfigError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

// ---- the TOML subset --------------------------------------------------------
struct TomlValue {
  enum Kind { STR, INT, FLOAT, BOOL, ARRAY } kind = STR;
  std::string s;
  long long i = 0;
  double f = 0;
  bool b = false;
  std::vector<TomlValue> items;
};

class Toml {
 public:
  explicit Toml(const std::string& text) { parse(text); }
  const TomlValue* find(const std::string& dotted) const {
    auto it = values_.find(dotted);
    return it == values_.end() ? nullptr : &it->second;
  }
  // toml++'s value_or: a number of either kind converts to double; anything else gives the default
  double number_or(const std::string& k, double d) const {
    const TomlValue* v = find(k);
    if (!v) return d;
    if (v->kind == TomlValue::FLOAT) return v->f;
    if (v->kind == TomlValue::INT) return (double)v->i;
    return d;
  }
  long long int_or(const std::string& k, long long d) const {
    const TomlValue* v = find(k);
    if (v && v->kind == TomlValue::INT) return v->i;
    if (v && v->kind == TomlValue::FLOAT && std::floor(v->f) == v->f) return (long long)v->f;
    return d;
  }
  std::string str_or(const std::string& k, const std::string& d) const {
    const TomlValue* v = find(k);
    return (v && v->kind == TomlValue::STR) ? v->s : d;
  }
  bool bool_or(const std::string& k, bool d) const {
    const TomlValue* v = find(k);
    return (v && v->kind == TomlValue::BOOL) ? v->b : d;
  }

 private:
  std::map<std::string, TomlValue> values_;
  std::string text_;
  size_t p_ = 0;
  int line_ = 1;

  [[noreturn]] void error(const std::string& what) const {
    throw ConfigError("config line " + std::to_string(line_) + ": " + what);
  }
  bool at_end() const { return p_ >= text_.size(); }
  char peek() const { return at_end() ? '\0' : text_[p_]; }
  void skip_space() {  // spaces and tabs on the current line
    while (!at_end() && (text_[p_] == ' ' || text_[p_] == '\t' || text_[p_] == '\r')) ++p_;
  }
  void skip_comment() {
    if (peek() == '#')
      while (!at_end() && text_[p_] != '\n') ++p_;
  }
  void skip_blank() {  // spaces, comments and newlines (inside arrays)
    for (;;) {
      skip_space();
      skip_comment();
      if (peek() == '\n') {
        ++p_;
        ++line_;
        continue;
      }
      return;
    }
  }
  void end_of_line() {
    skip_space();
    skip_comment();
    if (at_end()) return;
    if (peek() != '\n') error("unexpected text after a value");
    ++p_;
    ++line_;
  }
  std::string bare_key() {
    const size_t s = p_;
    while (!at_end() && (std::isalnum((unsigned char)peek()) || peek() == '_' || peek() == '-')) ++p_;
    if (p_ == s) error("expected a key");
    return text_.substr(s, p_ - s);
  }
  std::string dotted_key() {
    std::string k = bare_key();
    skip_space();
    while (peek() == '.') {
      ++p_;
      skip_space();
      k += "." + bare_key();
      skip_space();
    }
    return k;
  }
  TomlValue value() {
    TomlValue v;
    const char c = peek();
    if (c == '"') {
      ++p_;
      v.kind = TomlValue::STR;
      while (!at_end() && peek() != '"' && peek() != '\n') {
        if (peek() == '\\' && p_ + 1 < text_.size()) {
          const char e = text_[p_ + 1];
          v.s += (e == 'n') ? '\n' : (e == 't') ? '\t' : e;
          p_ += 2;
        } else {
          v.s += text_[p_++];
        }
      }
      if (peek() != '"') error("unterminated string");
      ++p_;
      return v;
    }
    if (c == '[') {
      ++p_;
      v.kind = TomlValue::ARRAY;
      skip_blank();
      while (peek() != ']') {
        if (at_end()) error("unterminated array");
        v.items.push_back(value());
        skip_blank();
        if (peek() == ',') {
          ++p_;
          skip_blank();
        } else if (peek() != ']') {
          error("expected ',' or ']' in an array");
        }
      }
      ++p_;
      return v;
    }
    const size_t s = p_;
    while (!at_end() && peek() != ',' && peek() != ']' && peek() != '\n' && peek() != '#' && peek() != ' ' &&
           peek() != '\t' && peek() != '\r')
      ++p_;
    std::string tok = text_.substr(s, p_ - s);
    if (tok == "true" || tok == "false") {
      v.kind = TomlValue::BOOL;
      v.b = (tok == "true");
      return v;
    }
    std::string num;
    for (char ch : tok)
      if (ch != '_') num += ch;
    if (num.empty()) error("expected a value");
    size_t used = 0;
    const bool is_float = num.find_first_of(".eE") != std::string::npos || num == "inf" || num == "+inf" ||
                          num == "-inf" || num == "nan";
    try {
      if (is_float) {
        v.kind = TomlValue::FLOAT;
        v.f = std::stod(num, &used);
      } else {
        v.kind = TomlValue::INT;
        v.i = std::stoll(num, &used, 10);
      }
    } catch (const std::exception&) {
      error("bad value '" + tok + "'");
    }
    if (used != num.size()) error("bad value '" + tok + "'");
    return v;
  }
  void parse(const std::string& text) {
    text_ = text;
    std::string table;
    for (;;) {
      skip_blank();
      if (at_end()) return;
      if (peek() == '[') {
        ++p_;
        skip_space();
        table = dotted_key();
        if (peek() != ']') error("expected ']' after a table name");
        ++p_;
        end_of_line();
        continue;
      }
      const std::string k = dotted_key();
      if (peek() != '=') error("expected '=' after key '" + k + "'");
      ++p_;
      skip_space();
      const std::string full = table.empty() ? k : table + "." + k;
      if (values_.count(full)) error("key '" + full + "' defined twice");
      values_[full] = value();
      end_of_line();
    }
  }
};

// ---- DqmcInitializer::parse_toml_config -------------------------------------
// MeasureHandler::ObservableAll (src/measure/measure_handler.cpp), equal-time then dynamic
inline const std::vector<std::string>& equaltime_observables() {
  static const std::vector<std::string> v = {
      "filling_number", "double_occupancy", "kinetic_energy", "momentum_distribution", "local_spin_corr",
      "spin_density_structure_factor", "charge_density_structure_factor", "s_wave_pairing_corr"};
  return v;
}
inline const std::vector<std::string>& dynamic_observables() {
  static const std::vector<std::string> v = {"greens_functions", "density_of_states", "superfluid_stiffness",
                                             "dynamic_spin_susceptibility"};
  return v;
}

struct RunConfig {
  std::string model = "RepulsiveHubbard";
  double hopping_t = 1.0, onsite_u = 4.0, chemical_potential = 0.0;
  std::string lattice = "Square";
  std::vector<int> cell = {4, 4};
  std::string momentum, momentum_list;
  bool checkerboard = false;
  double beta = 4.0;
  int time_size = 80, stabilization_pace = 10;
  int sweeps_warmup = 512, bin_num = 20, bin_size = 100, sweeps_between_bins = 20;
  std::vector<std::string> observables;

  int L() const { return cell[0]; }
  int dim() const { return (int)cell.size(); }
  bool has(const std::string& o) const {
    for (auto& x : observables)
      if (x == o) return true;
    return false;
  }
  bool equaltime() const {
    for (auto& o : equaltime_observables())
      if (has(o)) return true;
    return false;
  }
  bool dynamic() const {
    for (auto& o : dynamic_observables())
      if (has(o)) return true;
    return false;
  }
};

inline RunConfig parse_config(const std::string& text) {
  const Toml t(text);
  RunConfig c;
  c.model = t.str_or("Model.type", "RepulsiveHubbard");
  if (c.model != "RepulsiveHubbard" && c.model != "AttractiveHubbard")
    throw ConfigError("undefined model type '" + c.model + "'");
  c.hopping_t = t.number_or("Model.Params.hopping_t", 1.0);
  c.onsite_u = t.number_or("Model.Params.onsite_u", 4.0);
  c.chemical_potential = t.number_or("Model.Params.chemical_potential", 0.0);
  c.lattice = t.str_or("Lattice.type", "Square");
  int dim = 0;
  std::string what, count;
  if (c.lattice == "Square") {
    dim = 2, what = "2d square", count = "two";
  } else if (c.lattice == "Cubic") {
    dim = 3, what = "3d cubic", count = "three";
  } else {  // Honeycomb: left unimplemented by the reference
    throw ConfigError("undefined lattice type '" + c.lattice + "'");
  }
  const TomlValue* cell = t.find("Lattice.cell");
  const std::string cell_msg =
      "the input cell of " + what + " lattice should be a vector containing " + count + " positive integers";
  if (!cell || cell->kind != TomlValue::ARRAY || (int)cell->items.size() != dim) throw ConfigError(cell_msg);
  c.cell.clear();
  for (auto& v : cell->items) {
    if (v.kind != TomlValue::INT || v.i < 1) throw ConfigError(cell_msg);
    c.cell.push_back((int)v.i);
  }
  for (int v : c.cell)  // Square/Cubic::set_lattice_params assert equal sides
    if (v != c.cell[0]) throw ConfigError("the " + what + " lattice must have equal sides");
  c.momentum = t.str_or("Lattice.momentum", "");
  c.momentum_list = t.str_or("Lattice.momentum_list", "");
  c.checkerboard = t.bool_or("CheckerBoard.whether_or_not", false);
  if (c.checkerboard && c.lattice != "Square")
    throw ConfigError("the checkerboard method is currently only implemented for 2d square lattice");
  c.beta = t.number_or("MonteCarlo.beta", 4.0);
  c.time_size = (int)t.number_or("MonteCarlo.time_size", 80);  // read as a double (dqmc_initializer.cpp:190)
  c.stabilization_pace = (int)t.int_or("MonteCarlo.stabilization_pace", 10);
  c.sweeps_warmup = (int)t.int_or("Measure.sweeps_warmup", 512);
  c.bin_num = (int)t.int_or("Measure.bin_num", 20);
  c.bin_size = (int)t.int_or("Measure.bin_size", 100);
  c.sweeps_between_bins = (int)t.int_or("Measure.sweeps_between_bins", 20);
  const TomlValue* obs = t.find("Measure.observables");
  if (!obs || obs->kind != TomlValue::ARRAY) throw ConfigError("undefined observables, please check the config");
  for (auto& v : obs->items) {
    if (v.kind != TomlValue::STR) throw ConfigError("undefined observables, please check the config");
    c.observables.push_back(v.s);
  }
  if (c.observables.size() == 1 && (c.observables[0] == "all" || c.observables[0] == "All")) {
    c.observables = equaltime_observables();
    for (auto& o : dynamic_observables()) c.observables.push_back(o);
  } else if (c.observables.size() == 1 && (c.observables[0] == "none" || c.observables[0] == "None")) {
    c.observables.clear();
  }
  for (auto& o : c.observables) {
    bool known = false;
    for (auto& e : equaltime_observables()) known = known || o == e;
    for (auto& e : dynamic_observables()) known = known || o == e;
    if (!known) throw ConfigError("unsupported observable '" + o + "'");
  }
  if (c.lattice != "Square") {  // a square-lattice observable (dqmc_initializer.cpp:233-237)
    std::vector<std::string> kept;
    for (auto& o : c.observables)
      if (o != "superfluid_stiffness") kept.push_back(o);
    c.observables = kept;
  }
  return c;
}

}  // namespace dqmc_app
