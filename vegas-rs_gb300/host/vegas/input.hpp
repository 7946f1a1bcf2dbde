// input.hpp -- the TOML input of `vegas run` (src/input.rs:1-368) driving the
// GPU engine: model, algorithm, optional exchange, sample (unit cell, size,
// per-axis PBC), stages (Relax / CoolDown / Hysteresis) and outputs.
//
// The parser reads the subset of TOML the input uses (tables, arrays of
// tables, strings, numbers, booleans, comments).  Input::run mirrors
// src/input.rs:264-294 and :347-367: Compound(Exchange::from_lattice(J),
// Zeeman), a random initial state, T = 2.8 with zero field, StatSensor on
// stdout plus the optional observable / state outputs, then each stage in
// order.  Ising uses the flip proposal and Heisenberg the random proposal,
// as the reference picks; Wolff runs the GPU cluster steps for Ising and is
// not implemented for Heisenberg (src/input.rs:354-365).
#pragma once

#include <cctype>
#include <cstdio>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <variant>
#include <vector>

#include "energy.hpp"
#include "error.hpp"
#include "instrument.hpp"
#include "lattice.hpp"
#include "machine.hpp"
#include "program.hpp"

namespace vegas {

class TomlError : public VegasError {
 public:
  explicit TomlError(const std::string& m) : VegasError("toml deserialization error: " + m) {}
};

// flat view of a TOML document: "a.b.c" -> raw value; arrays of tables are
// kept as a list of flat tables.
struct TomlDoc {
  std::map<std::string, std::string> values;
  std::map<std::string, std::vector<std::map<std::string, std::string>>> arrays;

  static std::string trim(const std::string& s) {
    size_t a = 0, b = s.size();
    while (a < b && std::isspace((unsigned char)s[a])) ++a;
    while (b > a && std::isspace((unsigned char)s[b - 1])) --b;
    return s.substr(a, b - a);
  }

  static TomlDoc parse(const std::string& text) {
    TomlDoc d;
    std::istringstream in(text);
    std::string line, table;
    std::map<std::string, std::string>* target = nullptr;
    int lineno = 0;
    while (std::getline(in, line)) {
      ++lineno;
      // strip comments outside strings
      bool q = false;
      for (size_t i = 0; i < line.size(); ++i) {
        if (line[i] == '"') q = !q;
        if (line[i] == '#' && !q) {
          line = line.substr(0, i);
          break;
        }
      }
      line = trim(line);
      if (line.empty()) continue;
      if (line.rfind("[[", 0) == 0) {
        if (line.size() < 4 || line.substr(line.size() - 2) != "]]") throw TomlError("bad header at line " + std::to_string(lineno));
        table = trim(line.substr(2, line.size() - 4));
        d.arrays[table].emplace_back();
        target = &d.arrays[table].back();
        continue;
      }
      if (line[0] == '[') {
        if (line.back() != ']') throw TomlError("bad header at line " + std::to_string(lineno));
        table = trim(line.substr(1, line.size() - 2));
        target = nullptr;
        continue;
      }
      const size_t eq = line.find('=');
      if (eq == std::string::npos) throw TomlError("expected key = value at line " + std::to_string(lineno));
      const std::string key = trim(line.substr(0, eq)), val = trim(line.substr(eq + 1));
      if (target) (*target)[key] = val;
      else d.values[table.empty() ? key : table + "." + key] = val;
    }
    return d;
  }

  static bool has(const std::map<std::string, std::string>& m, const std::string& k) { return m.count(k) > 0; }
  static std::string str(const std::map<std::string, std::string>& m, const std::string& k) {
    auto it = m.find(k);
    if (it == m.end()) throw TomlError("missing field `" + k + "`");
    const std::string& v = it->second;
    if (v.size() < 2 || v.front() != '"' || v.back() != '"') throw TomlError("invalid type for `" + k + "`: expected a string");
    return v.substr(1, v.size() - 2);
  }
  static double num(const std::map<std::string, std::string>& m, const std::string& k) {
    auto it = m.find(k);
    if (it == m.end()) throw TomlError("missing field `" + k + "`");
    try {
      size_t pos = 0;
      const double v = std::stod(it->second, &pos);
      if (pos != it->second.size()) throw std::invalid_argument("trailing");
      return v;
    } catch (const std::exception&) {
      throw TomlError("invalid type for `" + k + "`: expected a number");
    }
  }
  static size_t count(const std::map<std::string, std::string>& m, const std::string& k) {
    const double v = num(m, k);
    if (v < 0 || v != (double)(size_t)v) throw TomlError("invalid value for `" + k + "`: expected an unsigned integer");
    return (size_t)v;
  }
  static bool boolean(const std::map<std::string, std::string>& m, const std::string& k) {
    auto it = m.find(k);
    if (it == m.end()) throw TomlError("missing field `" + k + "`");
    if (it->second == "true") return true;
    if (it->second == "false") return false;
    throw TomlError("invalid type for `" + k + "`: expected a boolean");
  }
};

struct StageSpec {
  std::variant<Relax, CoolDown, HysteresisLoop> program;
};

struct Input {
  std::string model = "Ising";          // Model (src/input.rs:19-26)
  std::string algorithm = "Metropolis"; // Algorithm (src/input.rs:28-35)
  bool has_exchange = false;
  double exchange = 1.0;
  std::string unitcell = "sc";
  int size[3] = {1, 1, 1};
  bool pbc[3] = {true, true, true};
  std::vector<StageSpec> stages;
  bool has_output = false;
  std::string observables;              // empty = none
  std::string state_path;               // empty = none
  size_t state_frequency = 1000;

  static Input parse(const std::string& text) {
    const TomlDoc d = TomlDoc::parse(text);
    Input in;
    in.model = TomlDoc::str(d.values, "model");
    in.algorithm = TomlDoc::str(d.values, "algorithm");
    if (in.model != "Ising" && in.model != "Heisenberg") throw TomlError("unknown variant `" + in.model + "`");
    if (in.algorithm != "Metropolis" && in.algorithm != "Wolff") throw TomlError("unknown variant `" + in.algorithm + "`");
    if (TomlDoc::has(d.values, "exchange")) {
      in.has_exchange = true;
      in.exchange = TomlDoc::num(d.values, "exchange");
    }
    if (TomlDoc::has(d.values, "sample.unitcell.path")) throw NotImplementedError();  // UnitCell::Path is todo!()
    in.unitcell = TomlDoc::str(d.values, "sample.unitcell.name");
    if (in.unitcell != "sc" && in.unitcell != "bcc" && in.unitcell != "fcc")
      throw TomlError("unknown variant `" + in.unitcell + "`");
    const char* ax[3] = {"x", "y", "z"};
    for (int a = 0; a < 3; ++a) {
      in.size[a] = (int)TomlDoc::count(d.values, std::string("sample.size.") + ax[a]);
      in.pbc[a] = TomlDoc::boolean(d.values, std::string("sample.pbc.") + ax[a]);
    }
    auto st = d.arrays.find("stages");
    if (st == d.arrays.end()) throw TomlError("missing field `stages`");
    for (const auto& t : st->second) {
      const std::string p = TomlDoc::str(t, "program");
      if (p == "Relax") {
        in.stages.push_back({Relax(TomlDoc::count(t, "steps"), TomlDoc::num(t, "temperature"))});
      } else if (p == "CoolDown") {
        in.stages.push_back({CoolDown(TomlDoc::num(t, "max_temperature"), TomlDoc::num(t, "min_temperature"),
                                      TomlDoc::num(t, "cool_rate"), TomlDoc::count(t, "relax"),
                                      TomlDoc::count(t, "steps"))});
      } else if (p == "Hysteresis") {
        in.stages.push_back({HysteresisLoop(TomlDoc::count(t, "steps"), TomlDoc::count(t, "relax"),
                                            TomlDoc::num(t, "temperature"), TomlDoc::num(t, "max_field"),
                                            TomlDoc::num(t, "field_step"))});
      } else {
        throw TomlError("unknown variant `" + p + "`");
      }
    }
    for (const auto& kv : d.values)
      if (kv.first.rfind("output.", 0) == 0) in.has_output = true;
    if (TomlDoc::has(d.values, "output.observables")) in.observables = TomlDoc::str(d.values, "output.observables");
    if (TomlDoc::has(d.values, "output.state.path")) {
      in.state_path = TomlDoc::str(d.values, "output.state.path");
      in.state_frequency = TomlDoc::count(d.values, "output.state.frequency");
    }
    return in;
  }

  static std::string default_text() {  // Input::default (src/input.rs:178-192)
    return "model = \"Ising\"\nalgorithm = \"Metropolis\"\n\n[sample.unitcell]\nname = \"sc\"\n\n"
           "[sample.size]\nx = 1\ny = 1\nz = 1\n\n[sample.pbc]\nx = true\ny = true\nz = true\n\n"
           "[[stages]]\nprogram = \"Relax\"\nsteps = 1000\ntemperature = 3.0\n\n"
           "[[stages]]\nprogram = \"CoolDown\"\nmax_temperature = 3.0\nmin_temperature = 0.05\n"
           "cool_rate = 0.1\nrelax = 1000\nsteps = 20000\n\n"
           "[output]\nobservables = \"./output.parquet\"\n\n[output.state]\npath = \"./state.parquet\"\n"
           "frequency = 1000\n";
  }

  Lattice lattice() const {
    Lattice l = unitcell == "sc" ? Lattice::sc(1.0) : unitcell == "bcc" ? Lattice::bcc(1.0) : Lattice::fcc(1.0);
    l = l.expand(size[0], size[1], size[2]);
    if (!pbc[0]) l = l.drop_x();
    if (!pbc[1]) l = l.drop_y();
    if (!pbc[2]) l = l.drop_z();
    return l;
  }

  template <typename S>
  typename Machine<Compound<Exchange, Zeeman<S>>, GpuIntegrator, S>::Instruments instruments(FILE* out) const {
    typename Machine<Compound<Exchange, Zeeman<S>>, GpuIntegrator, S>::Instruments v;
    v.push_back(std::make_unique<StatSensor<S>>(out));
    if (!observables.empty()) v.push_back(std::make_unique<ObservableSensor<S>>(observables));
    if (!state_path.empty()) v.push_back(std::make_unique<StateSensor<S>>(state_path, state_frequency));
    return v;
  }

  template <typename S>
  void run_with_spin(GpuIntegrator integrator, FILE* out) const {
    const Lattice l = lattice();
    auto H = hamiltonian(Exchange::from_lattice(has_exchange ? exchange : 1.0, l), Zeeman<S>());
    Machine<decltype(H), GpuIntegrator, S> m(Thermostat<S>(2.8, Field<S>::zero()), H, integrator, instruments<S>(out),
                                            State<S>::up_with_size(l.sites_len()));
    check(vg_init_random(m.context()), m.context());  // State::rand_with_size
    for (const auto& st : stages) std::visit([&](const auto& p) { p.run(m); }, st.program);
  }

  void run(uint64_t seed, FILE* out = stdout) const {
    if (algorithm == "Wolff") {
      if (model != "Ising") throw NotImplementedError();
      run_with_spin<IsingSpin>(WolffIntegrator(seed), out);
      return;
    }
    if (model == "Ising") run_with_spin<IsingSpin>(MetropolisFlipIntegrator(seed), out);
    else run_with_spin<HeisenbergSpin>(MetropolisIntegrator(seed), out);
  }
};

}  // namespace vegas
