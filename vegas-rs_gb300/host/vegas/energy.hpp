// energy.hpp -- the energy terms of vegas (src/energy.rs:41-290) as
// descriptions the GPU engine evaluates.
//
// Each term knows how to write itself into a vg_hamiltonian_desc; Compound
// nests like the reference's, and hamiltonian(...) flattens a list of terms
// the way the hamiltonian! macro does (src/energy.rs:273-290).  A single
// term keeps its own total_energy (Exchange halves the bond sum, Anisotropy
// drops K, Zeeman negates); any Compound reports sum_i energy(i)
// (src/energy.rs:55-59, :248-257).  The same semantics are applied by the
// engine when it turns per-sweep lattice sums into totals.
#pragma once

#include <optional>
#include <utility>

#include "error.hpp"
#include "lattice.hpp"
#include "state.hpp"
#include "vegas_gpu.h"

namespace vegas {

// Gauge (src/energy.rs:62-80)
struct Gauge {
  double value = 0.0;
  explicit Gauge(double v) : value(v) {}
  void describe(vg_hamiltonian_desc& d) const {
    d.has_gauge = 1;
    d.gauge += value;
  }
  std::optional<Lattice> lattice() const { return std::nullopt; }
};

// UniaxialAnisotropy (src/energy.rs:82-121)
template <typename S>
struct UniaxialAnisotropy {
  S reference;
  double strength;
  UniaxialAnisotropy(S s, double k) : reference(s), strength(k) {}
  void describe(vg_hamiltonian_desc& d) const {
    if (d.has_anisotropy && (d.anisotropy_axis[0] != reference.sx() || d.anisotropy_axis[1] != reference.sy() ||
                             d.anisotropy_axis[2] != reference.sz()))
      throw NotImplementedError();
    d.has_anisotropy = 1;
    d.anisotropy += strength;
    d.anisotropy_axis[0] = reference.sx();
    d.anisotropy_axis[1] = reference.sy();
    d.anisotropy_axis[2] = reference.sz();
  }
  std::optional<Lattice> lattice() const { return std::nullopt; }
};

// Zeeman (src/energy.rs:123-161): per site +|B| (s . orientation).
template <typename S>
struct Zeeman {
  void describe(vg_hamiltonian_desc& d) const {
    d.has_zeeman = 1;
    d.zeeman_sign += 1.0;
  }
  std::optional<Lattice> lattice() const { return std::nullopt; }
};

// Exchange::from_lattice (src/energy.rs:163-214)
struct Exchange {
  double J;
  Lattice lat;
  static Exchange from_lattice(double exchange, const Lattice& l) { return Exchange{exchange, l}; }
  void describe(vg_hamiltonian_desc& d) const {
    d.has_exchange = 1;
    d.exchange += J;
  }
  std::optional<Lattice> lattice() const { return lat; }
};

// Cubic anisotropy: an extension with no reference counterpart, per site
// -Kc (sx^4 + sy^4 + sz^4) (Kc > 0 favours the cube axes).
struct CubicAnisotropy {
  double Kc;
  explicit CubicAnisotropy(double k) : Kc(k) {}
  void describe(vg_hamiltonian_desc& d) const {
    d.has_cubic = 1;
    d.cubic += Kc;
  }
  std::optional<Lattice> lattice() const { return std::nullopt; }
};

// Compound (src/energy.rs:216-257)
template <typename A, typename B>
struct Compound {
  A a;
  B b;
  void describe(vg_hamiltonian_desc& d) const {
    a.describe(d);
    b.describe(d);
  }
  std::optional<Lattice> lattice() const {
    auto la = a.lattice();
    return la ? la : b.lattice();
  }
};

template <typename T>
struct is_compound : std::false_type {};
template <typename A, typename B>
struct is_compound<Compound<A, B>> : std::true_type {};

// hamiltonian(a, b, c, ...) == Compound(Compound(a, b), c) ...
template <typename A>
A hamiltonian(A a) {
  return a;
}
template <typename A, typename B, typename... R>
auto hamiltonian(A a, B b, R... rest) {
  return hamiltonian(Compound<A, B>{a, b}, rest...);
}

template <typename H>
vg_hamiltonian_desc describe(const H& h) {
  vg_hamiltonian_desc d{};
  h.describe(d);
  d.compound = is_compound<H>::value ? 1 : 0;
  return d;
}

}  // namespace vegas
