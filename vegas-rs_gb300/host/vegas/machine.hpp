// machine.hpp -- Machine (src/machine.rs:43-126) over the GPU integrator.
//
// The reference clones the state and calls Integrator::step once per sweep,
// then every instrument's after_step (src/machine.rs:91-101).  Here the
// state stays in device memory: run(n) issues vg_sweeps in chunks, receives
// the per-sweep total energy and |M| computed on the device, and replays
// them into the instruments sweep by sweep.  A chunk ends wherever an
// instrument needs the spins themselves (StateSensor), so the state it sees
// is the state after exactly that sweep.
//
// The integrators are the GPU counterparts of MetropolisIntegrator
// (random proposal, src/integrator.rs:56-92), MetropolisFlipIntegrator
// (flip proposal, :99-138) and WolffIntegrator (cluster steps, :140-230);
// their RNG is the engine's counter-based Philox
// stream keyed by (seed, replica, sweep), so relax_for / measure_for take no
// RNG argument.
#pragma once

#include <algorithm>
#include <memory>
#include <vector>

#include "energy.hpp"
#include "error.hpp"
#include "instrument.hpp"
#include "lattice.hpp"
#include "state.hpp"
#include "thermostat.hpp"
#include "vegas_gpu.h"

namespace vegas {

struct GpuIntegrator {
  int proposal;
  uint64_t seed = 0;
  uint32_t replica = 0;
  int path = VG_PATH_AUTO;
  int precision = VG_FP32;
  bool cluster = false;  // Wolff cluster steps (vg_wolff_steps) instead of Metropolis sweeps
};

struct MetropolisIntegrator : GpuIntegrator {
  explicit MetropolisIntegrator(uint64_t seed = 0) : GpuIntegrator{VG_PROPOSE_RANDOM, seed} {}
};

struct MetropolisFlipIntegrator : GpuIntegrator {
  explicit MetropolisFlipIntegrator(uint64_t seed = 0) : GpuIntegrator{VG_PROPOSE_FLIP, seed} {}
};

// WolffIntegrator (src/integrator.rs:140-230): one cluster flip per step,
// bond probability from the Hamiltonian's exchange constant; Ising only.
struct WolffIntegrator : GpuIntegrator {
  explicit WolffIntegrator(uint64_t seed = 0) : GpuIntegrator{VG_PROPOSE_FLIP, seed} { cluster = true; }
};

template <typename H, typename I, typename S>
class Machine {
 public:
  using Instruments = std::vector<std::unique_ptr<Instrument<S>>>;

  Machine(Thermostat<S> thermostat, H hamiltonian, I integrator, Instruments instruments, const State<S>& state)
      : thermostat_(thermostat), hamiltonian_(hamiltonian), integrator_(integrator),
        instruments_(std::move(instruments)) {
    auto lat = hamiltonian_.lattice();
    // without an exchange term the geometry is irrelevant: a chain of N sites
    const Lattice l = lat ? *lat : Lattice::sc(1.0).expand_x((int)state.len()).drop_y().drop_z();
    if (l.sites_len() != state.len()) throw VegasError("state size does not match the lattice");
    const vg_hamiltonian_desc hd = describe(hamiltonian_);
    vg_options o;
    check(vg_options_default(S::kind, &o));
    o.proposal = integrator_.proposal;
    o.path = integrator_.path;
    o.precision = integrator_.precision;
    o.replica = integrator_.replica;
    check(vg_ctx_create_ex(&l.desc(), &hd, &o, integrator_.seed, &ctx_));
    n_ = state.len();
    set_state(state);
    push_thermostat();
  }
  ~Machine() {
    if (ctx_) vg_ctx_destroy(ctx_);
  }
  Machine(const Machine&) = delete;
  Machine& operator=(const Machine&) = delete;

  const Thermostat<S>& thermostat() const { return thermostat_; }
  void set_thermostat(Thermostat<S> t) {
    thermostat_ = t;
    push_thermostat();
  }

  void relax_for(size_t steps) {
    for (auto& i : instruments_) i->on_relax_start(thermostat_, n_);
    run(steps);
    for (auto& i : instruments_) i->on_relax_end();
  }
  void measure_for(size_t steps) {
    for (auto& i : instruments_) i->on_measure_start(thermostat_, n_);
    run(steps);
    for (auto& i : instruments_) i->on_measure_end();
  }

  State<S> state() const {
    std::vector<typename S::Raw> raw(n_ * S::raw_per_site);
    check(vg_get_state(ctx_, raw.data(), (int64_t)n_), ctx_);
    return State<S>::from_raw(raw);
  }
  void set_state(const State<S>& s) {
    const auto raw = s.to_raw();
    check(vg_set_state(ctx_, raw.data(), (int64_t)n_), ctx_);
  }
  vg_ctx* context() const { return ctx_; }

  // Hamiltonian::energy(thermostat, state, i) of every site of the current
  // state (src/energy.rs:45-52), and Hamiltonian::total_energy
  // (src/energy.rs:55-59 with each term's own total), on the device.
  std::vector<double> site_energies() const {
    std::vector<double> e(n_);
    check(vg_site_energies(ctx_, e.data(), (int64_t)n_), ctx_);
    return e;
  }
  double energy(size_t index) const {
    if (index >= n_) throw VegasError("site index out of range");
    return site_energies()[index];
  }
  double total_energy() const {
    double e = 0.0;
    check(vg_total_energy(ctx_, &e), ctx_);
    return e;
  }

 private:
  void push_thermostat() {
    const auto b = thermostat_.field().b_hat();
    check(vg_set_thermostat(ctx_, thermostat_.temperature(), b.data(), thermostat_.field().magnitude()), ctx_);
  }

  void run(size_t steps) {
    bool measure = false;
    size_t freq = 0;
    for (auto& i : instruments_) {
      measure = measure || i->wants_observables();
      const size_t f = i->state_frequency();
      if (f) freq = freq ? std::min(freq, f) : f;
    }
    constexpr size_t kMaxChunk = 1 << 16;
    std::vector<double> E, M;
    size_t t = 0;
    while (t < steps) {
      // next sweep index (>= t) after which the spins are needed
      size_t stop = steps - 1;
      if (freq) stop = std::min(stop, ((t + freq - 1) / freq) * freq);
      const size_t chunk = std::min(stop - t + 1, kMaxChunk);
      if (measure) {
        E.resize(chunk);
        M.resize(chunk);
      }
      if (integrator_.cluster)
        check(vg_wolff_steps(ctx_, chunk, measure ? 1 : 0, measure ? E.data() : nullptr, measure ? M.data() : nullptr),
              ctx_);
      else
        check(vg_sweeps(ctx_, chunk, measure ? 1 : 0, measure ? E.data() : nullptr, measure ? M.data() : nullptr),
              ctx_);
      for (size_t k = 0; k < chunk; ++k) {
        const bool last = k + 1 == chunk;
        StepView<S> v{measure ? E[k] : 0.0, measure ? M[k] : 0.0, n_, [this, last]() {
                        if (!last) throw VegasError("internal: state requested mid-chunk");
                        return state();
                      }};
        for (auto& i : instruments_) i->after_step(v);
      }
      t += chunk;
    }
  }

  Thermostat<S> thermostat_;
  H hamiltonian_;
  I integrator_;
  Instruments instruments_;
  vg_ctx* ctx_ = nullptr;
  size_t n_ = 0;
};

}  // namespace vegas
