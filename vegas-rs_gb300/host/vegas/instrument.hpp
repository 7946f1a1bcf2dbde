// instrument.hpp -- instruments hooked into the machine (src/instrument.rs).
//
// The hooks are the reference's (on_relax_start/end, on_measure_start/end,
// after_step).  after_step receives a StepView: the sweep's total energy and
// |M| computed on the device with the Hamiltonian's total-energy semantics
// (what the reference's instruments compute from the state themselves,
// src/instrument.rs:133-141, :254-262) and a callback that copies the state
// back when an instrument needs the spins (StateSensor).
//
// Output files: Parquet with the reference's schemas (src/output.rs:37-46,
// :126-136), through "<path>.parquet.tmp" renamed on close as the reference
// does (src/output.rs:101-112, :189-200); see parquet.hpp.
#pragma once

#include <cstdio>
#include <functional>
#include <memory>
#include <string>

#include "accumulator.hpp"
#include "error.hpp"
#include "parquet.hpp"
#include "state.hpp"
#include "thermostat.hpp"

namespace vegas {

template <typename S>
struct StepView {
  double energy;
  double magnetization;
  size_t n;
  std::function<State<S>()> state;  // device -> host copy on demand
};

template <typename S>
class Instrument {
 public:
  virtual ~Instrument() = default;
  virtual void on_relax_start(const Thermostat<S>&, size_t /*n*/) {}
  virtual void on_relax_end() {}
  virtual void on_measure_start(const Thermostat<S>&, size_t /*n*/) {}
  virtual void on_measure_end() {}
  virtual void after_step(const StepView<S>&) {}
  // True if after_step needs E / |M| for this sweep (lets the machine skip
  // the per-sweep reduction when no instrument listens).
  virtual bool wants_observables() const { return false; }
  // Sweeps (within the current relax/measure run) at which the state is read.
  virtual size_t state_frequency() const { return 0; }
};

// StatSensor (src/instrument.rs:98-141): one line per measure run with
// T |B| <E> Var(E)/(N T^2) <|M|> Var(|M|)/(N T) U4, 16 decimals.
template <typename S>
class StatSensor : public Instrument<S> {
 public:
  explicit StatSensor(FILE* out) : out_(out) {}
  void on_measure_start(const Thermostat<S>& t, size_t n) override {
    thermostat_ = std::make_unique<Thermostat<S>>(t);
    n_ = n;
  }
  void on_measure_end() override {
    if (thermostat_) {
      const double T = thermostat_->temperature();
      std::fprintf(out_, "%.16f %.16f %.16f %.16f %.16f %.16f %.16f\n", T, thermostat_->field().magnitude(),
                   energy_.mean(), energy_.variance() / ((double)n_ * T * T), magnetization_.mean(),
                   magnetization_.variance() / ((double)n_ * T), magnetization_.binder_cumulant());
      std::fflush(out_);
    }
    thermostat_.reset();
    n_ = 0;
    energy_ = Accumulator();
    magnetization_ = Accumulator();
  }
  void after_step(const StepView<S>& v) override {
    if (!thermostat_) return;
    energy_.collect(v.energy);
    magnetization_.collect(v.magnetization);
  }
  bool wants_observables() const override { return thermostat_ != nullptr; }

 private:
  FILE* out_;
  std::unique_ptr<Thermostat<S>> thermostat_;
  size_t n_ = 0;
  Accumulator energy_, magnetization_;
};

// ObservableSensor (src/instrument.rs:144-263): per-sweep rows during relax
// and measure runs; schema of src/output.rs:37-46.
template <typename S>
class ObservableSensor : public Instrument<S> {
 public:
  explicit ObservableSensor(const std::string& path)
      : io_(path, parquet::with_extension(path, "parquet.tmp"),
            {{"relax", parquet::Type::Bool},
             {"stage", parquet::Type::UInt64},
             {"step", parquet::Type::UInt64},
             {"n", parquet::Type::UInt64},
             {"temperature", parquet::Type::Float64},
             {"field", parquet::Type::Float64},
             {"energy", parquet::Type::Float64},
             {"magnetization", parquet::Type::Float64}}) {}
  void on_relax_start(const Thermostat<S>& t, size_t n) override { start(t, n, true); }
  void on_relax_end() override { finish(); }
  void on_measure_start(const Thermostat<S>& t, size_t n) override { start(t, n, false); }
  void on_measure_end() override { finish(); }
  void after_step(const StepView<S>& v) override {
    if (!thermostat_) return;
    io_.add_bool(0, relax_);
    io_.add_u64(1, stage_);
    io_.add_u64(2, step_++);
    io_.add_u64(3, n_);
    io_.add_f64(4, thermostat_->temperature());
    io_.add_f64(5, thermostat_->field().magnitude());
    io_.add_f64(6, v.energy);
    io_.add_f64(7, v.magnetization);
    io_.end_row();
  }
  bool wants_observables() const override { return thermostat_ != nullptr; }

 private:
  void start(const Thermostat<S>& t, size_t n, bool relax) {
    thermostat_ = std::make_unique<Thermostat<S>>(t);
    n_ = n;
    relax_ = relax;
    step_ = 0;
  }
  void finish() {
    ++stage_;
    thermostat_.reset();
  }
  parquet::Writer io_;
  std::unique_ptr<Thermostat<S>> thermostat_;
  size_t n_ = 0, stage_ = 0, step_ = 0;
  bool relax_ = false;
};

// StateSensor (src/instrument.rs:265-351): the whole state every `frequency`
// sweeps; schema of src/output.rs:126-136.
template <typename S>
class StateSensor : public Instrument<S> {
 public:
  StateSensor(const std::string& path, size_t frequency)
      : io_(path, parquet::with_extension(path, "parquet.tmp"),
            {{"relax", parquet::Type::Bool},
             {"stage", parquet::Type::UInt64},
             {"step", parquet::Type::UInt64},
             {"temperature", parquet::Type::Float64},
             {"field", parquet::Type::Float64},
             {"id", parquet::Type::UInt64},
             {"sx", parquet::Type::Float64},
             {"sy", parquet::Type::Float64},
             {"sz", parquet::Type::Float64}}),
        frequency_(frequency ? frequency : 1) {}
  void on_relax_start(const Thermostat<S>& t, size_t) override {
    relax_ = 1;
    thermostat_ = std::make_unique<Thermostat<S>>(t);
  }
  void on_relax_end() override { end(); }
  void on_measure_start(const Thermostat<S>& t, size_t) override {
    relax_ = 0;
    thermostat_ = std::make_unique<Thermostat<S>>(t);
  }
  void on_measure_end() override { end(); }
  void after_step(const StepView<S>& v) override {
    if (step_ % frequency_ == 0 && relax_ >= 0 && thermostat_) {
      const State<S> st = v.state();
      for (size_t i = 0; i < st.len(); ++i) {
        const S& s = st.at(i);
        io_.add_bool(0, relax_ == 1);
        io_.add_u64(1, stage_);
        io_.add_u64(2, step_);
        io_.add_f64(3, thermostat_->temperature());
        io_.add_f64(4, thermostat_->field().magnitude());
        io_.add_u64(5, i);
        io_.add_f64(6, s.sx());
        io_.add_f64(7, s.sy());
        io_.add_f64(8, s.sz());
        io_.end_row();
      }
    }
    ++step_;
  }
  size_t state_frequency() const override { return frequency_; }

 private:
  void end() {
    relax_ = -1;
    step_ = 0;
    ++stage_;
    thermostat_.reset();
  }
  parquet::Writer io_;
  size_t frequency_;
  int relax_ = -1;
  size_t step_ = 0, stage_ = 0;
  std::unique_ptr<Thermostat<S>> thermostat_;
};

}  // namespace vegas
