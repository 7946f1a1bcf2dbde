// program.hpp -- the programs (src/program.rs:54-336): Relax, CoolDown and
// HysteresisLoop, with the reference's parameter checks, defaults and
// floating-point schedule loops replayed exactly (the CoolDown loop stops
// when T - rate*k drops below min, so it can end short of min; the
// hysteresis field runs 0 -> >max -> <-max -> >max with |B| applied along
// `up`, Field::magnitude being an absolute value).
#pragma once

#include "error.hpp"
#include "machine.hpp"
#include "state.hpp"

namespace vegas {

class Relax {
 public:
  Relax(size_t steps = 1000, double temperature = 3.0) : steps_(steps), temperature_(temperature) {}
  Relax set_steps(size_t s) const { return Relax(s, temperature_); }
  Relax set_temperature(double t) const { return Relax(steps_, t); }

  template <typename H, typename I, typename S>
  void run(Machine<H, I, S>& m) const {
    if (steps_ == 0) throw ProgramError(ProgramError::Kind::NoSteps);
    if (temperature_ < kEpsilon) throw ProgramError(ProgramError::Kind::ZeroTemperature);
    m.set_thermostat(m.thermostat().with_temperature(temperature_));
    m.relax_for(steps_);
  }

 private:
  size_t steps_;
  double temperature_;
};

class CoolDown {
 public:
  CoolDown(double max_temperature = 3.0, double min_temperature = 0.05, double cool_rate = 0.1, size_t relax = 1000,
           size_t steps = 20000)
      : max_(max_temperature), min_(min_temperature), rate_(cool_rate), relax_(relax), steps_(steps) {}
  CoolDown set_max_temperature(double v) const { return CoolDown(v, min_, rate_, relax_, steps_); }
  CoolDown set_min_temperature(double v) const { return CoolDown(max_, v, rate_, relax_, steps_); }
  CoolDown set_cool_rate(double v) const { return CoolDown(max_, min_, v, relax_, steps_); }
  CoolDown set_relax(size_t v) const { return CoolDown(max_, min_, rate_, v, steps_); }
  CoolDown set_steps(size_t v) const { return CoolDown(max_, min_, rate_, relax_, v); }

  void validate() const {
    if (max_ < min_) throw ProgramError(ProgramError::Kind::TemperatureMaxLessThanMin);
    if (steps_ == 0) throw ProgramError(ProgramError::Kind::NoSteps);
    if (min_ < kEpsilon) throw ProgramError(ProgramError::Kind::ZeroTemperature);
    if (rate_ < kEpsilon) throw ProgramError(ProgramError::Kind::ZeroCoolRate);
  }
  std::vector<double> temperatures() const {
    std::vector<double> out;
    double t = max_;
    for (;;) {
      out.push_back(t);
      t -= rate_;
      if (t < min_) break;
    }
    return out;
  }

  template <typename H, typename I, typename S>
  void run(Machine<H, I, S>& m) const {
    validate();
    for (double t : temperatures()) {
      m.set_thermostat(m.thermostat().with_temperature(t));
      m.relax_for(relax_);
      m.measure_for(steps_);
    }
  }

 private:
  double max_, min_, rate_;
  size_t relax_, steps_;
};

class HysteresisLoop {
 public:
  HysteresisLoop(size_t steps = 1000, size_t relax = 1000, double temperature = 3.0, double max_field = 1.0,
                 double field_step = 0.1)
      : steps_(steps), relax_(relax), temperature_(temperature), max_field_(max_field), field_step_(field_step) {}

  void validate() const {
    if (steps_ == 0) throw ProgramError(ProgramError::Kind::NoSteps);
    if (temperature_ < kEpsilon) throw ProgramError(ProgramError::Kind::ZeroTemperature);
    if (max_field_ < kEpsilon) throw ProgramError(ProgramError::Kind::ZeroField);
    if (field_step_ < kEpsilon) throw ProgramError(ProgramError::Kind::ZeroFieldStep);
  }
  std::vector<double> fields() const {
    std::vector<double> out;
    double m = 0.0;
    for (;;) {
      out.push_back(m);
      m += field_step_;
      if (m > max_field_) break;
    }
    for (;;) {
      out.push_back(m);
      m -= field_step_;
      if (m < -max_field_) break;
    }
    for (;;) {
      out.push_back(m);
      m += field_step_;
      if (m > max_field_) break;
    }
    return out;
  }

  template <typename H, typename I, typename S>
  void run(Machine<H, I, S>& m) const {
    validate();
    m.set_thermostat(m.thermostat().with_temperature(temperature_));
    for (double b : fields()) {
      m.set_thermostat(m.thermostat().with_field(Field<S>(S::up(), b)));
      m.relax_for(relax_);
      m.measure_for(steps_);
    }
  }

 private:
  size_t steps_, relax_;
  double temperature_, max_field_, field_step_;
};

}  // namespace vegas
