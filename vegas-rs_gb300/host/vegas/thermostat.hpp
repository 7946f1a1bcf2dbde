// thermostat.hpp -- Thermostat<S> (src/thermostat.rs:17-79): a temperature
// clamped to at least f64::EPSILON and a Field<S>.
#pragma once

#include "state.hpp"

namespace vegas {

template <typename S>
class Thermostat {
 public:
  Thermostat(double temperature, Field<S> field) : temperature_(clamp(temperature)), field_(field) {}
  static Thermostat near_zero() { return Thermostat(kEpsilon, Field<S>::zero()); }

  Thermostat with_temperature(double t) const { return Thermostat(t, field_); }
  Thermostat with_field(Field<S> f) const {
    Thermostat r = *this;
    r.field_ = f;
    return r;
  }
  double temperature() const { return temperature_; }
  const Field<S>& field() const { return field_; }

 private:
  static double clamp(double t) { return t < kEpsilon ? kEpsilon : t; }
  double temperature_;
  Field<S> field_;
};

}  // namespace vegas
