// error.hpp -- the error kinds of vegas (src/error.rs:13-87) as C++ exceptions.
//
// Where the reference returns Err(..) and `main` prints "Error: {e}" and exits
// with status 1 (src/main.rs:84-89), this host throws and its CLI does the
// same.  GpuError is the new variant for a failed call into libvegas_gpu.
#pragma once

#include <stdexcept>
#include <string>

#include "vegas_gpu.h"

namespace vegas {

class VegasError : public std::runtime_error {
 public:
  using std::runtime_error::runtime_error;
};

// ProgramError (src/error.rs:39-56)
class ProgramError : public VegasError {
 public:
  enum class Kind { TemperatureMaxLessThanMin, NoSteps, ZeroTemperature, ZeroCoolRate, ZeroField, ZeroFieldStep };
  explicit ProgramError(Kind k) : VegasError(message(k)), kind(k) {}
  Kind kind;

  static std::string message(Kind k) {
    switch (k) {
      case Kind::TemperatureMaxLessThanMin: return "program error: maximum temperature must be greater than minimum temperature";
      case Kind::NoSteps: return "program error: there should be at least one step";
      case Kind::ZeroTemperature: return "program error: temperature must be greater than zero";
      case Kind::ZeroCoolRate: return "program error: cooling rate must be greater than zero";
      case Kind::ZeroField: return "program error: maximum field must be greater than zero";
      case Kind::ZeroFieldStep: return "program error: field step must be greater than zero";
    }
    return "program error";
  }
};

class IoError : public VegasError {
 public:
  using VegasError::VegasError;
};

class NotImplementedError : public VegasError {
 public:
  NotImplementedError() : VegasError("not implemented error") {}
};

// A non-zero status from the C ABI, with the library's message.
class GpuError : public VegasError {
 public:
  GpuError(int status, const std::string& msg)
      : VegasError("gpu error: " + std::string(vg_status_string(status)) + ": " + msg), status(status) {}
  int status;
};

inline void check(int status, const vg_ctx* ctx = nullptr) {
  if (status != VG_OK) throw GpuError(status, vg_last_error(ctx));
}

}  // namespace vegas
