// accumulator.hpp -- Accumulator (src/accumulator.rs:22-70): running sums of
// x, x^2 and x^4 in f64; naive variance E[x^2] - E[x]^2 and the Binder
// cumulant, exactly as the reference forms them.
#pragma once

#include <cstddef>

namespace vegas {

class Accumulator {
 public:
  void collect(double v) {
    sum_ += v;
    sum_sq_ += v * v;
    sum_fourth_ += v * v * v * v;
    ++count_;
  }
  double mean() const { return sum_ / (double)count_; }
  double variance() const {
    const double m = mean();
    return sum_sq_ / (double)count_ - m * m;
  }
  double binder_cumulant() const {
    const double s2 = sum_sq_ / (double)count_;
    return 1.0 - (sum_fourth_ / (double)count_) / (3.0 * s2 * s2);
  }
  size_t count() const { return count_; }

 private:
  double sum_ = 0.0, sum_sq_ = 0.0, sum_fourth_ = 0.0;
  size_t count_ = 0;
};

}  // namespace vegas
