// state.hpp -- spins, fields and states (src/state.rs:28-318).
//
// IsingSpin / HeisenbergSpin keep the reference's semantics (dot, flip,
// projections, from_projections); State<S> is the host-side copy that
// crosses the C ABI in site order.  The engine itself keeps the state on the
// device; a State is materialised only when a caller asks for it.
#pragma once

#include <array>
#include <cmath>
#include <cstdint>
#include <limits>
#include <vector>

namespace vegas {

constexpr double kEpsilon = std::numeric_limits<double>::epsilon();

template <typename S>
struct Field;

// IsingSpin (src/state.rs:59-130)
struct IsingSpin {
  enum Value : int8_t { Down = -1, Up = 1 } v = Up;
  static constexpr int kind = 0;  // VG_SPIN_ISING

  static IsingSpin up() { return {Up}; }
  static IsingSpin down() { return {Down}; }
  IsingSpin flip() const { return {v == Up ? Down : Up}; }
  double dot(const IsingSpin& o) const { return v == o.v ? 1.0 : -1.0; }
  double sx() const { return 0.0; }
  double sy() const { return 0.0; }
  double sz() const { return v == Up ? 1.0 : -1.0; }
  bool operator==(const IsingSpin& o) const { return v == o.v; }
  static Field<IsingSpin> from_projections(double, double, double sz);
  // host encoding crossing the C ABI: one int8 per site
  using Raw = int8_t;
  static constexpr int raw_per_site = 1;
};

// HeisenbergSpin (src/state.rs:132-192)
struct HeisenbergSpin {
  std::array<double, 3> s{0.0, 0.0, 1.0};
  static constexpr int kind = 1;  // VG_SPIN_HEISENBERG

  static HeisenbergSpin up() { return {{0.0, 0.0, 1.0}}; }
  static HeisenbergSpin down() { return {{0.0, 0.0, -1.0}}; }
  HeisenbergSpin flip() const { return {{-s[0], -s[1], -s[2]}}; }
  double dot(const HeisenbergSpin& o) const { return s[0] * o.s[0] + s[1] * o.s[1] + s[2] * o.s[2]; }
  double sx() const { return s[0]; }
  double sy() const { return s[1]; }
  double sz() const { return s[2]; }
  bool operator==(const HeisenbergSpin& o) const { return s == o.s; }
  static Field<HeisenbergSpin> from_projections(double sx, double sy, double sz);
  using Raw = double;
  static constexpr int raw_per_site = 3;
};

// Field<S> (src/state.rs:194-227): magnitude() returns the absolute value.
template <typename S>
struct Field {
  S orientation = S::up();
  double magnitude_ = 0.0;

  Field() = default;
  Field(S o, double m) : orientation(o), magnitude_(m) {}
  static Field zero() { return Field(S::up(), 0.0); }
  double magnitude() const { return std::fabs(magnitude_); }
  // orientation as the 3-vector the C ABI takes
  std::array<double, 3> b_hat() const { return {orientation.sx(), orientation.sy(), orientation.sz()}; }
};

inline Field<IsingSpin> IsingSpin::from_projections(double, double, double sz) {
  return sz >= 0.0 ? Field<IsingSpin>(IsingSpin::up(), std::fabs(sz)) : Field<IsingSpin>(IsingSpin::down(), std::fabs(sz));
}

inline Field<HeisenbergSpin> HeisenbergSpin::from_projections(double sx, double sy, double sz) {
  const double m = std::sqrt(sx * sx + sy * sy + sz * sz);
  if (std::fabs(m) < kEpsilon) return Field<HeisenbergSpin>::zero();
  return Field<HeisenbergSpin>(HeisenbergSpin{{sx / m, sy / m, sz / m}}, m);
}

// State<S> (src/state.rs:244-318)
template <typename S>
class State {
 public:
  State() = default;
  explicit State(std::vector<S> v) : spins_(std::move(v)) {}
  static State up_with_size(size_t n) { return State(std::vector<S>(n, S::up())); }
  static State down_with_size(size_t n) { return State(std::vector<S>(n, S::down())); }

  const std::vector<S>& spins() const { return spins_; }
  const S& at(size_t i) const { return spins_.at(i); }
  void set_at(size_t i, S s) { spins_.at(i) = s; }
  size_t len() const { return spins_.size(); }
  bool is_empty() const { return spins_.empty(); }

  // magnetization(): Sum of projections -> S::from_projections (src/state.rs:235-242, :291-297)
  Field<S> magnetization() const {
    double px = 0.0, py = 0.0, pz = 0.0;
    for (const S& s : spins_) {
      px += s.sx();
      py += s.sy();
      pz += s.sz();
    }
    return S::from_projections(px, py, pz);
  }

  // raw site-order encoding for vg_set_state / vg_get_state
  std::vector<typename S::Raw> to_raw() const;
  static State from_raw(const std::vector<typename S::Raw>& raw);

 private:
  std::vector<S> spins_;
};

template <>
inline std::vector<int8_t> State<IsingSpin>::to_raw() const {
  std::vector<int8_t> r(spins_.size());
  for (size_t i = 0; i < spins_.size(); ++i) r[i] = spins_[i].v;
  return r;
}
template <>
inline State<IsingSpin> State<IsingSpin>::from_raw(const std::vector<int8_t>& raw) {
  std::vector<IsingSpin> v(raw.size());
  for (size_t i = 0; i < raw.size(); ++i) v[i] = raw[i] > 0 ? IsingSpin::up() : IsingSpin::down();
  return State<IsingSpin>(std::move(v));
}
template <>
inline std::vector<double> State<HeisenbergSpin>::to_raw() const {
  std::vector<double> r(3 * spins_.size());
  for (size_t i = 0; i < spins_.size(); ++i)
    for (int a = 0; a < 3; ++a) r[3 * i + a] = spins_[i].s[a];
  return r;
}
template <>
inline State<HeisenbergSpin> State<HeisenbergSpin>::from_raw(const std::vector<double>& raw) {
  std::vector<HeisenbergSpin> v(raw.size() / 3);
  for (size_t i = 0; i < v.size(); ++i) v[i] = HeisenbergSpin{{raw[3 * i], raw[3 * i + 1], raw[3 * i + 2]}};
  return State<HeisenbergSpin>(std::move(v));
}

}  // namespace vegas
