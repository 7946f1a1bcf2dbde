// lattice.hpp -- the slice of vegas-lattice 0.13 the hot path uses:
// Lattice::sc/bcc/fcc(a), expand(x, y, z), expand_all(n), expand_x/y/z(n) and
// drop_x/y/z() (call sites src/input.rs:296-322, src/main.rs:25,
// src/lib.rs:111).  The geometry itself (sites, nearest-neighbour bonds,
// periodic wrap) is built inside libvegas_gpu from the descriptor.
#pragma once

#include <cstdint>
#include <vector>

#include "error.hpp"
#include "vegas_gpu.h"

namespace vegas {

class Lattice {
 public:
  static Lattice sc(double /*a*/) { return Lattice(VG_CELL_SC); }
  static Lattice bcc(double /*a*/) { return Lattice(VG_CELL_BCC); }
  static Lattice fcc(double /*a*/) { return Lattice(VG_CELL_FCC); }

  Lattice expand(int x, int y, int z) const {
    Lattice l = *this;
    l.d_.nx *= x;
    l.d_.ny *= y;
    l.d_.nz *= z;
    return l;
  }
  Lattice expand_all(int n) const { return expand(n, n, n); }
  Lattice expand_x(int n) const { return expand(n, 1, 1); }
  Lattice expand_y(int n) const { return expand(1, n, 1); }
  Lattice expand_z(int n) const { return expand(1, 1, n); }
  Lattice drop_x() const {
    Lattice l = *this;
    l.d_.pbc_x = 0;
    return l;
  }
  Lattice drop_y() const {
    Lattice l = *this;
    l.d_.pbc_y = 0;
    return l;
  }
  Lattice drop_z() const {
    Lattice l = *this;
    l.d_.pbc_z = 0;
    return l;
  }

  size_t sites_len() const {
    const int nb = d_.cell == VG_CELL_SC ? 1 : d_.cell == VG_CELL_BCC ? 2 : 4;
    return (size_t)d_.nx * d_.ny * d_.nz * nb;
  }
  const vg_lattice_desc& desc() const { return d_; }

  // neighbour table as the engine builds it (nbr[i*z + k], -1 = absent)
  std::vector<int32_t> neighbours(int32_t* zmax) const {
    int64_t n = 0;
    check(vg_lattice_neighbours(&d_, nullptr, 0, &n, zmax));
    std::vector<int32_t> out((size_t)n * *zmax);
    check(vg_lattice_neighbours(&d_, out.data(), (int64_t)out.size(), &n, zmax));
    return out;
  }

 private:
  explicit Lattice(int cell) {
    d_.cell = cell;
    d_.nx = d_.ny = d_.nz = 1;
    d_.pbc_x = d_.pbc_y = d_.pbc_z = 1;
  }
  vg_lattice_desc d_{};
};

}  // namespace vegas
