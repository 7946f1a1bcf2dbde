// vg_sublattice.cuh -- neighbour runs of the bcc / fcc sublattice layout,
// shared by the single-lattice Heisenberg kernel (vg_heis.cu) and the
// batched hysteresis kernels (vg_hbatch.cu).
//
// A class (basis sublattice) is an array [cell], cell = (z ny + y) nx + x;
// the SoA planes of a state are [class][xyz][cell].  The neighbours of basis
// b on basis q sit in the cells c + sum_{a in D(b,q)} {0, d_b[a]} e_a, where
// D(b,q) are the axes on which the two basis positions differ by half a cell
// (bcc: all three, 8 neighbours; fcc: two, 4 neighbours per other
// sublattice) and d_b[a] = +1 if basis b sits at the half-cell position on
// axis a, -1 otherwise (Exchange::from_lattice, src/energy.rs:176-187, over
// the edges of src/input.rs:296-322).  A run of W cells along x is one
// vector load per plane (W = 4) or one scalar (W = 1); the x-shifted run
// reuses it plus one scalar at the run's edge.
//
// The argument structs A carry nx, ny, nz, ncell (cells per class) and
// pbx, pby, pbz.
#pragma once

#include "vg_heis_common.cuh"

namespace vg {

template <typename R, int W>
struct Run {
  R v[W];
};

template <typename R, int W>
__device__ __forceinline__ Run<R, W> load_run(const R* p) {
  Run<R, W> r;
  if constexpr (W == 4) {
    const Vec4<R> t = ld4(p);
#pragma unroll
    for (int k = 0; k < 4; ++k) r.v[k] = t.v[k];
  } else {
    r.v[0] = __ldg(p);
  }
  return r;
}

template <typename R, int W>
__device__ __forceinline__ void store_run(R* p, const Run<R, W>& r) {
  if constexpr (W == 4) {
    Vec4<R> t;
#pragma unroll
    for (int k = 0; k < 4; ++k) t.v[k] = r.v[k];
    st4(p, t);
  } else {
    *p = r.v[0];
  }
}

// Shifted coordinates of a run's neighbours along each axis and whether
// the bond exists there (an open axis drops it).
struct RunNbr {
  int xe, ys, zs;
  bool xok, yok, zok;
};

// Adds the neighbours of a run of W cells of class CLS that lie on class Q.
template <typename R, int NB, int CLS, int Q, int W, typename A>
__device__ __forceinline__ void add_class(const A& a, const R* rep_base, int x0, int y, int z,
                                          const RunNbr& nb, Run<R, W> (&acc)[3]) {
  constexpr bool Dx = half_pos<NB>(Q, 0) != half_pos<NB>(CLS, 0);
  constexpr bool Dy = half_pos<NB>(Q, 1) != half_pos<NB>(CLS, 1);
  constexpr bool Dz = half_pos<NB>(Q, 2) != half_pos<NB>(CLS, 2);
  constexpr int dx = half_pos<NB>(CLS, 0) ? 1 : -1;
#pragma unroll
  for (int iz = 0; iz < (Dz ? 2 : 1); ++iz) {
    if (iz && !nb.zok) continue;
    const int zz = iz ? nb.zs : z;
#pragma unroll
    for (int iy = 0; iy < (Dy ? 2 : 1); ++iy) {
      if (iy && !nb.yok) continue;
      const int yy = iy ? nb.ys : y;
      const uint32_t row = ((uint32_t)zz * (uint32_t)a.ny + (uint32_t)yy) * (uint32_t)a.nx;  // < ncell < 2^32
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const R* pl = rep_base + (uint32_t)(Q * 3 + c) * a.ncell;  // a replica holds < 2^32 values
        const Run<R, W> v = load_run<R, W>(pl + row + x0);
#pragma unroll
        for (int k = 0; k < W; ++k) acc[c].v[k] += v.v[k];
        if constexpr (Dx) {  // the x-shifted run: W-1 entries of v plus the edge
          const R e = nb.xok ? __ldg(pl + row + nb.xe) : (R)0;
          if constexpr (dx < 0) {
            acc[c].v[0] += e;
#pragma unroll
            for (int k = 1; k < W; ++k) acc[c].v[k] += v.v[k - 1];
          } else {
#pragma unroll
            for (int k = 0; k < W - 1; ++k) acc[c].v[k] += v.v[k + 1];
            acc[c].v[W - 1] += e;
          }
        }
      }
    }
  }
}

template <int NB, int CLS, int W, typename A>
__device__ __forceinline__ RunNbr make_nbr(const A& a, int x0, int y, int z) {
  constexpr int dx = half_pos<NB>(CLS, 0) ? 1 : -1;
  constexpr int dy = half_pos<NB>(CLS, 1) ? 1 : -1;
  constexpr int dz = half_pos<NB>(CLS, 2) ? 1 : -1;
  RunNbr nb;
  nb.xe = dx < 0 ? x0 - 1 : x0 + W;
  nb.xok = true;
  if (nb.xe < 0) {
    nb.xe = a.nx - 1;
    nb.xok = a.pbx;
  } else if (nb.xe >= a.nx) {
    nb.xe = 0;
    nb.xok = a.pbx;
  }
  nb.ys = y + dy;
  nb.yok = true;
  if (nb.ys < 0 || nb.ys >= a.ny) {
    nb.ys = nb.ys < 0 ? a.ny - 1 : 0;
    nb.yok = a.pby;
  }
  nb.zs = z + dz;
  nb.zok = true;
  if (nb.zs < 0 || nb.zs >= a.nz) {
    nb.zs = nb.zs < 0 ? a.nz - 1 : 0;
    nb.zok = a.pbz;
  }
  return nb;
}

template <typename R, int W>
__device__ __forceinline__ void zero_runs(Run<R, W> (&v)[3]) {
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int k = 0; k < W; ++k) v[c].v[k] = (R)0;
}

// Neighbour field of a run of W cells of class CLS.
template <typename R, int NB, int CLS, int W, typename A>
__device__ __forceinline__ void run_field(const A& a, const R* rep_base, int x0, int y, int z,
                                          Run<R, W> (&h)[3]) {
  const RunNbr nb = make_nbr<NB, CLS, W>(a, x0, y, z);
  zero_runs(h);
  if constexpr (CLS != 0) add_class<R, NB, CLS, 0, W>(a, rep_base, x0, y, z, nb, h);
  if constexpr (CLS != 1) add_class<R, NB, CLS, 1, W>(a, rep_base, x0, y, z, nb, h);
  if constexpr (NB == 4) {
    if constexpr (CLS != 2) add_class<R, NB, CLS, 2, W>(a, rep_base, x0, y, z, nb, h);
    if constexpr (CLS != 3) add_class<R, NB, CLS, 3, W>(a, rep_base, x0, y, z, nb, h);
  }
}

// Field of the classes below CLS only (each bond counted once, from its
// higher-class end).
template <typename R, int NB, int CLS, int W, typename A>
__device__ __forceinline__ void low_field(const A& a, const R* rep_base, int x0, int y, int z,
                                          Run<R, W> (&h)[3]) {
  const RunNbr nb = make_nbr<NB, CLS, W>(a, x0, y, z);
  zero_runs(h);
  if constexpr (CLS > 0) add_class<R, NB, CLS, 0, W>(a, rep_base, x0, y, z, nb, h);
  if constexpr (CLS > 1) add_class<R, NB, CLS, 1, W>(a, rep_base, x0, y, z, nb, h);
  if constexpr (CLS > 2) add_class<R, NB, CLS, 2, W>(a, rep_base, x0, y, z, nb, h);
}

}  // namespace vg
