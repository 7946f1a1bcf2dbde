// vg_heis.cu -- Heisenberg colour-class Metropolis passes (FP32 and FP64).
//
// Replaces MetropolisIntegrator::step (proposal Spin::rand, a uniform point
// on S^2, src/integrator.rs:66-92, src/util.rs:21-34) and
// MetropolisFlipIntegrator::step (proposal -s, :113-137) for HeisenbergSpin,
// with the energy terms of src/energy.rs (Exchange, UniaxialAnisotropy,
// Zeeman with the reference's per-site sign, Gauge) plus a cubic term.
// Each site consumes one Philox block keyed (class entry j, sweep, tag,
// colour): words 0/1 give the proposal (Archimedes map: z uniform in (-1,1),
// azimuth uniform), word 2 the acceptance uniform.  dE is formed as a
// difference of per-term changes (no cancellation of two O(z) energies),
// accepted if dE <= 0 or u < exp(-dE/T).
//
// Per-sweep sums: each site adds its terms after its own update; the bond
// sum takes, for each site, only neighbours of lower colour, which are final
// for the sweep when that site's pass runs, so every bond is counted once.
#include "vg_heis_common.cuh"
#include "vg_sublattice.cuh"

namespace vg {

// ------------------------------------------------------------------ sc
template <typename R, int C, bool ALLPER, bool MEASURE, bool UPDATE, int PROP>
__global__ void __launch_bounds__(256) heis_sc_kernel(const HeisScArgs<R> a, const HeisParams<R> P, const RngKey key,
                                                      double* __restrict__ part) {
  R* __restrict__ ox = a.x[C];
  R* __restrict__ oy = a.y[C];
  R* __restrict__ oz = a.z[C];
  const R* __restrict__ nx = a.x[C ^ 1];
  const R* __restrict__ ny = a.y[C ^ 1];
  const R* __restrict__ nz = a.z[C ^ 1];
  R acc[kNumSums];
#pragma unroll
  for (int i = 0; i < kNumSums; ++i) acc[i] = (R)0;
  pdl_launch_dependents();
  pdl_wait();
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < a.n_c; j += stride) {
    const int row = (int)fdiv(j, a.fHx);
    const int h = (int)(j - (uint32_t)row * a.Hx);
    const int z = (int)fdiv((uint32_t)row, a.fLy);
    const int y = row - z * a.Ly;
    const int p = (y + z + C) & 1;
    const int rb = row * a.Hx;
    V3<R> hs = {(R)0, (R)0, (R)0};
    auto add = [&](int q) {
      hs.x += __ldg(nx + q);
      hs.y += __ldg(ny + q);
      hs.z += __ldg(nz + q);
    };
    add(rb + h);
    int hx = p ? h + 1 : h - 1;
    bool hxok = true;
    if (hx < 0) {
      hx = a.Hx - 1;
      hxok = ALLPER || a.pbx;
    } else if (hx >= a.Hx) {
      hx = 0;
      hxok = ALLPER || a.pbx;
    }
    if (hxok) add(rb + hx);
    if (y > 0) add(rb - a.Hx + h);
    else if (ALLPER || a.pby) add(rb + (a.Ly - 1) * a.Hx + h);
    if (y < a.Ly - 1) add(rb + a.Hx + h);
    else if (ALLPER || a.pby) add(rb - (a.Ly - 1) * a.Hx + h);
    const int plane = a.Ly * a.Hx;
    if (z > 0) add(rb - plane + h);
    else if (ALLPER || a.pbz) add(rb + (a.Lz - 1) * plane + h);
    if (z < a.Lz - 1) add(rb + plane + h);
    else if (ALLPER || a.pbz) add(rb - (a.Lz - 1) * plane + h);

    const int q = rb + h;
    V3<R> s = {ox[q], oy[q], oz[q]};
    if (UPDATE) {
      const uint4 w = philox_ks<kHeisRounds>(
          make_uint4(j, key.sweep, (kTagHeis << 24) | ((uint32_t)C << 8), key.replica), key.ks);
      V3<R> sn;
      if (heis_update<R, PROP>(s, hs, P, w, sn)) {
        ox[q] = sn.x;
        oy[q] = sn.y;
        oz[q] = sn.z;
        s = sn;
        acc[7] += (R)1;
      }
    }
    if (MEASURE) {
      const V3<R> low = C == 1 ? hs : V3<R>{(R)0, (R)0, (R)0};
      add_site_sums(acc, s, low, P);
    }
  }
  if (MEASURE) flush_sums(acc, part);
}

// Four consecutive class entries per thread (x extent a multiple of 8):
// float4 loads of the SoA planes; the x neighbour outside the same float4 is
// one scalar per plane, as in the Ising checkerboard kernel.
template <typename R, int C, bool ALLPER, bool MEASURE, bool UPDATE, int PROP>
__global__ void __launch_bounds__(256) heis_sc4_kernel(const HeisScArgs<R> a, const HeisParams<R> P, const RngKey key,
                                                       double* __restrict__ part) {
  R* own[3] = {a.x[C], a.y[C], a.z[C]};
  const R* oth[3] = {a.x[C ^ 1], a.y[C ^ 1], a.z[C ^ 1]};
  R acc[kNumSums];
#pragma unroll
  for (int i = 0; i < kNumSums; ++i) acc[i] = (R)0;
  pdl_launch_dependents();
  pdl_wait();
  const uint32_t n4 = a.n_c >> 2;
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n4; q += stride) {
    const uint32_t j0 = q << 2;
    const int row = (int)fdiv(j0, a.fHx);
    const int h0 = (int)(j0 - (uint32_t)row * a.Hx);
    const int z = (int)fdiv((uint32_t)row, a.fLy);
    const int y = row - z * a.Ly;
    const int p = (y + z + C) & 1;
    const int rb = row * a.Hx;
    const int plane = a.Ly * a.Hx;
    const int rym = y > 0 ? rb - a.Hx : ((ALLPER || a.pby) ? rb + (a.Ly - 1) * a.Hx : -1);
    const int ryp = y < a.Ly - 1 ? rb + a.Hx : ((ALLPER || a.pby) ? rb - (a.Ly - 1) * a.Hx : -1);
    const int rzm = z > 0 ? rb - plane : ((ALLPER || a.pbz) ? rb + (a.Lz - 1) * plane : -1);
    const int rzp = z < a.Lz - 1 ? rb + plane : ((ALLPER || a.pbz) ? rb - (a.Lz - 1) * plane : -1);
    // x neighbour not inside the float4: h0-1 (p = 0) or h0+4 (p = 1)
    int xe;
    bool xok = true;
    if (p == 0) {
      xe = h0 > 0 ? rb + h0 - 1 : rb + a.Hx - 1;
      xok = h0 > 0 || ALLPER || a.pbx;
    } else {
      xe = h0 + 4 < a.Hx ? rb + h0 + 4 : rb;
      xok = h0 + 4 < a.Hx || ALLPER || a.pbx;
    }
    Vec4<R> hs[3], S[3];
#pragma unroll
    for (int c3 = 0; c3 < 3; ++c3) {
      const Vec4<R> X0 = ld4(oth[c3] + rb + h0);
      const R e = xok ? __ldg(oth[c3] + xe) : (R)0;
      Vec4<R> t = X0;
      if (p == 0) {
        t.v[0] += e;
        t.v[1] += X0.v[0];
        t.v[2] += X0.v[1];
        t.v[3] += X0.v[2];
      } else {
        t.v[0] += X0.v[1];
        t.v[1] += X0.v[2];
        t.v[2] += X0.v[3];
        t.v[3] += e;
      }
      if (rym >= 0) {
        const Vec4<R> u = ld4(oth[c3] + rym + h0);
#pragma unroll
        for (int k = 0; k < 4; ++k) t.v[k] += u.v[k];
      }
      if (ryp >= 0) {
        const Vec4<R> u = ld4(oth[c3] + ryp + h0);
#pragma unroll
        for (int k = 0; k < 4; ++k) t.v[k] += u.v[k];
      }
      if (rzm >= 0) {
        const Vec4<R> u = ld4(oth[c3] + rzm + h0);
#pragma unroll
        for (int k = 0; k < 4; ++k) t.v[k] += u.v[k];
      }
      if (rzp >= 0) {
        const Vec4<R> u = ld4(oth[c3] + rzp + h0);
#pragma unroll
        for (int k = 0; k < 4; ++k) t.v[k] += u.v[k];
      }
      hs[c3] = t;
      S[c3] = ld4(own[c3] + rb + h0);
    }
    bool changed = false;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      V3<R> s = {S[0].v[k], S[1].v[k], S[2].v[k]};
      const V3<R> h = {hs[0].v[k], hs[1].v[k], hs[2].v[k]};
      if (UPDATE) {
        const uint4 w = philox_ks<kHeisRounds>(
            make_uint4(j0 + (uint32_t)k, key.sweep, (kTagHeis << 24) | ((uint32_t)C << 8), key.replica), key.ks);
        V3<R> sn;
        if (heis_update<R, PROP>(s, h, P, w, sn)) {
          S[0].v[k] = sn.x;
          S[1].v[k] = sn.y;
          S[2].v[k] = sn.z;
          s = sn;
          changed = true;
          acc[7] += (R)1;
        }
      }
      if (MEASURE) {
        const V3<R> low = C == 1 ? h : V3<R>{(R)0, (R)0, (R)0};
        add_site_sums(acc, s, low, P);
      }
    }
    if (changed) {
#pragma unroll
      for (int c3 = 0; c3 < 3; ++c3) st4(own[c3] + rb + h0, S[c3]);
    }
  }
  if (MEASURE) flush_sums(acc, part);
}

// ------------------------------------------------------------- generic
// NI class entries per thread at a time (j, j + stride, ...), the loads of
// all NI issued before any store: a pass writes only its own class and reads
// only the others, which the compiler cannot see across loop iterations.
// Entries keep their order within a thread, so the per-thread sums are the
// same.  Classes with no more entries than the grid has threads run NI = 1.
template <typename R, int ZT, int NI, bool MEASURE, bool UPDATE, int PROP>
__global__ void __launch_bounds__(256) heis_gen_kernel(const HeisGenArgs<R> a, const HeisParams<R> P, const RngKey key,
                                                       const int colour, double* __restrict__ part) {
  R acc[kNumSums];
#pragma unroll
  for (int i = 0; i < kNumSums; ++i) acc[i] = (R)0;
  pdl_launch_dependents();
  pdl_wait();
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long j0 = (long long)blockIdx.x * blockDim.x + threadIdx.x; j0 < a.n_c; j0 += NI * stride) {
    int site[NI];
    uint32_t lm[NI];
    bool live[NI];
    V3<R> hs[NI], low[NI], s[NI];
#pragma unroll
    for (int b = 0; b < NI; ++b) {
      const long long j = j0 + b * stride;
      live[b] = j < a.n_c;
      const long long jj = live[b] ? j : j0;  // past the class's end: entry j0's data, dropped
      site[b] = __ldg(a.sites + jj);
      lm[b] = __ldg(a.lowmask + jj);
      hs[b] = {(R)0, (R)0, (R)0};
      low[b] = {(R)0, (R)0, (R)0};
    }
#pragma unroll
    for (int k = 0; k < ZT; ++k) {
      if (k < a.zc) {
#pragma unroll
        for (int b = 0; b < NI; ++b) {
          const long long jj = live[b] ? j0 + b * stride : j0;
          const uint32_t e = (uint32_t)k * (uint32_t)a.n_c + (uint32_t)jj;
          const int t = __ldg(a.nbr + e);
          if (t >= 0) {
            const R wk = a.jb ? __ldg(a.jb + e) : (R)1;
            const R vx = wk * a.x[t], vy = wk * a.y[t], vz = wk * a.z[t];
            hs[b].x += vx;
            hs[b].y += vy;
            hs[b].z += vz;
            if ((lm[b] >> k) & 1u) {
              low[b].x += vx;
              low[b].y += vy;
              low[b].z += vz;
            }
          }
        }
      }
    }
#pragma unroll
    for (int b = 0; b < NI; ++b) s[b] = {a.x[site[b]], a.y[site[b]], a.z[site[b]]};
#pragma unroll
    for (int b = 0; b < NI; ++b) {
      if (!live[b]) continue;
      const long long j = j0 + b * stride;
      if (UPDATE) {
        const uint4 w = philox_ks<kHeisRounds>(
            make_uint4((uint32_t)j, key.sweep, (kTagHeis << 24) | ((uint32_t)colour << 8), key.replica), key.ks);
        V3<R> sn;
        if (heis_update<R, PROP>(s[b], hs[b], P, w, sn)) {
          a.x[site[b]] = sn.x;
          a.y[site[b]] = sn.y;
          a.z[site[b]] = sn.z;
          s[b] = sn;
          acc[7] += (R)1;
        }
      }
      if (MEASURE) add_site_sums(acc, s[b], low[b], P);
    }
  }
  if (MEASURE) flush_sums(acc, part);
}

// ------------------------------------------------------------ dispatch
template <typename R, int C, bool ALLPER>
static void sc_go(const HeisScArgs<R>& a, const HeisParams<R>& p, RngKey key, int proposal, bool update, double* part,
                  int grid, int tpb, cudaStream_t s) {
  const bool m = part != nullptr;
  if (!update) {
    launch_pdl(heis_sc_kernel<R, C, ALLPER, true, false, VG_PROPOSE_FLIP>, grid, tpb, s, a, p, key, part);
  } else if (proposal == VG_PROPOSE_RANDOM) {
    if (m) launch_pdl(heis_sc_kernel<R, C, ALLPER, true, true, VG_PROPOSE_RANDOM>, grid, tpb, s, a, p, key, part);
    else launch_pdl(heis_sc_kernel<R, C, ALLPER, false, true, VG_PROPOSE_RANDOM>, grid, tpb, s, a, p, key, part);
  } else {
    if (m) launch_pdl(heis_sc_kernel<R, C, ALLPER, true, true, VG_PROPOSE_FLIP>, grid, tpb, s, a, p, key, part);
    else launch_pdl(heis_sc_kernel<R, C, ALLPER, false, true, VG_PROPOSE_FLIP>, grid, tpb, s, a, p, key, part);
  }
}

template <typename R, int C, bool ALLPER>
static void sc4_go(const HeisScArgs<R>& a, const HeisParams<R>& p, RngKey key, int proposal, bool update, double* part,
                   int grid, int tpb, cudaStream_t s) {
  const bool m = part != nullptr;
  if (!update) {
    launch_pdl(heis_sc4_kernel<R, C, ALLPER, true, false, VG_PROPOSE_FLIP>, grid, tpb, s, a, p, key, part);
  } else if (proposal == VG_PROPOSE_RANDOM) {
    if (m) launch_pdl(heis_sc4_kernel<R, C, ALLPER, true, true, VG_PROPOSE_RANDOM>, grid, tpb, s, a, p, key, part);
    else launch_pdl(heis_sc4_kernel<R, C, ALLPER, false, true, VG_PROPOSE_RANDOM>, grid, tpb, s, a, p, key, part);
  } else {
    if (m) launch_pdl(heis_sc4_kernel<R, C, ALLPER, true, true, VG_PROPOSE_FLIP>, grid, tpb, s, a, p, key, part);
    else launch_pdl(heis_sc4_kernel<R, C, ALLPER, false, true, VG_PROPOSE_FLIP>, grid, tpb, s, a, p, key, part);
  }
}

template <typename R>
cudaError_t launch_heis_sc(const HeisScArgs<R>& a, const HeisParams<R>& p, RngKey key, int colour, int proposal,
                           bool update, double* part, int grid, int tpb, cudaStream_t s) {
  const bool allper = a.pbx && a.pby && a.pbz;
  if (a.Hx % 4 == 0) {  // four sites per thread
    if (colour == 0) {
      if (allper) sc4_go<R, 0, true>(a, p, key, proposal, update, part, grid, tpb, s);
      else sc4_go<R, 0, false>(a, p, key, proposal, update, part, grid, tpb, s);
    } else {
      if (allper) sc4_go<R, 1, true>(a, p, key, proposal, update, part, grid, tpb, s);
      else sc4_go<R, 1, false>(a, p, key, proposal, update, part, grid, tpb, s);
    }
    return cudaGetLastError();
  }
  if (colour == 0) {
    if (allper) sc_go<R, 0, true>(a, p, key, proposal, update, part, grid, tpb, s);
    else sc_go<R, 0, false>(a, p, key, proposal, update, part, grid, tpb, s);
  } else {
    if (allper) sc_go<R, 1, true>(a, p, key, proposal, update, part, grid, tpb, s);
    else sc_go<R, 1, false>(a, p, key, proposal, update, part, grid, tpb, s);
  }
  return cudaGetLastError();
}

template <typename R, int ZT, int NI>
static void gen_go_ni(const HeisGenArgs<R>& a, const HeisParams<R>& p, RngKey key, int colour, int proposal,
                      bool update, double* part, int grid, int tpb, cudaStream_t s) {
  const bool m = part != nullptr;
  if (!update) {
    launch_pdl(heis_gen_kernel<R, ZT, NI, true, false, VG_PROPOSE_FLIP>, grid, tpb, s, a, p, key, colour, part);
  } else if (proposal == VG_PROPOSE_RANDOM) {
    if (m) launch_pdl(heis_gen_kernel<R, ZT, NI, true, true, VG_PROPOSE_RANDOM>, grid, tpb, s, a, p, key, colour, part);
    else launch_pdl(heis_gen_kernel<R, ZT, NI, false, true, VG_PROPOSE_RANDOM>, grid, tpb, s, a, p, key, colour, part);
  } else {
    if (m) launch_pdl(heis_gen_kernel<R, ZT, NI, true, true, VG_PROPOSE_FLIP>, grid, tpb, s, a, p, key, colour, part);
    else launch_pdl(heis_gen_kernel<R, ZT, NI, false, true, VG_PROPOSE_FLIP>, grid, tpb, s, a, p, key, colour, part);
  }
}

template <typename R, int ZT>
static void gen_go(const HeisGenArgs<R>& a, const HeisParams<R>& p, RngKey key, int colour, int proposal, bool update,
                   double* part, int grid, int tpb, cudaStream_t s) {
  if (a.n_c > (long long)grid * tpb) gen_go_ni<R, ZT, 2>(a, p, key, colour, proposal, update, part, grid, tpb, s);
  else gen_go_ni<R, ZT, 1>(a, p, key, colour, proposal, update, part, grid, tpb, s);
}

template <typename R>
cudaError_t launch_heis_gen(const HeisGenArgs<R>& a, const HeisParams<R>& p, RngKey key, int colour, int proposal,
                            bool update, double* part, int grid, int tpb, cudaStream_t s) {
  if (a.zc <= 6) gen_go<R, 6>(a, p, key, colour, proposal, update, part, grid, tpb, s);
  else if (a.zc <= 8) gen_go<R, 8>(a, p, key, colour, proposal, update, part, grid, tpb, s);
  else gen_go<R, 12>(a, p, key, colour, proposal, update, part, grid, tpb, s);
  return cudaGetLastError();
}

// ------------------------------------------------------------- sublattice
// bcc / fcc: one thread per run of W cells of class CLS (the basis
// sublattice), SoA planes [class][xyz][cell].  The field adds the classes in
// ascending order, the lower ones first: their partial sum is the bond field
// the class's lattice sums count (each bond once, from its higher-class end).
// Entry j of the class is cell j, so the draws are the generic path's.
template <typename R, int NB, int CLS, int W, bool MEASURE, bool UPDATE, int PROP>
__global__ void __launch_bounds__(256, sizeof(R) == 4 ? 3 : 2) heis_sub_kernel(const HeisSubArgs<R> a, const HeisParams<R> P,
                                                          const RngKey key, double* __restrict__ part) {
  R* own[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) own[c] = a.spin + (size_t)(CLS * 3 + c) * a.ncell;
  R acc[kNumSums];
#pragma unroll
  for (int i = 0; i < kNumSums; ++i) acc[i] = (R)0;
  pdl_launch_dependents();
  pdl_wait();
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < a.runs; u += stride) {
    const int row = (int)fdiv(u, a.frow);
    const int x0 = (int)(u - (uint32_t)row * (uint32_t)a.rpr) * W;
    const int z = (int)fdiv((uint32_t)row, a.fny);
    const int y = row - z * a.ny;
    const RunNbr nb = make_nbr<NB, CLS, W>(a, x0, y, z);
    Run<R, W> hf[3], lo[3];
    zero_runs(hf);
    if constexpr (CLS > 0) add_class<R, NB, CLS, 0, W>(a, a.spin, x0, y, z, nb, hf);
    if constexpr (CLS > 1) add_class<R, NB, CLS, 1, W>(a, a.spin, x0, y, z, nb, hf);
    if constexpr (CLS > 2) add_class<R, NB, CLS, 2, W>(a, a.spin, x0, y, z, nb, hf);
    if (MEASURE) {
#pragma unroll
      for (int c = 0; c < 3; ++c) lo[c] = hf[c];
    }
    if constexpr (CLS < 1) add_class<R, NB, CLS, 1, W>(a, a.spin, x0, y, z, nb, hf);
    if constexpr (NB == 4 && CLS < 2) add_class<R, NB, CLS, 2, W>(a, a.spin, x0, y, z, nb, hf);
    if constexpr (NB == 4 && CLS < 3) add_class<R, NB, CLS, 3, W>(a, a.spin, x0, y, z, nb, hf);
    const uint32_t j0 = (uint32_t)row * (uint32_t)a.nx + (uint32_t)x0;
    Run<R, W> S[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) S[c] = load_run<R, W>(own[c] + j0);
    bool changed = false;
#pragma unroll
    for (int k = 0; k < W; ++k) {
      V3<R> s = {S[0].v[k], S[1].v[k], S[2].v[k]};
      if (UPDATE) {
        const V3<R> h = {hf[0].v[k], hf[1].v[k], hf[2].v[k]};
        const uint4 w = philox_ks<kHeisRounds>(
            make_uint4(j0 + (uint32_t)k, key.sweep, (kTagHeis << 24) | ((uint32_t)CLS << 8), key.replica), key.ks);
        V3<R> sn;
        if (heis_update<R, PROP>(s, h, P, w, sn)) {
          S[0].v[k] = sn.x;
          S[1].v[k] = sn.y;
          S[2].v[k] = sn.z;
          s = sn;
          changed = true;
          acc[7] += (R)1;
        }
      }
      if (MEASURE) {
        const V3<R> low = {lo[0].v[k], lo[1].v[k], lo[2].v[k]};
        add_site_sums(acc, s, low, P);
      }
    }
    if (changed) {
#pragma unroll
      for (int c = 0; c < 3; ++c) store_run<R, W>(own[c] + j0, S[c]);
    }
  }
  if (MEASURE) flush_sums(acc, part);
}

template <typename R, int NB, int CLS, int W>
static void sub_go(const HeisSubArgs<R>& a, const HeisParams<R>& p, RngKey key, int proposal, bool update,
                   double* part, int grid, int tpb, cudaStream_t s) {
  const bool m = part != nullptr;
  if (!update) {
    launch_pdl(heis_sub_kernel<R, NB, CLS, W, true, false, VG_PROPOSE_FLIP>, grid, tpb, s, a, p, key, part);
  } else if (proposal == VG_PROPOSE_RANDOM) {
    if (m) launch_pdl(heis_sub_kernel<R, NB, CLS, W, true, true, VG_PROPOSE_RANDOM>, grid, tpb, s, a, p, key, part);
    else launch_pdl(heis_sub_kernel<R, NB, CLS, W, false, true, VG_PROPOSE_RANDOM>, grid, tpb, s, a, p, key, part);
  } else {
    if (m) launch_pdl(heis_sub_kernel<R, NB, CLS, W, true, true, VG_PROPOSE_FLIP>, grid, tpb, s, a, p, key, part);
    else launch_pdl(heis_sub_kernel<R, NB, CLS, W, false, true, VG_PROPOSE_FLIP>, grid, tpb, s, a, p, key, part);
  }
}

template <typename R, int W>
static void sub_cls(const HeisSubArgs<R>& a, int nb, const HeisParams<R>& p, RngKey key, int colour, int proposal,
                    bool update, double* part, int grid, int tpb, cudaStream_t s) {
  if (nb == 2) {
    if (colour == 0) sub_go<R, 2, 0, W>(a, p, key, proposal, update, part, grid, tpb, s);
    else sub_go<R, 2, 1, W>(a, p, key, proposal, update, part, grid, tpb, s);
    return;
  }
  switch (colour) {
    case 0: sub_go<R, 4, 0, W>(a, p, key, proposal, update, part, grid, tpb, s); break;
    case 1: sub_go<R, 4, 1, W>(a, p, key, proposal, update, part, grid, tpb, s); break;
    case 2: sub_go<R, 4, 2, W>(a, p, key, proposal, update, part, grid, tpb, s); break;
    default: sub_go<R, 4, 3, W>(a, p, key, proposal, update, part, grid, tpb, s); break;
  }
}

template <typename R>
cudaError_t launch_heis_sub(const HeisSubArgs<R>& a, int nb, int W, const HeisParams<R>& p, RngKey key, int colour,
                            int proposal, bool update, double* part, int grid, int tpb, cudaStream_t s) {
  if (W == 4) sub_cls<R, 4>(a, nb, p, key, colour, proposal, update, part, grid, tpb, s);
  else sub_cls<R, 1>(a, nb, p, key, colour, proposal, update, part, grid, tpb, s);
  return cudaGetLastError();
}

template cudaError_t launch_heis_sc<float>(const HeisScArgs<float>&, const HeisParams<float>&, RngKey, int, int, bool,
                                           double*, int, int, cudaStream_t);
template cudaError_t launch_heis_sc<double>(const HeisScArgs<double>&, const HeisParams<double>&, RngKey, int, int,
                                            bool, double*, int, int, cudaStream_t);
template cudaError_t launch_heis_gen<float>(const HeisGenArgs<float>&, const HeisParams<float>&, RngKey, int, int,
                                            bool, double*, int, int, cudaStream_t);
template cudaError_t launch_heis_gen<double>(const HeisGenArgs<double>&, const HeisParams<double>&, RngKey, int, int,
                                             bool, double*, int, int, cudaStream_t);
template cudaError_t launch_heis_sub<float>(const HeisSubArgs<float>&, int, int, const HeisParams<float>&, RngKey, int,
                                            int, bool, double*, int, int, cudaStream_t);
template cudaError_t launch_heis_sub<double>(const HeisSubArgs<double>&, int, int, const HeisParams<double>&, RngKey,
                                             int, int, bool, double*, int, int, cudaStream_t);

}  // namespace vg
