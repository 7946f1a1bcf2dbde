// vg_energy.cu -- per-site energies of a context's state
// (Hamiltonian::energy, src/energy.rs:45-52 with the terms of
// src/energy.rs:75-80, 108-112, 147-152, 194-208) and single-site energy
// changes of proposed Heisenberg spins, on natural-order copies of the state.
//
// The site energy is the sum of the Hamiltonian's terms at the site, as
// Compound::energy forms it: -sum_j J_ij s_i.s_j + K (s.e)^2 + B (s.b) + g,
// plus the cubic term -Kc (sx^4 + sy^4 + sz^4) when the Hamiltonian has one;
// absent terms contribute nothing.  It is computed in FP64 from the state as
// the context holds it (an FP32 state converts exactly).  The energy change
// runs heis_delta_e, the function of the sweeps, in the context's precision.
#include <cuda_runtime.h>

#include "vg_heis_common.cuh"

namespace vg {

namespace {

// Ising spins: int8 +-1; the anisotropy axis and the field orientation are
// Ising spins too (their z sign).
__global__ void ising_site_energy_kernel(const int8_t* __restrict__ s, int64_t n, int z,
                                         const int32_t* __restrict__ nbr, const double* __restrict__ jnat,
                                         SiteTerms t, double* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double si = (double)s[i];
    double e = 0.0;
    if (t.has_exchange) {
      double acc = 0.0;
      for (int k = 0; k < z; ++k) {
        const int32_t q = nbr[i * z + k];
        if (q < 0) continue;
        const double J = jnat ? jnat[i * z + k] : t.J;
        acc += -J * (si * (double)s[q]);
      }
      e = acc;
    }
    if (t.has_anisotropy) {
      const double d = si * t.axis_sign;
      e += d * d * t.K;
    }
    if (t.has_zeeman) e += t.hz * (si * t.field_sign);
    if (t.has_gauge) e += t.gauge;
    out[i] = e;
  }
}

__global__ void heis_site_energy_kernel(const double* __restrict__ s, int64_t n, int z,
                                        const int32_t* __restrict__ nbr, const double* __restrict__ jnat,
                                        SiteTerms t, double* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double x = s[3 * i], y = s[3 * i + 1], w = s[3 * i + 2];
    double e = 0.0;
    if (t.has_exchange) {
      double acc = 0.0;
      for (int k = 0; k < z; ++k) {
        const int32_t q = nbr[i * z + k];
        if (q < 0) continue;
        const double J = jnat ? jnat[i * z + k] : t.J;
        acc += -J * (x * s[3 * q] + y * s[3 * q + 1] + w * s[3 * q + 2]);
      }
      e = acc;
    }
    if (t.has_anisotropy) {
      const double d = x * t.axis[0] + y * t.axis[1] + w * t.axis[2];
      e += d * d * t.K;
    }
    if (t.has_zeeman) e += t.hz * (x * t.b[0] + y * t.b[1] + w * t.b[2]);
    if (t.has_gauge) e += t.gauge;
    if (t.has_cubic) {
      const V3<double> v = {x, y, w};
      e += -t.Kc * quart(v);
    }
    out[i] = e;
  }
}

// dE of replacing spin i by prop[i] with every other spin as it is, in R:
// the neighbour field is summed in R from the R-valued state in neighbour
// table order (per-bond constants weigh it when jnat is set, with P.J = 1).
template <typename R>
__global__ void heis_delta_kernel(const double* __restrict__ s, const double* __restrict__ prop, int64_t n, int z,
                                  const int32_t* __restrict__ nbr, const double* __restrict__ jnat, HeisParams<R> P,
                                  double* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    V3<R> h = {(R)0, (R)0, (R)0};
    for (int k = 0; k < z; ++k) {
      const int32_t q = nbr[i * z + k];
      if (q < 0) continue;
      const R J = jnat ? (R)jnat[i * z + k] : (R)1;
      h.x += J * (R)s[3 * q];
      h.y += J * (R)s[3 * q + 1];
      h.z += J * (R)s[3 * q + 2];
    }
    const V3<R> si = {(R)s[3 * i], (R)s[3 * i + 1], (R)s[3 * i + 2]};
    const V3<R> p = {(R)prop[3 * i], (R)prop[3 * i + 1], (R)prop[3 * i + 2]};
    out[i] = (double)heis_delta_e<R>(si, p, h, P);
  }
}

int grid_for(int64_t n) { return (int)std::min<int64_t>((n + 255) / 256, 4096); }

}  // namespace

cudaError_t launch_site_energies(bool ising, const void* spins, int64_t n, int z, const int32_t* nbr,
                                 const double* jnat, const SiteTerms& t, double* out, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  if (ising)
    ising_site_energy_kernel<<<grid_for(n), 256, 0, s>>>((const int8_t*)spins, n, z, nbr, jnat, t, out);
  else
    heis_site_energy_kernel<<<grid_for(n), 256, 0, s>>>((const double*)spins, n, z, nbr, jnat, t, out);
  return cudaGetLastError();
}

template <typename R>
cudaError_t launch_heis_delta(const double* spins, const double* prop, int64_t n, int z, const int32_t* nbr,
                              const double* jnat, const HeisParams<R>& P, double* out, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  heis_delta_kernel<R><<<grid_for(n), 256, 0, s>>>(spins, prop, n, z, nbr, jnat, P, out);
  return cudaGetLastError();
}

template cudaError_t launch_heis_delta<float>(const double*, const double*, int64_t, int, const int32_t*,
                                              const double*, const HeisParams<float>&, double*, cudaStream_t);
template cudaError_t launch_heis_delta<double>(const double*, const double*, int64_t, int, const int32_t*,
                                               const double*, const HeisParams<double>&, double*, cudaStream_t);

}  // namespace vg
