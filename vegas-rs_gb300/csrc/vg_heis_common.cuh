// vg_heis_common.cuh -- device code shared by the Heisenberg kernels of the
// single-lattice passes (vg_heis.cu) and of the batched replicas
// (vg_hbatch.cu): the proposal / acceptance step, the per-site sums and
// their block reduction, the vector load helpers and the initial-state map.
// Both paths draw the same Philox blocks for the same (seed, replica, sweep,
// colour, class entry), so a replica of the batch follows the single-lattice
// trajectory of the same seed.
#pragma once

#include "vg_internal.cuh"

namespace vg {

__device__ __forceinline__ void sincospi_(float t, float* s, float* c) { sincospif(t, s, c); }
__device__ __forceinline__ void sincospi_(double t, double* s, double* c) { sincospi(t, s, c); }
__device__ __forceinline__ float sqrt_(float x) { return sqrtf(x); }
__device__ __forceinline__ double sqrt_(double x) { return sqrt(x); }
__device__ __forceinline__ float exp_(float x) { return expf(x); }
__device__ __forceinline__ double exp_(double x) { return exp(x); }

// Uniform variates from Philox words without the integer-to-float
// conversion instruction (it issues to the FP64 pipe, which is narrow on
// this part): k * 2^-24 for k < 2^24 is built exactly from the 23 high bits
// as the mantissa of a number in [1, 2), minus 1, plus 2^-24 if k is odd.
__device__ __forceinline__ float u24_unit(uint32_t k) {
  const float hi = __uint_as_float(0x3F800000u | (k >> 1)) - 1.0f;
  return hi + __uint_as_float((k & 1u) * 0x33800000u);
}

// (2k + 1 - 2^24) * 2^-24 for k < 2^24 (an odd multiple of 2^-24 in (-1, 1)).
__device__ __forceinline__ float z_unit(uint32_t k) {
  const int m = (int)(k << 1) + 1 - (1 << 24);
  const uint32_t a = (uint32_t)(m < 0 ? -m : m);
  return __uint_as_float(__float_as_uint(u24_unit(a)) | ((uint32_t)m & 0x80000000u));
}

// The three variates of a proposal and its acceptance: z in (-1, 1), the
// azimuth t in [0, 2) (angle pi t) and u in [0, 1), each a 24-bit value.
template <typename R>
__device__ __forceinline__ void draw_zt(const uint4& w, R& z, R& t) {
  if constexpr (sizeof(R) == 4) {
    z = z_unit(w.x >> 8);
    t = 2.0f * u24_unit(w.y >> 8);
  } else {
    z = (R)((int)((w.x >> 8) << 1) + 1 - (1 << 24)) * (R)(1.0 / 16777216.0);
    t = (R)(w.y >> 8) * (R)(1.0 / 8388608.0);
  }
}

template <typename R>
__device__ __forceinline__ R draw_u(const uint4& w) {
  if constexpr (sizeof(R) == 4) return u24_unit(w.z >> 8);
  else return (R)(w.z >> 8) * (R)(1.0 / 16777216.0);
}

template <typename R>
struct V3 {
  R x, y, z;
};

template <typename R>
__device__ __forceinline__ R quart(const V3<R>& s) {
  const R a = s.x * s.x, b = s.y * s.y, c = s.z * s.z;
  return a * a + b * b + c * c;
}

// Energy change of replacing spin s by p at a site whose neighbour field
// (sum of J_ij s_j, or of s_j with P.J the uniform constant) is h: the
// difference of the site's Compound energy (src/energy.rs:108-112, 147-152,
// 194-208) plus the cubic term -Kc (sx^4 + sy^4 + sz^4).
template <typename R>
__device__ __forceinline__ R heis_delta_e(const V3<R>& s, const V3<R>& p, const V3<R>& h, const HeisParams<R>& P) {
  const R dx = p.x - s.x, dy = p.y - s.y, dz = p.z - s.z;
  const R pe = p.x * P.ax + p.y * P.ay + p.z * P.az;
  const R se = s.x * P.ax + s.y * P.ay + s.z * P.az;
  R de = -P.J * (dx * h.x + dy * h.y + dz * h.z);
  de += P.K * (pe * pe - se * se);
  de += P.hz * (dx * P.bx + dy * P.by + dz * P.bz);
  if (P.Kc != (R)0) de -= P.Kc * (quart(p) - quart(s));  // skipped: the same value without the two quartics
  return de;
}

// Proposal and acceptance draw of one site; returns the new spin and whether
// it was accepted.
//
// The FP32 kernels form the proposal's sine and cosine, its sqrt(1 - z^2)
// and the acceptance exponential with CUDA's fast intrinsics: __sinf /
// __cosf of x = pi (t - 1) in [-pi, pi) (sin(pi t) = -sin x, cos(pi t) =
// -cos x; absolute error below 2^-21.4 there), w rsqrt(w) for sqrt(w)
// (w >= 2^-23: z = (2k + 1 - 2^24) 2^-24 never reaches +-1), and __expf.
// The proposal components then lie within 5e-7 of the FP64 kernels' (the
// FP32 tolerance against the FP64 oracle is 2e-6), and a decision differs
// only where u lies within a few ulp of exp(-dE / T).  The FP64 kernels
// use sincospi, sqrt and exp.
template <typename R, int PROP>
__device__ __forceinline__ bool heis_update(const V3<R>& s, const V3<R>& h, const HeisParams<R>& P, const uint4& w,
                                            V3<R>& out) {
  V3<R> p;
  if (PROP == VG_PROPOSE_RANDOM) {
    // z = (2k + 1 - 2^24) / 2^24 is exact in FP32; azimuth pi * t, t in [0, 2)
    R z, t;
    draw_zt<R>(w, z, t);
    R sn, cs, r;
    if constexpr (sizeof(R) == 4) {
      const float x = 3.14159265358979f * (t - 1.0f);  // t - 1 is exact
      sn = -__sinf(x);
      cs = -__cosf(x);
      const float w2 = (1.0f - z) * (1.0f + z);
      r = w2 * rsqrtf(w2);
    } else {
      sincospi_(t, &sn, &cs);
      r = sqrt_(((R)1 - z) * ((R)1 + z));
    }
    p.x = r * cs;
    p.y = r * sn;
    p.z = z;
  } else {
    p.x = -s.x;
    p.y = -s.y;
    p.z = -s.z;
  }
  const R de = heis_delta_e<R>(s, p, h, P);
  const R u = draw_u<R>(w);
  R q;
  if constexpr (sizeof(R) == 4) q = __expf(-de * P.beta);
  else q = exp_(-de * P.beta);
  const bool acc = de <= (R)0 || u < q;
  out = acc ? p : s;
  return acc;
}

template <typename R>
__device__ __forceinline__ void add_site_sums(R (&acc)[kNumSums], const V3<R>& s, const V3<R>& low,
                                              const HeisParams<R>& P) {
  const R se = s.x * P.ax + s.y * P.ay + s.z * P.az;
  acc[0] += s.x * low.x + s.y * low.y + s.z * low.z;
  acc[1] += se * se;
  acc[2] += s.x * P.bx + s.y * P.by + s.z * P.bz;
  acc[3] += quart(s);
  acc[4] += s.x;
  acc[5] += s.y;
  acc[6] += s.z;
}

// Thread partials in R, warp sums in R, the block's warps summed in R in a
// fixed order by threads 0..kNumSums-1, which store the block row of
// kNumSums doubles (FP32 kernels convert once per value: the FP64 pipe is
// narrow, and the FP64 combination happens across blocks).
template <typename R>
__device__ __forceinline__ void flush_sums(R (&acc)[kNumSums], double* part) {
  __shared__ R red[32][kNumSums];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < kNumSums; ++i) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc[i] += __shfl_down_sync(0xffffffffu, acc[i], o);
  }
  if (lane == 0) {
#pragma unroll
    for (int i = 0; i < kNumSums; ++i) red[warp][i] = acc[i];
  }
  __syncthreads();
  if (threadIdx.x < kNumSums) {
    R t = (R)0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w][threadIdx.x];
    part[(size_t)blockIdx.x * kNumSums + threadIdx.x] = (double)t;
  }
}

// Runs of four consecutive entries of one SoA plane (16-byte aligned).
template <typename R>
struct Vec4 {
  R v[4];
};
__device__ __forceinline__ Vec4<float> ld4(const float* p) {
  const float4 t = __ldg(reinterpret_cast<const float4*>(p));
  return Vec4<float>{{t.x, t.y, t.z, t.w}};
}
__device__ __forceinline__ Vec4<double> ld4(const double* p) {
  const double2 a = __ldg(reinterpret_cast<const double2*>(p)), b = __ldg(reinterpret_cast<const double2*>(p) + 1);
  return Vec4<double>{{a.x, a.y, b.x, b.y}};
}
__device__ __forceinline__ void st4(float* p, const Vec4<float>& v) {
  *reinterpret_cast<float4*>(p) = make_float4(v.v[0], v.v[1], v.v[2], v.v[3]);
}
__device__ __forceinline__ void st4(double* p, const Vec4<double>& v) {
  reinterpret_cast<double2*>(p)[0] = make_double2(v.v[0], v.v[1]);
  reinterpret_cast<double2*>(p)[1] = make_double2(v.v[2], v.v[3]);
}

// State::rand_with_size for Heisenberg (src/state.rs:260-262): the same
// uniform-on-sphere map as the proposals, from block (site, 0, tag, replica).
template <typename R>
__device__ __forceinline__ V3<R> heis_init_spin(uint32_t site, const RngKey& key) {
  const uint4 w = philox(make_uint4(site, 0u, kTagInitHeis << 24, key.replica), key.k0, key.k1);
  const R z = (R)((int)((w.x >> 8) << 1) + 1 - (1 << 24)) * (R)(1.0 / 16777216.0);
  const R t = (R)(w.y >> 8) * (R)(1.0 / 8388608.0);
  R sn, cs;
  if (sizeof(R) == 4) {
    float a, b;
    sincospif((float)t, &a, &b);
    sn = (R)a;
    cs = (R)b;
  } else {
    double a, b;
    sincospi((double)t, &a, &b);
    sn = (R)a;
    cs = (R)b;
  }
  const R r = (R)sqrt((double)(((R)1 - z) * ((R)1 + z)));
  return V3<R>{r * cs, r * sn, z};
}

}  // namespace vg
