// vg_resident.cu -- Ising sweeps of a small lattice held in one thread
// block's shared memory, many sweeps per launch.
//
// For lattices of a few thousand sites (the reference's own CPU examples,
// e.g. 32x32 with open z under a 39-temperature CoolDown of 21,000 sweeps
// each) a colour pass is far shorter than a kernel launch.  One block loads
// both checkerboard classes into shared memory, runs all n sweeps of a
// vg_sweeps call with a block barrier between colour passes, writes each
// sweep's raw sums (bond sum, up spins, accepted moves) and stores the spins
// back.  One thread handles one site per step: it forms the neighbour sum,
// looks up the site's threshold and compares its 32-bit uniform digit by
// digit with the same Philox blocks the grid kernels use (byte (j & 15) of
// block (j >> 4, sweep, tag, colour | digit)), so results are bit-identical
// to the grid path.
#include <cuda_runtime.h>

#include "vg_internal.cuh"

namespace vg {

namespace {

__device__ __forceinline__ uint32_t block_byte_k(const uint4& b, int k) {
  const uint32_t w = (k >> 2) == 0 ? b.x : (k >> 2) == 1 ? b.y : (k >> 2) == 2 ? b.z : b.w;
  return (w >> (8 * (k & 3))) & 0xFFu;
}

template <int PROP>
__global__ void __launch_bounds__(1024) ising_resident_kernel(IsingScArgs a, IsingTable tab, RngKey key,
                                                              uint32_t n_sweeps, double* __restrict__ sums) {
  extern __shared__ uint8_t s_spin[];  // class 0 then class 1, n_c bytes each
  __shared__ unsigned long long s_thr[2 * 13];
  __shared__ int s_red[3][32];
  const uint32_t n_c = a.groups * 16u;
  uint8_t* cls[2] = {s_spin, s_spin + n_c};
  for (uint32_t i = threadIdx.x; i < n_c; i += blockDim.x) {
    cls[0][i] = a.cls[0][i];
    cls[1][i] = a.cls[1][i];
  }
  for (int i = threadIdx.x; i < 26; i += blockDim.x) s_thr[i] = tab.thr[i];
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (uint32_t t = 0; t < n_sweeps; ++t) {
    const uint32_t sweep = key.sweep + t;
    int bond = 0, ups = 0, nacc = 0;
    for (int C = 0; C < 2; ++C) {
      uint8_t* own = cls[C];
      const uint8_t* oth = cls[C ^ 1];
      for (uint32_t j = threadIdx.x; j < n_c; j += blockDim.x) {
        const int row = (int)fdiv(j >> 4, a.fG);  // a row holds G groups of 16
        const int h = (int)(j - (uint32_t)row * a.Hx);
        const int z = (int)fdiv((uint32_t)row, a.fLy);
        const int y = row - z * a.Ly;
        const int p = (y + z + C) & 1;
        const int rb = row * a.Hx;
        int nsum = 0, nb = 0;
        auto add = [&](int q) {
          nsum += 2 * (int)oth[q] - 1;
          ++nb;
        };
        add(rb + h);
        const int hx = p ? h + 1 : h - 1;
        if (hx >= 0 && hx < a.Hx) add(rb + hx);
        else if (a.pbx) add(rb + (hx < 0 ? a.Hx - 1 : 0));
        if (y > 0) add(rb - a.Hx + h);
        else if (a.pby) add(rb + (a.Ly - 1) * a.Hx + h);
        if (y < a.Ly - 1) add(rb + a.Hx + h);
        else if (a.pby) add(rb - (a.Ly - 1) * a.Hx + h);
        const int plane = a.Ly * a.Hx;
        if (z > 0) add(rb - plane + h);
        else if (a.pbz) add(rb + (a.Lz - 1) * plane + h);
        if (z < a.Lz - 1) add(rb + plane + h);
        else if (a.pbz) add(rb - (a.Lz - 1) * plane + h);
        (void)nb;
        const uint32_t s01 = own[j];
        const uint32_t g = j >> 4;
        const int k = (int)(j & 15u);
        bool cand = true;
        if (PROP == VG_PROPOSE_RANDOM) {
          const uint4 pb = philox_ks(make_uint4(g, sweep, (kTagIsingPropose << 24) | ((uint32_t)C << 8), key.replica),
                                     key.ks);
          const uint32_t up = block_byte_k(pb, k) < 128 ? 1u : 0u;
          cand = up != s01;
        }
        bool acc = false;
        if (cand) {
          const unsigned long long th = s_thr[s01 * 13 + nsum + 6];
          if (th >= (1ull << 32)) {
            acc = true;
          } else if (th > 0ull) {
            for (int d = 0; d < 4; ++d) {
              const uint4 bd = philox_ks(
                  make_uint4(g, sweep, (kTagIsingAccept << 24) | ((uint32_t)C << 8) | (uint32_t)d, key.replica),
                  key.ks);
              const uint32_t ub = block_byte_k(bd, k), tb = ((uint32_t)th >> (24 - 8 * d)) & 0xFFu;
              if (ub != tb) {
                acc = ub < tb;
                break;
              }
            }
          }
        }
        const uint32_t sn = acc ? (s01 ^ 1u) : s01;
        if (acc) own[j] = (uint8_t)sn;
        ups += (int)sn;
        nacc += acc;
        if (C == 1) bond += sn ? nsum : -nsum;
      }
      __syncthreads();
    }
    // block sums of this sweep
    for (int o = 16; o > 0; o >>= 1) {
      bond += __shfl_down_sync(0xffffffffu, bond, o);
      ups += __shfl_down_sync(0xffffffffu, ups, o);
      nacc += __shfl_down_sync(0xffffffffu, nacc, o);
    }
    if (lane == 0) {
      s_red[0][warp] = bond;
      s_red[1][warp] = ups;
      s_red[2][warp] = nacc;
    }
    __syncthreads();
    if (threadIdx.x == 0 && sums) {
      long long b = 0, u = 0, c = 0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
        b += s_red[0][w];
        u += s_red[1][w];
        c += s_red[2][w];
      }
      double* o = sums + (size_t)t * kNumSums;
      o[0] = (double)b;
      o[1] = o[2] = o[3] = o[4] = o[5] = 0.0;
      o[6] = (double)u;
      o[7] = (double)c;
    }
    __syncthreads();
  }
  for (uint32_t i = threadIdx.x; i < n_c; i += blockDim.x) {
    a.cls[0][i] = cls[0][i];
    a.cls[1][i] = cls[1][i];
  }
}

}  // namespace

size_t ising_resident_smem(const IsingScArgs& a) { return (size_t)a.groups * 16u * 2u; }

cudaError_t launch_ising_resident(const IsingScArgs& a, const IsingTable& tab, RngKey key, int proposal,
                                  uint32_t n_sweeps, double* sums, int tpb, cudaStream_t s) {
  const size_t smem = ising_resident_smem(a);
  cudaError_t e;
  if (proposal == VG_PROPOSE_RANDOM) {
    e = cudaFuncSetAttribute(ising_resident_kernel<VG_PROPOSE_RANDOM>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
    if (e != cudaSuccess) return e;
    ising_resident_kernel<VG_PROPOSE_RANDOM><<<1, tpb, smem, s>>>(a, tab, key, n_sweeps, sums);
  } else {
    e = cudaFuncSetAttribute(ising_resident_kernel<VG_PROPOSE_FLIP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
    if (e != cudaSuccess) return e;
    ising_resident_kernel<VG_PROPOSE_FLIP><<<1, tpb, smem, s>>>(a, tab, key, n_sweeps, sums);
  }
  return cudaGetLastError();
}

}  // namespace vg
