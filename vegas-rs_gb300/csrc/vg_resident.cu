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
// to the grid path.  When every thread holds at most one site per class
// (lattices up to 2,048 sites) the neighbour indices are formed once per
// launch and the first digit's block starts before the neighbour loads; up
// to 1,024 sites the sixteen threads of a group also share the first-digit
// blocks of eight sweeps (one Philox block per thread per eight sweeps).
// The sweep sums go through double-buffered shared slots, so a sweep costs
// two block barriers.
#include <cuda_runtime.h>

#include <algorithm>

#include "vg_internal.cuh"

namespace vg {

namespace {

__device__ __forceinline__ uint32_t block_byte_k(const uint4& b, int k) {
  const uint32_t w = (k >> 2) == 0 ? b.x : (k >> 2) == 1 ? b.y : (k >> 2) == 2 ? b.z : b.w;
  return (w >> (8 * (k & 3))) & 0xFFu;
}

// Shared-memory indices (in the other class) of the neighbours of class-C
// entry j; -1 where an open axis drops the bond.
__device__ __forceinline__ void resident_nbrs(const IsingScArgs& a, int C, uint32_t j, int (&nb)[6]) {
  const int row = (int)fdiv(j >> 4, a.fG);  // a row holds G groups of 16
  const int h = (int)(j - (uint32_t)row * a.Hx);
  const int z = (int)fdiv((uint32_t)row, a.fLy);
  const int y = row - z * a.Ly;
  const int p = (y + z + C) & 1;
  const int rb = row * a.Hx;
  const int plane = a.Ly * a.Hx;
  nb[0] = rb + h;
  const int hx = p ? h + 1 : h - 1;
  nb[1] = (hx >= 0 && hx < a.Hx) ? rb + hx : (a.pbx ? rb + (hx < 0 ? a.Hx - 1 : 0) : -1);
  nb[2] = y > 0 ? rb - a.Hx + h : (a.pby ? rb + (a.Ly - 1) * a.Hx + h : -1);
  nb[3] = y < a.Ly - 1 ? rb + a.Hx + h : (a.pby ? rb - (a.Ly - 1) * a.Hx + h : -1);
  nb[4] = z > 0 ? rb - plane + h : (a.pbz ? rb + (a.Lz - 1) * plane + h : -1);
  nb[5] = z < a.Lz - 1 ? rb + plane + h : (a.pbz ? rb - (a.Lz - 1) * plane + h : -1);
}

// One site's update in a colour pass; adds to the sweep's sums.
// r0: the word of the first digit's block holding this site's byte, when the
// caller already has it (otherwise null: the block is drawn here).
template <int PROP>
__device__ __forceinline__ void resident_site(int C, uint32_t j, const int (&nb)[6], uint8_t* own,
                                              const uint8_t* oth, const unsigned long long* s_thr,
                                              const RngKey& key, uint32_t sweep, const uint32_t* r0, int& bond,
                                              int& ups, int& nacc) {
  const uint32_t g = j >> 4;
  const int k = (int)(j & 15u);
  // the first digit's block does not depend on the spins: start it first
  uint4 b0 = make_uint4(0u, 0u, 0u, 0u);
  if (r0) b0.x = b0.y = b0.z = b0.w = *r0;
  else b0 = philox_ks(make_uint4(g, sweep, (kTagIsingAccept << 24) | ((uint32_t)C << 8), key.replica), key.ks);
  int nsum = 0;
#pragma unroll
  for (int i = 0; i < 6; ++i)
    if (nb[i] >= 0) nsum += 2 * (int)oth[nb[i]] - 1;
  const uint32_t s01 = own[j];
  bool cand = true;
  if (PROP == VG_PROPOSE_RANDOM) {
    const uint4 pb = philox_ks(make_uint4(g, sweep, (kTagIsingPropose << 24) | ((uint32_t)C << 8), key.replica),
                               key.ks);
    cand = (block_byte_k(pb, k) < 128 ? 1u : 0u) != s01;
  }
  bool acc = false;
  if (cand) {
    const unsigned long long th = s_thr[s01 * 13 + nsum + 6];
    if (th >= (1ull << 32)) {
      acc = true;
    } else if (th > 0ull) {
      uint32_t ub = block_byte_k(b0, k), tb = ((uint32_t)th >> 24) & 0xFFu;
      if (ub != tb) {
        acc = ub < tb;
      } else {  // tie on the first digit (probability 1/256): later digits
        for (int d = 1; d < 4; ++d) {
          const uint4 bd = philox_ks(
              make_uint4(g, sweep, (kTagIsingAccept << 24) | ((uint32_t)C << 8) | (uint32_t)d, key.replica), key.ks);
          ub = block_byte_k(bd, k);
          tb = ((uint32_t)th >> (24 - 8 * d)) & 0xFFu;
          if (ub != tb) {
            acc = ub < tb;
            break;
          }
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

// MAXT: the block bound.  Lattices of up to 1,024 sites run 512 threads at
// most, with the registers to keep the neighbours and the shared first-digit
// blocks without spilling (sc 32x32x1: 0.77 -> 0.91 flips/ns); larger ones
// run up to 1,024 threads and draw each pass's block per site (a 512-thread
// bound there would put two sites on a thread: 2,048 sites 0.98 -> 0.69).
template <int PROP, int MAXT>
__global__ void __launch_bounds__(MAXT) ising_resident_kernel(IsingScArgs a, IsingTable tab, RngKey key,
                                                              uint32_t n_sweeps, double* __restrict__ sums) {
  extern __shared__ uint8_t s_spin[];  // class 0 then class 1, n_c bytes each
  __shared__ unsigned long long s_thr[2 * 13];
  __shared__ int s_red[2][3][32];      // per sweep parity: no barrier after the read
  const uint32_t n_c = a.groups * 16u;
  uint8_t* cls[2] = {s_spin, s_spin + n_c};
  for (uint32_t i = threadIdx.x; i < n_c; i += blockDim.x) {
    cls[0][i] = a.cls[0][i];
    cls[1][i] = a.cls[1][i];
  }
  for (int i = threadIdx.x; i < 26; i += blockDim.x) s_thr[i] = tab.thr[i];
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = (int)(blockDim.x >> 5);
  // at most one site per thread and class: its neighbours once per launch
  constexpr bool kShare = MAXT <= 512;  // shared first-digit blocks
  const bool one = n_c <= blockDim.x;
  const bool mine = threadIdx.x < n_c;
  int nb0[6], nb1[6];
  if (one && mine) {
    resident_nbrs(a, 0, threadIdx.x, nb0);
    resident_nbrs(a, 1, threadIdx.x, nb1);
  }
  // One site per thread: the sixteen lanes of a half warp share one group,
  // so every eight sweeps lane i of the half warp draws the first-digit
  // block of colour pass i (sweep i / 2, colour i % 2) and each pass takes
  // its site's word from that lane by shuffles: one Philox block per lane
  // per eight sweeps instead of one per pass.
  uint4 blk = make_uint4(0u, 0u, 0u, 0u);
  const uint32_t grp = threadIdx.x >> 4, wq = (threadIdx.x >> 2) & 3u;
  for (uint32_t t = 0; t < n_sweeps; ++t) {
    const uint32_t sweep = key.sweep + t;
    if (kShare && one && (t & 7u) == 0u) {
      const uint32_t pi = (uint32_t)lane & 15u;
      blk = philox_ks(make_uint4(grp, sweep + (pi >> 1), (kTagIsingAccept << 24) | ((pi & 1u) << 8), key.replica),
                      key.ks);
    }
    int bond = 0, ups = 0, nacc = 0;
#pragma unroll
    for (int C = 0; C < 2; ++C) {
      uint8_t* own = cls[C];
      const uint8_t* oth = cls[C ^ 1];
      if (kShare && one) {
        const int src = (lane & 16) | (int)(2u * (t & 7u) + (uint32_t)C);
        const uint32_t w0 = __shfl_sync(0xffffffffu, blk.x, src), w1 = __shfl_sync(0xffffffffu, blk.y, src),
                       w2 = __shfl_sync(0xffffffffu, blk.z, src), w3 = __shfl_sync(0xffffffffu, blk.w, src);
        const uint32_t r0 = wq == 0 ? w0 : wq == 1 ? w1 : wq == 2 ? w2 : w3;
        if (mine)
          resident_site<PROP>(C, threadIdx.x, C ? nb1 : nb0, own, oth, s_thr, key, sweep, &r0, bond, ups, nacc);
      } else if (one) {
        if (mine)
          resident_site<PROP>(C, threadIdx.x, C ? nb1 : nb0, own, oth, s_thr, key, sweep, nullptr, bond, ups, nacc);
      } else {
        for (uint32_t j = threadIdx.x; j < n_c; j += blockDim.x) {
          int nb[6];
          resident_nbrs(a, C, j, nb);
          resident_site<PROP>(C, j, nb, own, oth, s_thr, key, sweep, nullptr, bond, ups, nacc);
        }
      }
      if (C == 0) __syncthreads();
    }
    // sweep sums: per warp (one warp-reduce instruction each), then over the
    // warps by warp 0, off the next pass's path
    bond = __reduce_add_sync(0xffffffffu, bond);
    ups = __reduce_add_sync(0xffffffffu, ups);
    nacc = __reduce_add_sync(0xffffffffu, nacc);
    int (*red)[32] = s_red[t & 1];
    if (lane == 0) {
      red[0][warp] = bond;
      red[1][warp] = ups;
      red[2][warp] = nacc;
    }
    __syncthreads();  // also ends the class-1 pass
    if (warp == 0 && sums) {
      int b = lane < nwarp ? red[0][lane] : 0, u = lane < nwarp ? red[1][lane] : 0,
          c = lane < nwarp ? red[2][lane] : 0;
      b = __reduce_add_sync(0xffffffffu, b);
      u = __reduce_add_sync(0xffffffffu, u);
      c = __reduce_add_sync(0xffffffffu, c);
      if (lane == 0) {
        double* o = sums + (size_t)t * kNumSums;
        o[0] = (double)b;
        o[1] = o[2] = o[3] = o[4] = o[5] = 0.0;
        o[6] = (double)u;
        o[7] = (double)c;
      }
    }
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < n_c; i += blockDim.x) {
    a.cls[0][i] = cls[0][i];
    a.cls[1][i] = cls[1][i];
  }
}

}  // namespace

size_t ising_resident_smem(const IsingScArgs& a) { return (size_t)a.groups * 16u * 2u; }

namespace {

template <int PROP, int MAXT>
cudaError_t launch_resident(const IsingScArgs& a, const IsingTable& tab, RngKey key, uint32_t n_sweeps,
                            double* sums, int tpb, size_t smem, cudaStream_t s) {
  const cudaError_t e = cudaFuncSetAttribute(ising_resident_kernel<PROP, MAXT>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  ising_resident_kernel<PROP, MAXT><<<1, std::min(tpb, MAXT), smem, s>>>(a, tab, key, n_sweeps, sums);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_ising_resident(const IsingScArgs& a, const IsingTable& tab, RngKey key, int proposal,
                                  uint32_t n_sweeps, double* sums, int tpb, cudaStream_t s) {
  const size_t smem = ising_resident_smem(a);
  const bool small = a.groups * 16u <= 512u;  // one site per thread within 512 threads
  if (proposal == VG_PROPOSE_RANDOM)
    return small ? launch_resident<VG_PROPOSE_RANDOM, 512>(a, tab, key, n_sweeps, sums, tpb, smem, s)
                 : launch_resident<VG_PROPOSE_RANDOM, 1024>(a, tab, key, n_sweeps, sums, tpb, smem, s);
  return small ? launch_resident<VG_PROPOSE_FLIP, 512>(a, tab, key, n_sweeps, sums, tpb, smem, s)
               : launch_resident<VG_PROPOSE_FLIP, 1024>(a, tab, key, n_sweeps, sums, tpb, smem, s);
}

}  // namespace vg
