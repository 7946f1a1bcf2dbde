// vg_wolff.cu -- Wolff cluster steps for Ising spins (WolffIntegrator::step,
// src/integrator.rs:140-230), all steps of a call in one thread block.
//
// A step picks a source site, grows the cluster of aligned spins joined by
// active bonds and flips it.  Every bond of the lattice carries its own
// random number per step, Philox(min site, max site, tag | occurrence |
// replica, step): a bond is active iff that word is below
// ceil((1 - exp(-2 J / T)) 2^32).  The cluster is the connected component of
// the source in the graph of active bonds between spins equal to the
// source's, which is what the reference's queue builds (it tries each bond
// from the cluster to an aligned outside neighbour once, with probability
// p), and it does not depend on the order in which the frontier is
// expanded.  Repeated bonds between one pair of sites (a periodic axis of
// extent 2) are distinct bonds (occurrence 0, 1, ...), as in the
// reference's neighbour list.
//
// The block keeps the spins (int8 +-1, natural site order), a cluster bit
// mask and two frontier lists in shared memory and expands the frontier one
// level per round; after the flip it writes the step's raw sums (bond sum,
// up spins, cluster size) in the layout of the Metropolis kernels.
#include <cuda_runtime.h>

#include "vg_internal.cuh"

namespace vg {

namespace {

constexpr uint32_t kTagWolffSource = 9, kTagWolffBond = 10;

__global__ void __launch_bounds__(1024) ising_wolff_kernel(int8_t* __restrict__ spins, int n, int z,
                                                           const int32_t* __restrict__ nbr,
                                                           const uint8_t* __restrict__ occ,
                                                           unsigned long long thr, RngKey key, uint32_t n_steps,
                                                           double* __restrict__ sums) {
  extern __shared__ uint32_t s_mem[];
  uint32_t* inc = s_mem;                            // cluster bits, (n + 31) / 32 words
  int32_t* fa = (int32_t*)(inc + ((n + 31) >> 5));  // frontier lists
  int32_t* fb = fa + n;
  int8_t* s = (int8_t*)(fb + n);
  __shared__ int s_count[2];
  __shared__ int s_src;
  __shared__ int s_red[3][32];
  const int nw = (n + 31) >> 5;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s[i] = spins[i];
  __syncthreads();
  for (uint32_t t = 0; t < n_steps; ++t) {
    const uint32_t step = key.sweep + t;
    for (int i = threadIdx.x; i < nw; i += blockDim.x) inc[i] = 0u;
    if (threadIdx.x == 0) {
      const uint4 w = philox_ks(make_uint4(step, 0u, kTagWolffSource << 24, key.replica), key.ks);
      s_src = (int)(((unsigned long long)w.x * (unsigned long long)n) >> 32);
      s_count[0] = 1;
      s_count[1] = 0;
    }
    __syncthreads();
    const int src = s_src;
    const int8_t ref = s[src];
    if (threadIdx.x == 0) {
      inc[src >> 5] = 1u << (src & 31);
      fa[0] = src;
    }
    __syncthreads();
    int32_t* cur = fa;
    int32_t* nxt = fb;
    int ci = 0;
    int na = 1;
    while (na > 0) {
      for (int e = threadIdx.x; e < na; e += blockDim.x) {
        const int site = cur[e];
        for (int k = 0; k < z; ++k) {
          const int j = __ldg(nbr + (size_t)site * z + k);
          if (j < 0 || s[j] != ref) continue;
          if ((inc[j >> 5] >> (j & 31)) & 1u) continue;
          const uint32_t lo = (uint32_t)min(site, j), hi = (uint32_t)max(site, j);
          const uint32_t o = __ldg(occ + (size_t)site * z + k);
          const uint4 w = philox_ks(make_uint4(lo, hi, (kTagWolffBond << 24) | (o << 20) | (key.replica & 0xFFFFFu), step),
                                    key.ks);
          if ((unsigned long long)w.x < thr) {
            const uint32_t bit = 1u << (j & 31);
            if (!(atomicOr(&inc[j >> 5], bit) & bit)) nxt[atomicAdd(&s_count[ci ^ 1], 1)] = j;
          }
        }
      }
      __syncthreads();
      na = s_count[ci ^ 1];
      __syncthreads();
      if (threadIdx.x == 0) s_count[ci] = 0;  // the list just consumed becomes the next one to fill
      int32_t* tmp = cur;
      cur = nxt;
      nxt = tmp;
      ci ^= 1;
      __syncthreads();
    }
    // flip the cluster, then this step's sums
    int ups = 0, csize = 0, bond = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const bool in = (inc[i >> 5] >> (i & 31)) & 1u;
      if (in) s[i] = (int8_t)(-s[i]);
      csize += in;
    }
    __syncthreads();
    if (sums) {
      for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int si = s[i];
        ups += si > 0;
        for (int k = 0; k < z; ++k) {  // each bond once, from its lower site
          const int j = __ldg(nbr + (size_t)i * z + k);
          if (j > i) bond += si * s[j];
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        bond += __shfl_down_sync(0xffffffffu, bond, o);
        ups += __shfl_down_sync(0xffffffffu, ups, o);
        csize += __shfl_down_sync(0xffffffffu, csize, o);
      }
      if (lane == 0) {
        s_red[0][warp] = bond;
        s_red[1][warp] = ups;
        s_red[2][warp] = csize;
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        long long b = 0, u = 0, cs = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
          b += s_red[0][w];
          u += s_red[1][w];
          cs += s_red[2][w];
        }
        double* out = sums + (size_t)t * kNumSums;
        out[0] = (double)b;
        out[1] = out[2] = out[3] = out[4] = out[5] = 0.0;
        out[6] = (double)u;
        out[7] = (double)cs;
      }
      __syncthreads();
    }
  }
  for (int i = threadIdx.x; i < n; i += blockDim.x) spins[i] = s[i];
}

}  // namespace

size_t ising_wolff_smem(int n) { return (size_t)((n + 31) / 32) * 4 + (size_t)n * 8 + (size_t)n; }

cudaError_t launch_ising_wolff(int8_t* spins, int n, int z, const int32_t* nbr, const uint8_t* occ,
                               unsigned long long thr, RngKey key, uint32_t n_steps, double* sums, cudaStream_t s) {
  const size_t smem = ising_wolff_smem(n);
  cudaError_t e = cudaFuncSetAttribute(ising_wolff_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const int tpb = n >= 1024 ? 1024 : ((n + 31) / 32) * 32;
  ising_wolff_kernel<<<1, tpb, smem, s>>>(spins, n, z, nbr, occ, thr, key, n_steps, sums);
  return cudaGetLastError();
}

}  // namespace vg
