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
// The block keeps the spins (int8 +-1, natural site order), a per-site
// stamp (the step that last put the site in a cluster, so that nothing is
// cleared between steps) and the cluster as one queue in shared memory.  The
// queue grows one breadth-first level per round, with one barrier a level:
// level L appends through counter L mod 3, whose value every thread reads
// after the barrier, and thread 0 zeroes the counter of level L + 2 then, two
// barriers before it is used again.  After the last level one pass over the
// cluster's bonds flips the cluster and sums the bonds it cuts, which updates
// the bond sum and the up count of the previous step instead of recounting
// the lattice: the step's raw sums (bond sum, up spins, cluster size) land in
// the layout of the Metropolis kernels.
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
  uint32_t* mark = s_mem;                  // step stamp + 1 of the last cluster holding the site
  int32_t* q = (int32_t*)(mark + n);       // the cluster, in breadth-first order
  int8_t* s = (int8_t*)(q + n);
  __shared__ int s_cnt[3];
  __shared__ int s_red[2][32];
  __shared__ int s_cut;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    s[i] = spins[i];
    mark[i] = 0u;
  }
  if (threadIdx.x < 3) s_cnt[threadIdx.x] = 0;
  if (threadIdx.x == 0) s_cut = 0;
  __syncthreads();
  // the bond sum and up count of the incoming state, once per call
  long long bond = 0, ups = 0;
  if (sums) {
    int b = 0, u = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const int si = s[i];
      u += si > 0;
      for (int k = 0; k < z; ++k) {  // each bond once, from its lower site
        const int j = __ldg(nbr + (size_t)i * z + k);
        if (j > i) b += si * s[j];
      }
    }
    b = __reduce_add_sync(0xffffffffu, b);
    u = __reduce_add_sync(0xffffffffu, u);
    if (lane == 0) {
      s_red[0][warp] = b;
      s_red[1][warp] = u;
    }
    __syncthreads();
    if (threadIdx.x == 0)
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
        bond += s_red[0][w];
        ups += s_red[1][w];
      }
  }
  for (uint32_t t = 0; t < n_steps; ++t) {
    const uint32_t step = key.sweep + t;
    const uint32_t stamp = t + 1;
    // the source depends on the step alone: every thread draws it
    const uint4 w0 = philox_ks(make_uint4(step, 0u, kTagWolffSource << 24, key.replica), key.ks);
    const int src = (int)(((unsigned long long)w0.x * (unsigned long long)n) >> 32);
    const int8_t ref = s[src];
    mark[src] = stamp;  // the same value from every thread
    if (threadIdx.x == 0) q[0] = src;
    int lo = 0, hi = 1, lev = 0;
    for (;;) {
      // one thread per (frontier site, neighbour slot) of this level
      const int items = (hi - lo) * z;
      int* cnt = &s_cnt[lev % 3];
      for (int e = threadIdx.x; e < items; e += blockDim.x) {
        const int fi = e / z, k = e - fi * z;
        const int site = lo == 0 ? src : q[lo + fi];
        const int j = __ldg(nbr + (size_t)site * z + k);
        if (j < 0 || s[j] != ref || mark[j] == stamp) continue;
        const uint32_t a = (uint32_t)min(site, j), b = (uint32_t)max(site, j);
        const uint32_t o = __ldg(occ + (size_t)site * z + k);
        const uint4 w = philox_ks(make_uint4(a, b, (kTagWolffBond << 24) | (o << 20) | (key.replica & 0xFFFFFu), step),
                                  key.ks);
        if ((unsigned long long)w.x < thr && atomicExch(&mark[j], stamp) != stamp) q[hi + atomicAdd(cnt, 1)] = j;
      }
      __syncthreads();
      const int added = *cnt;
      if (threadIdx.x == 0) s_cnt[(lev + 2) % 3] = 0;
      if (added == 0) break;
      lo = hi;
      hi += added;
      ++lev;
    }
    // flip the cluster and sum the spins across its boundary (the cluster's
    // sites only change, the boundary sites are only read)
    int cut = 0;
    for (int e = threadIdx.x; e < hi * z; e += blockDim.x) {
      const int fi = e / z, k = e - fi * z;
      const int site = q[fi];
      const int j = __ldg(nbr + (size_t)site * z + k);
      if (j >= 0 && mark[j] != stamp) cut += s[j];
      if (k == 0) s[site] = (int8_t)(-ref);
    }
    if (sums) {
      cut = __reduce_add_sync(0xffffffffu, cut);
      if (lane == 0 && cut) atomicAdd(&s_cut, cut);
    }
    __syncthreads();
    if (sums && threadIdx.x == 0) {
      // cut bonds change sign: bond sum -= 2 ref sum(boundary spins)
      bond -= 2ll * ref * s_cut;
      ups += ref > 0 ? -(long long)hi : (long long)hi;
      s_cut = 0;  // read again only after the next step's first barrier
      double* out = sums + (size_t)t * kNumSums;
      out[0] = (double)bond;
      out[1] = out[2] = out[3] = out[4] = out[5] = 0.0;
      out[6] = (double)ups;
      out[7] = (double)hi;
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) spins[i] = s[i];
}

// ------------------------------------------------------------ multi-block
// Lattices beyond one block's shared memory: one cooperative launch runs
// every step of a call with the same steps as above, the spins, stamps and
// queue in global memory (read through L2: other blocks write them within
// the launch), each level's frontier spread over the whole grid, and a grid
// barrier after every level and after the flip.  Appends are aggregated
// per warp.  A barrier wait gives up after two seconds: the block raises
// the abort flag, every block leaves at its next barrier, and the host
// reports the failure.

__device__ __forceinline__ unsigned int ld_acquire_gpu(const unsigned int* p) {
  unsigned int v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

constexpr unsigned long long kBarrierTimeoutNs = 2000000000ull;

__device__ __forceinline__ unsigned long long ld_acquire_gpu64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_gpu64(unsigned long long* p, unsigned long long v) {
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned int atom_add_acq_rel_gpu(unsigned int* p, unsigned int v) {
  unsigned int old;
  asm volatile("atom.add.acq_rel.gpu.global.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}
__device__ __forceinline__ unsigned int ld_relaxed_gpu(const unsigned int* p) {
  unsigned int v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// All blocks of the grid.  The release word carries (generation, value):
// the last block to arrive reads *fold (every block's writes before the
// barrier are visible to it) and hands it to all blocks with the release,
// so a level's append count costs no extra round trip.  Returns false when
// the barrier was abandoned (a wait ran out, here or in another block).
__device__ bool grid_barrier(WolffGrid* g, const unsigned int* fold, unsigned int* folded) {
  __shared__ int s_ok;
  __shared__ unsigned int s_fold;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    const unsigned int gen = (unsigned int)(ld_acquire_gpu64(&g->bar_word) >> 32);
    unsigned long long w;
    if (atom_add_acq_rel_gpu(&g->bar_count, 1u) == gridDim.x - 1) {
      g->bar_count = 0u;  // ordered before the release below
      w = ((unsigned long long)(gen + 1u) << 32) | (fold ? ld_relaxed_gpu(fold) : 0u);
      st_release_gpu64(&g->bar_word, w);
    } else {
      const unsigned long long t0 = global_ns();
      for (unsigned int k = 1;; ++k) {
        w = ld_acquire_gpu64(&g->bar_word);
        if ((unsigned int)(w >> 32) != gen) break;
        if ((k & 255u) == 0u && (ld_acquire_gpu(&g->abort_flag) || global_ns() - t0 > kBarrierTimeoutNs)) {
          atomicExch(&g->abort_flag, 1u);
          ok = 0;
          break;
        }
      }
    }
    s_ok = ok;
    s_fold = (unsigned int)w;
  }
  __syncthreads();
  if (folded) *folded = s_fold;
  return s_ok != 0;
}

__global__ void __launch_bounds__(kWolffGridTpb) ising_wolff_grid_kernel(
    int8_t* __restrict__ spins, int n, int z, const int32_t* __restrict__ nbr, const uint8_t* __restrict__ occ,
    unsigned long long thr, RngKey key, uint32_t n_steps, double* __restrict__ sums, uint32_t* __restrict__ mark,
    int32_t* __restrict__ q, WolffGrid* __restrict__ g) {
  const int lane = threadIdx.x & 31;
  const int gtid = blockIdx.x * blockDim.x + threadIdx.x, gsz = gridDim.x * blockDim.x;
  const bool lead = gtid == 0;
  for (int i = gtid; i < n; i += gsz) mark[i] = 0u;
  if (sums) {  // the bond sum and up count of the incoming state
    int b = 0, u = 0;
    for (int i = gtid; i < n; i += gsz) {
      const int si = spins[i];
      u += si > 0;
      for (int k = 0; k < z; ++k) {
        const int j = __ldg(nbr + (size_t)i * z + k);
        if (j > i) b += si * spins[j];
      }
    }
    b = __reduce_add_sync(0xffffffffu, b);
    u = __reduce_add_sync(0xffffffffu, u);
    if (lane == 0) {
      atomicAdd(&g->bond0, (unsigned long long)(long long)b);
      atomicAdd(&g->ups0, (unsigned long long)(long long)u);
    }
  }
  if (!grid_barrier(g, nullptr, nullptr)) return;
  long long bond = (long long)__ldcg(&g->bond0), ups = (long long)__ldcg(&g->ups0);
  for (uint32_t t = 0; t < n_steps; ++t) {
    const uint32_t step = key.sweep + t;
    const uint32_t stamp = t + 1;
    const uint4 w0 = philox_ks(make_uint4(step, 0u, kTagWolffSource << 24, key.replica), key.ks);
    const int src = (int)(((unsigned long long)w0.x * (unsigned long long)n) >> 32);
    const int8_t ref = __ldcg(spins + src);
    if (lead) {
      mark[src] = stamp;
      q[0] = src;
    }
    int lo = 0, hi = 1, lev = 0;
    for (;;) {
      const int items = (hi - lo) * z;
      unsigned int* cnt = &g->cnt[lev % 3];
      for (int base = gtid - lane; base < items; base += gsz) {
        const int e = base + lane;
        int j = -1;
        bool want = false;
        if (e < items) {
          const int fi = e / z, k = e - fi * z;
          const int site = lo == 0 ? src : __ldcg(q + lo + fi);
          j = __ldg(nbr + (size_t)site * z + k);
          if (j >= 0 && __ldcg(spins + j) == ref && __ldcg(mark + j) != stamp) {
            const uint32_t a = (uint32_t)min(site, j), b = (uint32_t)max(site, j);
            const uint32_t o = __ldg(occ + (size_t)site * z + k);
            const uint4 w = philox_ks(
                make_uint4(a, b, (kTagWolffBond << 24) | (o << 20) | (key.replica & 0xFFFFFu), step), key.ks);
            want = (unsigned long long)w.x < thr && atomicExch(mark + j, stamp) != stamp;
          }
        }
        const unsigned int m = __ballot_sync(0xffffffffu, want);
        if (m) {
          const int leader = __ffs(m) - 1;
          unsigned int pos = 0;
          if (lane == leader) pos = atomicAdd(cnt, (unsigned int)__popc(m));
          pos = __shfl_sync(0xffffffffu, pos, leader);
          if (want) q[hi + (int)pos + __popc(m & ((1u << lane) - 1u))] = j;
        }
      }
      unsigned int added;
      if (!grid_barrier(g, cnt, &added)) return;
      if (lead) g->cnt[(lev + 2) % 3] = 0u;  // used again two barriers later
      if (added == 0) break;
      lo = hi;
      hi += added;
      ++lev;
    }
    // flip the cluster and sum the spins across its boundary
    int cut = 0;
    for (int e = gtid; e < hi * z; e += gsz) {
      const int fi = e / z, k = e - fi * z;
      const int site = __ldcg(q + fi);
      const int j = __ldg(nbr + (size_t)site * z + k);
      if (j >= 0 && __ldcg(mark + j) != stamp) cut += __ldcg(spins + j);
      if (k == 0) spins[site] = (int8_t)(-ref);
    }
    if (sums) {
      cut = __reduce_add_sync(0xffffffffu, cut);
      if (lane == 0 && cut) atomicAdd(&g->cut, (unsigned long long)(long long)cut);
    }
    if (!grid_barrier(g, nullptr, nullptr)) return;
    if (sums && lead) {
      const long long c = (long long)atomicExch(&g->cut, 0ull);  // read and clear for the next step
      bond -= 2ll * ref * c;
      ups += ref > 0 ? -(long long)hi : (long long)hi;
      double* out = sums + (size_t)t * kNumSums;
      out[0] = (double)bond;
      out[1] = out[2] = out[3] = out[4] = out[5] = 0.0;
      out[6] = (double)ups;
      out[7] = (double)hi;
    }
  }
}

// ------------------------------------------------------------ mid-size
// Lattices beyond 16,384 sites whose spins and cluster marks fit one block's
// shared memory as bits (a quarter byte per site): the same steps in one
// block, the queue in global memory (written and read by this block only),
// a block barrier per level.  One SM's bond draws against a grid barrier per
// level: near T_c the levels, not the draws, set the time of a step.
__global__ void __launch_bounds__(1024) ising_wolff_mid_kernel(int8_t* __restrict__ spins, int n, int z,
                                                               const int32_t* __restrict__ nbr,
                                                               const uint8_t* __restrict__ occ,
                                                               unsigned long long thr, RngKey key, uint32_t n_steps,
                                                               double* __restrict__ sums, int32_t* __restrict__ q) {
  extern __shared__ uint32_t s_bits[];
  const int nw = (n + 31) >> 5;
  uint32_t* up = s_bits;        // bit i: site i is up
  uint32_t* in = s_bits + nw;   // bit i: site i is in this step's cluster
  __shared__ int s_cnt[3];
  __shared__ int s_red[2][32];
  __shared__ int s_cut;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int w = threadIdx.x; w < nw; w += blockDim.x) {
    uint32_t b = 0;
    for (int i = 0; i < 32 && 32 * w + i < n; ++i) b |= (uint32_t)(spins[32 * w + i] > 0) << i;
    up[w] = b;
    in[w] = 0u;
  }
  if (threadIdx.x < 3) s_cnt[threadIdx.x] = 0;
  if (threadIdx.x == 0) s_cut = 0;
  __syncthreads();
  auto spin_of = [&](int i) { return (int)((up[i >> 5] >> (i & 31)) & 1u) * 2 - 1; };
  long long bond = 0, ups = 0;
  if (sums) {  // the bond sum and up count of the incoming state, once per call
    int b = 0, u = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const int si = spin_of(i);
      u += si > 0;
      for (int k = 0; k < z; ++k) {
        const int j = __ldg(nbr + (size_t)i * z + k);
        if (j > i) b += si * spin_of(j);
      }
    }
    b = __reduce_add_sync(0xffffffffu, b);
    u = __reduce_add_sync(0xffffffffu, u);
    if (lane == 0) {
      s_red[0][warp] = b;
      s_red[1][warp] = u;
    }
    __syncthreads();
    if (threadIdx.x == 0)
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
        bond += s_red[0][w];
        ups += s_red[1][w];
      }
  }
  for (uint32_t t = 0; t < n_steps; ++t) {
    const uint32_t step = key.sweep + t;
    const uint4 w0 = philox_ks(make_uint4(step, 0u, kTagWolffSource << 24, key.replica), key.ks);
    const int src = (int)(((unsigned long long)w0.x * (unsigned long long)n) >> 32);
    const int ref = spin_of(src);
    if (threadIdx.x == 0) {
      q[0] = src;
      atomicOr(&in[src >> 5], 1u << (src & 31));
    }
    int lo = 0, hi = 1, lev = 0;
    for (;;) {
      const int items = (hi - lo) * z;
      int* cnt = &s_cnt[lev % 3];
      for (int e = threadIdx.x; e < items; e += blockDim.x) {
        const int fi = e / z, k = e - fi * z;
        const int site = lo == 0 ? src : q[lo + fi];
        const int j = __ldg(nbr + (size_t)site * z + k);
        if (j < 0 || spin_of(j) != ref || ((in[j >> 5] >> (j & 31)) & 1u)) continue;
        const uint32_t a = (uint32_t)min(site, j), b = (uint32_t)max(site, j);
        const uint32_t o = __ldg(occ + (size_t)site * z + k);
        const uint4 w = philox_ks(make_uint4(a, b, (kTagWolffBond << 24) | (o << 20) | (key.replica & 0xFFFFFu), step),
                                  key.ks);
        if ((unsigned long long)w.x >= thr) continue;
        const uint32_t bit = 1u << (j & 31);
        if (!(atomicOr(&in[j >> 5], bit) & bit)) q[hi + atomicAdd(cnt, 1)] = j;
      }
      __syncthreads();
      const int added = *cnt;
      if (threadIdx.x == 0) s_cnt[(lev + 2) % 3] = 0;
      if (added == 0) break;
      lo = hi;
      hi += added;
      ++lev;
    }
    // flip the cluster and sum the spins across its boundary
    int cut = 0;
    for (int e = threadIdx.x; e < hi * z; e += blockDim.x) {
      const int fi = e / z, k = e - fi * z;
      const int site = q[fi];
      const int j = __ldg(nbr + (size_t)site * z + k);
      if (j >= 0 && !((in[j >> 5] >> (j & 31)) & 1u)) cut += spin_of(j);
      if (k == 0) atomicXor(&up[site >> 5], 1u << (site & 31));
    }
    if (sums) {
      cut = __reduce_add_sync(0xffffffffu, cut);
      if (lane == 0 && cut) atomicAdd(&s_cut, cut);
    }
    __syncthreads();
    // clear the cluster marks for the next step
    for (int i = threadIdx.x; i < hi; i += blockDim.x) {
      const int site = q[i];
      atomicAnd(&in[site >> 5], ~(1u << (site & 31)));
    }
    if (sums && threadIdx.x == 0) {
      bond -= 2ll * ref * s_cut;
      ups += ref > 0 ? -(long long)hi : (long long)hi;
      s_cut = 0;
      double* out = sums + (size_t)t * kNumSums;
      out[0] = (double)bond;
      out[1] = out[2] = out[3] = out[4] = out[5] = 0.0;
      out[6] = (double)ups;
      out[7] = (double)hi;
    }
    __syncthreads();
  }
  for (int i = threadIdx.x; i < n; i += blockDim.x) spins[i] = (int8_t)spin_of(i);
}

// Self-test of the barrier's bounded wait: block `skip` (none for skip < 0)
// never arrives, so the other blocks' waits run out after 2 s and set
// g->abort_flag; with every block arriving the barrier completes.  The wait
// ends either way: nothing here spins without a limit.
__global__ void wolff_barrier_probe_kernel(WolffGrid* g, int skip) {
  if ((int)blockIdx.x == skip) return;
  grid_barrier(g, nullptr, nullptr);
}

}  // namespace

cudaError_t launch_wolff_barrier_probe(WolffGrid* g, int blocks, int skip, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(g, 0, sizeof(WolffGrid), s);
  if (e != cudaSuccess) return e;
  void* args[] = {&g, &skip};
  return cudaLaunchCooperativeKernel((const void*)wolff_barrier_probe_kernel, dim3((unsigned)blocks), dim3(32), args,
                                     0, s);
}

size_t ising_wolff_smem(int n) { return (size_t)n * 9; }

cudaError_t launch_ising_wolff_grid(int8_t* spins, int n, int z, const int32_t* nbr, const uint8_t* occ,
                                    unsigned long long thr, RngKey key, uint32_t n_steps, double* sums,
                                    uint32_t* mark, int32_t* q, WolffGrid* g, int sm_count, cudaStream_t s) {
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ising_wolff_grid_kernel, kWolffGridTpb, 0);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorCooperativeLaunchTooLarge;
  // one block per SM: every block must be resident (cooperative launch), and
  // a barrier costs one atomic per block
  dim3 grid((unsigned)sm_count), block(kWolffGridTpb);
  if ((e = cudaMemsetAsync(g, 0, sizeof(WolffGrid), s)) != cudaSuccess) return e;
  void* args[] = {&spins, &n, &z, &nbr, &occ, &thr, &key, &n_steps, &sums, &mark, &q, &g};
  return cudaLaunchCooperativeKernel((const void*)ising_wolff_grid_kernel, grid, block, args, 0, s);
}

size_t ising_wolff_mid_smem(int n) { return (size_t)((n + 31) / 32) * 8; }

cudaError_t launch_ising_wolff_mid(int8_t* spins, int n, int z, const int32_t* nbr, const uint8_t* occ,
                                   unsigned long long thr, RngKey key, uint32_t n_steps, double* sums, int32_t* q,
                                   cudaStream_t s) {
  const size_t smem = ising_wolff_mid_smem(n);
  cudaError_t e =
      cudaFuncSetAttribute(ising_wolff_mid_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  ising_wolff_mid_kernel<<<1, 1024, smem, s>>>(spins, n, z, nbr, occ, thr, key, n_steps, sums, q);
  return cudaGetLastError();
}

cudaError_t launch_ising_wolff(int8_t* spins, int n, int z, const int32_t* nbr, const uint8_t* occ,
                               unsigned long long thr, RngKey key, uint32_t n_steps, double* sums, cudaStream_t s) {
  const size_t smem = ising_wolff_smem(n);
  cudaError_t e = cudaFuncSetAttribute(ising_wolff_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  // about one thread per four sites, a power of two in [128, 1024]: small
  // lattices spend their levels in barriers, not in bond draws (ncu on sc
  // 10^3 near T_c: 12 barrier stalls per issue at 512 threads; cluster
  // steps/s at 1024 / 512 / 256 / 128 / 64 threads: 83,000 / 98,000 /
  // 102,000 / 93,000 / 49,000; sc 6^3 best at 128-256, sc 16^3 at 1024)
  int tpb = 128;
  while (tpb < 1024 && tpb < (n + 3) / 4) tpb *= 2;
  ising_wolff_kernel<<<1, tpb, smem, s>>>(spins, n, z, nbr, occ, thr, key, n_steps, sums);
  return cudaGetLastError();
}

}  // namespace vg
