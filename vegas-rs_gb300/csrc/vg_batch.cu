// vg_batch.cu -- batched, multi-spin-coded Ising Metropolis with on-device
// replica exchange (the vg_batch_* ABI).
//
// Many independent replicas of MetropolisFlipIntegrator (src/integrator.rs:
// 99-138) with J > 0 or < 0 and no field run at once.  A replica group is a
// set of n replicas (a multiple of 32) of one sc lattice; every lattice site
// holds one 32-bit word per 32 replicas (bit l = replica lane l, 1 = Up), in
// the checkerboard class layout [z][y][x/2] of the single-lattice path.
//
// One colour pass updates a word (32 replicas) at once:
//   * anti-aligned neighbour count per lane, bit-sliced with full adders
//     (three-input XOR / majority), 3 bit planes;
//   * dE = 2 J (z - 2 n_anti); moves with dE <= 0 always accept;
//   * the rest compare their 32-bit uniform U with their threshold
//     thr(T_lane, n_anti) most significant bit first: plane k is a Philox
//     word (Philox4x32-7, kMscRounds) whose bit l is bit 31-k of lane l's U; the thresholds are stored
//     transposed (bit l of tab[q][k] = bit 31-k of lane l's threshold for the
//     q-th drawing category).  A lane is decided at its first plane where the
//     bits differ, so a word usually needs 6-11 planes (2-3 Philox blocks)
//     for its 32 flips, and the outcome is exactly "U < thr".
// The last colour-1 pass of every `sweeps_per_round` sweeps also counts
// anti-aligned bonds and up spins per replica of the new state (bit-sliced
// counters over the words a thread settles, turned into per-replica counts by
// warp transposes once at the end), and an exchange kernel swaps the temperatures of adjacent ladder entries with
// probability min(1, exp((b_i - b_j)(E_i - E_j))), then re-transposes the
// threshold tables.  A round (passes, measurement, exchange, counter advance)
// is captured once into a CUDA graph and replayed.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <utility>
#include <vector>

#include "vg_internal.cuh"

using namespace vg;

namespace {

constexpr uint32_t kTagMsc = 6, kTagMscInit = 7, kTagExchange = 8;
// The threshold planes come from Philox4x32-7: Salmon et al. ("Parallel
// random numbers: as easy as 1, 2, 3", SC'11) report Philox4x32 passing
// TestU01's Crush batteries from 7 rounds on and take 10 as the default for a
// safety margin of 3 rounds.  The planes (two blocks per 32-replica word)
// were about a third of the batched pass's time, so they use the 7-round
// function; initial states and exchange decisions keep 10 rounds.
constexpr int kMscRounds = 7;
constexpr int kTabWords = 4 * 33;  // 4 drawing categories x (32 planes + always-lanes word)

struct MscSeg {          // one replica word of one group
  uint32_t* cls[2];
  uint32_t n_c;          // words per class
  int Hx, Ly, Lz;
  int dim3;              // 1: z bonds (3D, periodic); 0: 2D (nz = 1, open z)
  FastDiv fHx, fLy, fLx;
  uint32_t word_id;      // Philox counter word 3
  int group;
  int nd;                // drawing categories (dE > 0)
  int dn[4];             // their anti-aligned counts
  int rep0;              // global index of lane 0
  int plane, zwrap;      // words per z plane, (Lz - 1) planes
};

struct MscGroupDev {
  int n_rep, rep_off, seg0, z;
  double J, nbonds;
  const double* beta;                 // 1/T per ladder entry
  const unsigned long long* thr;      // [ladder][z + 1]
  int* tau;                           // ladder entry of each replica
  int* rep_at;                        // replica at each ladder entry
  unsigned long long* accepted;       // swaps accepted per pair (i, i+1)
  unsigned long long* attempted;
};

struct MscDev {
  uint32_t sweep0;
  uint32_t round;
  uint32_t round_base;   // first round of the current run (ring slot 0)
  uint32_t pad;
};


// (b2 b1 b0) = number of set lanes among the inputs, per lane
__device__ __forceinline__ void count6(uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t a4, uint32_t a5,
                                       uint32_t& b0, uint32_t& b1, uint32_t& b2) {
  const uint32_t sa = a0 ^ a1 ^ a2, ca = (a0 & a1) | (a0 & a2) | (a1 & a2);
  const uint32_t sb = a3 ^ a4 ^ a5, cb = (a3 & a4) | (a3 & a5) | (a4 & a5);
  b0 = sa ^ sb;
  const uint32_t cab = sa & sb;
  b1 = ca ^ cb ^ cab;
  b2 = (ca & cb) | (ca & cab) | (cb & cab);
}
__device__ __forceinline__ void count4(uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t& b0,
                                       uint32_t& b1, uint32_t& b2) {
  const uint32_t sa = a0 ^ a1 ^ a2, ca = (a0 & a1) | (a0 & a2) | (a1 & a2);
  b0 = sa ^ a3;
  const uint32_t cx = sa & a3;
  b1 = ca ^ cx;
  b2 = ca & cx;
}
__device__ __forceinline__ uint32_t lanes_equal(uint32_t b0, uint32_t b1, uint32_t b2, int v) {
  return ((v & 1) ? b0 : ~b0) & ((v & 2) ? b1 : ~b1) & ((v & 4) ? b2 : ~b2);
}

// Neighbour words of class entry j in the other class, xor'ed with s.
__device__ __forceinline__ void msc_anti(const MscSeg& sg, int C, uint32_t j, uint32_t s, const uint32_t* oth,
                                         uint32_t (&a)[6]) {
  const int row = (int)fdiv(j, sg.fHx);
  const int h = (int)(j - (uint32_t)row * sg.Hx);
  const int z = (int)fdiv((uint32_t)row, sg.fLy);
  const int y = row - z * sg.Ly;
  const int p = (y + z + C) & 1;
  // 32-bit word offsets (a class holds fewer than 2^31 words): no wide
  // multiplies beside Philox's
  const int rb = row * sg.Hx;
  const int plane = sg.plane;
  const int hx = p ? (h + 1 == sg.Hx ? 0 : h + 1) : (h == 0 ? sg.Hx - 1 : h - 1);
  const int oym = y == 0 ? rb + plane - sg.Hx : rb - sg.Hx;
  const int oyp = y == sg.Ly - 1 ? rb - plane + sg.Hx : rb + sg.Hx;
  a[0] = s ^ __ldg(oth + (uint32_t)(rb + h));
  a[1] = s ^ __ldg(oth + (uint32_t)(rb + hx));
  a[2] = s ^ __ldg(oth + (uint32_t)(oym + h));
  a[3] = s ^ __ldg(oth + (uint32_t)(oyp + h));
  if (sg.dim3) {
    const int ozm = z == 0 ? rb + sg.zwrap : rb - plane;
    const int ozp = z == sg.Lz - 1 ? rb - sg.zwrap : rb + plane;
    a[4] = s ^ __ldg(oth + (uint32_t)(ozm + h));
    a[5] = s ^ __ldg(oth + (uint32_t)(ozp + h));
  } else {
    a[4] = a[5] = 0u;
  }
}

// Bit-plane decision state of one word (32 replicas at one site).
template <int ND>
struct WordState {
  uint32_t m[ND];   // lanes in each drawing category
  uint32_t und;     // lanes still undecided
  uint32_t acc;     // lanes accepted so far
  uint32_t b0, b1, b2, s0;  // for a measuring pass: anti-aligned count before the update, class-0 word at j
};

// Per-replica sums of a measuring pass, bit-sliced (bit l of c[k] is bit k of
// lane l's count).  A lane settles at most its own WPT <= 8 words and one
// queued word per drain (at most WPT + 1 drains): <= 17 words, so bonds
// <= 102 < 2^7 and up spins <= 34 < 2^6.
struct MscTally {
  uint32_t bond[7];
  uint32_t up[6];
};

// c += (x2 x1 x0), lane-wise
template <int NP>
__device__ __forceinline__ void slice_add(uint32_t (&c)[NP], uint32_t x0, uint32_t x1, uint32_t x2) {
  uint32_t k = c[0] & x0;
  c[0] ^= x0;
  uint32_t t = c[1];
  c[1] = t ^ x1 ^ k;
  k = (t & x1) | (t & k) | (x1 & k);
  t = c[2];
  c[2] = t ^ x2 ^ k;
  k = (t & x2) | (t & k) | (x2 & k);
#pragma unroll
  for (int i = 3; i < NP; ++i) {
    t = c[i];
    c[i] = t ^ k;
    k &= t;
  }
}

// A settled word into the tally: the lanes in acc flipped, so their
// anti-aligned count n (of ZZ bonds) became ZZ - n (n and ZZ - n have the
// same parity: b0 stays).
template <int ZZ, int ND>
__device__ __forceinline__ void msc_tally(MscTally& t, const WordState<ND>& w, uint32_t s) {
  uint32_t r1, r2;
  if (ZZ == 6) {
    r1 = ~(w.b1 ^ w.b0);
    r2 = ~(w.b2 | (w.b1 & w.b0));
  } else {
    r1 = w.b1 ^ w.b0;
    r2 = ~(w.b2 | w.b1 | w.b0);
  }
  slice_add(t.bond, w.b0, (w.acc & r1) | (~w.acc & w.b1), (w.acc & r2) | (~w.acc & w.b2));
  const uint32_t s1 = s ^ w.acc;
  slice_add(t.up, w.s0 ^ s1, w.s0 & s1, 0u);
}

// Threshold plane k of every drawing category for the lanes in its mask
// (s_tab: the block's table plane-major, one uint4 of categories per plane).
template <int ND>
__device__ __forceinline__ uint32_t msc_plane(const WordState<ND>& w, const uint4* s_tab, int k) {
  const uint4 t = s_tab[k];  // one shared-memory load for all categories
  uint32_t T = w.m[0] & t.x;
  if (ND > 1) T |= w.m[1] & t.y;
  if (ND > 2) T |= w.m[2] & t.z;
  if (ND > 3) T |= w.m[3] & t.w;
  return T;
}

// Planes 4*blkno .. 4*blkno+3 of word j.
template <int C, int ND>
__device__ __forceinline__ void msc_block(WordState<ND>& w, uint32_t j, uint32_t sweep, uint32_t word_id,
                                          int blkno, const uint4* s_tab, const KeySchedule& ks) {
  const uint4 bk =
      philox_ks<kMscRounds>(make_uint4(j, sweep, (kTagMsc << 24) | ((uint32_t)C << 8) | (uint32_t)blkno, word_id), ks);
  const uint32_t R[4] = {bk.x, bk.y, bk.z, bk.w};
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const uint32_t T = msc_plane<ND>(w, s_tab, 4 * blkno + i);
    w.acc |= w.und & ~R[i] & T;
    w.und &= ~(R[i] ^ T);
  }
}

// Categories of word j and its first 8 planes.  ZZ is the coordination (4 or
// 6); the drawing categories are the anti-aligned counts with dE > 0:
// n < ZZ/2 for J > 0, n > ZZ/2 for J < 0 (none for J = 0).
template <int C, int ZZ>
__device__ __forceinline__ WordState<ZZ / 2> msc_word_start(const MscSeg& sg, uint32_t j, uint32_t s,
                                                            const uint32_t* oth, const uint4* s_tab,
                                                            uint32_t sweep, const KeySchedule& ks, int jsign) {
  constexpr int ND = ZZ / 2;
  WordState<ND> w;
  uint32_t a[6];
  msc_anti(sg, C, j, s, oth, a);
  uint32_t b0, b1, b2;
  if (ZZ == 6) count6(a[0], a[1], a[2], a[3], a[4], a[5], b0, b1, b2);
  else count4(a[0], a[1], a[2], a[3], b0, b1, b2);
  w.b0 = b0;
  w.b1 = b1;
  w.b2 = b2;
  w.s0 = a[0] ^ s;  // the other class's word at the same index
  uint32_t draw = 0;
#pragma unroll
  for (int q = 0; q < ND; ++q) {
    const int n = jsign > 0 ? q : ZZ / 2 + 1 + q;
    w.m[q] = jsign == 0 ? 0u : lanes_equal(b0, b1, b2, n);
    draw |= w.m[q];
  }
  const uint32_t alw = msc_plane<ND>(w, s_tab, 32);
  w.acc = ~draw | alw;
  w.und = draw & ~alw;
  msc_block<C, ND>(w, j, sweep, sg.word_id, 0, s_tab, ks);
  msc_block<C, ND>(w, j, sweep, sg.word_id, 1, s_tab, ks);
  return w;
}

// Transpose of the 32 x 32 bit matrix whose row t is lane t's word: lane l
// gets the word whose bit t is bit l of lane t's x (five exchange stages,
// each swapping the off-diagonal blocks of every 2j x 2j block).
__device__ __forceinline__ uint32_t warp_columns(uint32_t x) {
  const int lane = threadIdx.x & 31;
  const uint32_t m[5] = {0x0000FFFFu, 0x00FF00FFu, 0x0F0F0F0Fu, 0x33333333u, 0x55555555u};
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    const int j = 16 >> k;
    const uint32_t y = __shfl_xor_sync(0xffffffffu, x, j);
    x = (lane & j) ? ((x & ~m[k]) | ((y & ~m[k]) >> j)) : ((x & m[k]) | ((y & m[k]) << j));
  }
  return x;
}

// Launch shape of a pass (chosen by the autotuner, vg_batch_autotune): a
// block of TPB threads covers TPB x WPT consecutive words of one segment;
// each thread takes its WPT words WIF at a time (WIF = 2 interleaves two
// independent words' Philox chains and loads; four at a time, 72 registers,
// ran the c4 batch at 2,556 flips/ns against 2,586 with two).  Every shape
// makes the same decisions for every word.
//
// Words still undecided after 8 planes are queued per warp and finished 32
// at a time, so the rare long comparisons run with full warps.  MEAS: the
// measuring pass (C = 1), which tallies every settled word and returns lane
// l's counts for replica l in ca (anti-aligned bonds) and cu (up spins).
constexpr int kQueue = 64;  // per-warp queue entries
template <bool MEAS>
__host__ __device__ constexpr int queue_words() {
  return 4 + 3 + (MEAS ? 4 : 0);  // j, s, und, acc, m[<= 3] (+ b0, b1, b2, s0)
}

template <int C, int ZZ, int TPB, int WPT, int WIF, bool MEAS>
__device__ __forceinline__ void msc_pass_body(const MscSeg& sg, uint32_t j0, uint32_t* own, const uint32_t* oth,
                                              const uint4* s_tab, uint32_t sweep, const KeySchedule& ks,
                                              int jsign, uint32_t (*s_q)[kQueue][queue_words<MEAS>()],
                                              unsigned& ca, unsigned& cu) {
  constexpr int ND = ZZ / 2, QW = queue_words<MEAS>();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int qn = 0;
  MscTally tal;
  if (MEAS) {
#pragma unroll
    for (int i = 0; i < 7; ++i) tal.bond[i] = 0u;
#pragma unroll
    for (int i = 0; i < 6; ++i) tal.up[i] = 0u;
  }
  auto finish = [&](int n) {  // complete the first n queued words, one per lane
    __syncwarp();
    if (lane < n) {
      const uint32_t* e = s_q[warp][lane];
      WordState<ND> w;
      const uint32_t j = e[0], s = e[1];
      w.und = e[2];
      w.acc = e[3];
#pragma unroll
      for (int q = 0; q < ND; ++q) w.m[q] = e[4 + q];
      if (MEAS) {
        w.b0 = e[7];
        w.b1 = e[8];
        w.b2 = e[9];
        w.s0 = e[10];
      }
#pragma unroll 1
      for (int blkno = 2; w.und != 0u && blkno < 8; ++blkno) msc_block<C, ND>(w, j, sweep, sg.word_id, blkno, s_tab, ks);
      if (w.acc) own[j] = s ^ w.acc;
      if (MEAS) msc_tally<ZZ>(tal, w, s);
    }
    __syncwarp();
    const int rest = qn - n;
    uint32_t tmp[QW];
    if (lane < rest)
#pragma unroll
      for (int i = 0; i < QW; ++i) tmp[i] = s_q[warp][n + lane][i];
    __syncwarp();
    if (lane < rest)
#pragma unroll
      for (int i = 0; i < QW; ++i) s_q[warp][lane][i] = tmp[i];
    __syncwarp();
    qn = rest;
  };
#pragma unroll 1
  for (int u = 0; u < WPT; u += WIF) {
    uint32_t j[WIF], s[WIF];
    bool live[WIF], pend[WIF];
    WordState<ND> w[WIF];
#pragma unroll
    for (int i = 0; i < WIF; ++i) {
      j[i] = j0 + (uint32_t)((u + i) * TPB) + threadIdx.x;
      live[i] = j[i] < sg.n_c;
      const uint32_t jj = live[i] ? j[i] : 0u;  // dead lanes work on a valid word and discard it
      s[i] = own[jj];
      w[i] = msc_word_start<C, ZZ>(sg, jj, s[i], oth, s_tab, sweep, ks, jsign);
      pend[i] = live[i] && w[i].und != 0u;
      if (live[i] && !pend[i] && w[i].acc) own[j[i]] = s[i] ^ w[i].acc;
      if (MEAS && live[i] && !pend[i]) msc_tally<ZZ>(tal, w[i], s[i]);
    }
#pragma unroll
    for (int i = 0; i < WIF; ++i) {
      const unsigned pmask = __ballot_sync(0xffffffffu, pend[i]);
      if (pmask) {
        if (pend[i]) {
          uint32_t* e = s_q[warp][qn + __popc(pmask & ((1u << lane) - 1u))];
          e[0] = j[i];
          e[1] = s[i];
          e[2] = w[i].und;
          e[3] = w[i].acc;
#pragma unroll
          for (int q = 0; q < ND; ++q) e[4 + q] = w[i].m[q];
          if (MEAS) {
            e[7] = w[i].b0;
            e[8] = w[i].b1;
            e[9] = w[i].b2;
            e[10] = w[i].s0;
          }
        }
        qn += __popc(pmask);
        if (qn >= 32) finish(32);
      }
    }
  }
  if (qn > 0) finish(qn);
  if (MEAS) {  // lane l: replica l's sums over the warp's words
#pragma unroll
    for (int k = 0; k < 7; ++k) ca += (unsigned)__popc(warp_columns(tal.bond[k])) << k;
#pragma unroll
    for (int k = 0; k < 6; ++k) cu += (unsigned)__popc(warp_columns(tal.up[k])) << k;
  }
}

// MEAS (the last colour-1 pass of a round): also add the new state's
// anti-aligned bonds (over class-1 sites, whose neighbours are all class 0)
// and up spins per replica into obs[slot][replica][2].
template <int C, int TPB, int WPT, int WIF, bool MEAS>
__global__ void __launch_bounds__(TPB) msc_pass(const MscSeg* __restrict__ segs, const int2* __restrict__ blocks,
                                                const uint32_t* __restrict__ tabs, const MscDev* __restrict__ dev,
                                                uint32_t t_off, KeySchedule ks, int jsign, int total_rep,
                                                unsigned long long* __restrict__ obs) {
  static_assert(!MEAS || C == 1, "the measuring pass is the colour-1 pass");
  __shared__ uint4 s_tab[33];  // plane k: the 4 categories' threshold words
  __shared__ uint32_t s_q[TPB / 32][kQueue][queue_words<MEAS>()];
  __shared__ unsigned int s_cnt[2][32];
  pdl_launch_dependents();
  const int2 bl = blocks[blockIdx.x];
  const MscSeg sg = segs[bl.x];
  if (MEAS && threadIdx.x < 32) {
    s_cnt[0][threadIdx.x] = 0;
    s_cnt[1][threadIdx.x] = 0;
  }
  // Tables and counters change only in the exchange / advance kernels, which
  // complete before any pass of the next round starts; spins are read after
  // the wait for the previous pass.
  for (int i = threadIdx.x; i < kTabWords; i += blockDim.x)  // category-major in memory, plane-major here
    reinterpret_cast<uint32_t*>(s_tab)[(i % 33) * 4 + i / 33] = tabs[(size_t)bl.x * kTabWords + i];
  const uint32_t sweep = dev->sweep0 + t_off;
  __syncthreads();
  pdl_wait();
  uint32_t* own = sg.cls[C];
  const uint32_t* oth = sg.cls[C ^ 1];
  unsigned ca = 0, cu = 0;
  if (sg.dim3)
    msc_pass_body<C, 6, TPB, WPT, WIF, MEAS>(sg, (uint32_t)bl.y, own, oth, s_tab, sweep, ks, jsign, s_q, ca, cu);
  else
    msc_pass_body<C, 4, TPB, WPT, WIF, MEAS>(sg, (uint32_t)bl.y, own, oth, s_tab, sweep, ks, jsign, s_q, ca, cu);
  if (MEAS) {
    const int lane = threadIdx.x & 31;
    atomicAdd(&s_cnt[0][lane], ca);
    atomicAdd(&s_cnt[1][lane], cu);
    __syncthreads();
    if (threadIdx.x < 32) {
      const uint32_t slot = dev->round - dev->round_base;
      unsigned long long* o = obs + ((size_t)slot * total_rep + sg.rep0 + threadIdx.x) * 2;
      atomicAdd(o, (unsigned long long)s_cnt[0][threadIdx.x]);
      atomicAdd(o + 1, (unsigned long long)s_cnt[1][threadIdx.x]);
    }
  }
}

// Threshold planes of every replica word of group g from the current
// temperature assignment.
__device__ void msc_build_tabs(const MscGroupDev& G, const MscSeg* segs, uint32_t* tabs) {
  const int nw = G.n_rep / 32;
  const MscSeg& s0 = segs[G.seg0];
  for (int e = threadIdx.x; e < nw * kTabWords; e += blockDim.x) {
    const int w = e / kTabWords, r = e % kTabWords, q = r / 33, k = r % 33;
    uint32_t v = 0;
    if (q < s0.nd) {
      for (int l = 0; l < 32; ++l) {
        const unsigned long long th = G.thr[(size_t)G.tau[w * 32 + l] * (G.z + 1) + s0.dn[q]];
        uint32_t bit;
        if (k == 32) bit = th >= (1ull << 32) ? 1u : 0u;
        else bit = th >= (1ull << 32) ? 0u : (uint32_t)((th >> (31 - k)) & 1ull);
        v |= bit << l;
      }
    }
    tabs[(size_t)(G.seg0 + w) * kTabWords + r] = v;
  }
}

__global__ void msc_tabs_kernel(const MscGroupDev* __restrict__ groups, const MscSeg* __restrict__ segs,
                                uint32_t* __restrict__ tabs) {
  msc_build_tabs(groups[blockIdx.x], segs, tabs);
}

// One block per group: energies, ladder swaps, threshold tables.
__global__ void msc_exchange(const MscGroupDev* __restrict__ groups, const MscSeg* __restrict__ segs,
                             uint32_t* __restrict__ tabs, const MscDev* __restrict__ dev, int total_rep,
                             const unsigned long long* __restrict__ obs, int* __restrict__ tau_ring, int do_exchange,
                             KeySchedule ks) {
  extern __shared__ double s_E[];
  const MscGroupDev G = groups[blockIdx.x];
  const uint32_t round = dev->round;
  const uint32_t slot = round - dev->round_base;
  for (int r = threadIdx.x; r < G.n_rep; r += blockDim.x) {
    const unsigned long long anti = obs[((size_t)slot * total_rep + G.rep_off + r) * 2];
    s_E[r] = -G.J * (G.nbonds - 2.0 * (double)anti);
    tau_ring[(size_t)slot * total_rep + G.rep_off + r] = G.tau[r];
  }
  __syncthreads();
  if (do_exchange) {
    for (int i = (int)(round & 1u) + 2 * threadIdx.x; i + 1 < G.n_rep; i += 2 * blockDim.x) {
      const int r1 = G.rep_at[i], r2 = G.rep_at[i + 1];
      const double x = (G.beta[i] - G.beta[i + 1]) * (s_E[r1] - s_E[r2]);
      const uint4 w = philox_ks(make_uint4((uint32_t)i, round, (kTagExchange << 24) | (uint32_t)blockIdx.x, 0u), ks);
      const double u = (double)w.x * (1.0 / 4294967296.0);
      G.attempted[i] += 1;
      if (x >= 0.0 || u < exp(x)) {
        G.rep_at[i] = r2;
        G.rep_at[i + 1] = r1;
        G.tau[r1] = i + 1;
        G.tau[r2] = i;
        G.accepted[i] += 1;
      }
    }
    __syncthreads();
    msc_build_tabs(G, segs, tabs);
  }
}

__global__ void msc_advance(MscDev* dev, uint32_t sweeps) {
  dev->sweep0 += sweeps;
  dev->round += 1;
}

// Initial state: bit l of word 0 of Philox(site, 0, tag, word id) is lane l.
__global__ void msc_init(const MscSeg* __restrict__ segs, int nseg, KeySchedule ks) {
  const MscSeg sg = segs[blockIdx.y];
  const uint32_t Lx = 2u * (uint32_t)sg.Hx;
  const uint32_t n = 2u * sg.n_c;
  const FastDiv fLx = sg.fLx;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint4 w = philox_ks(make_uint4(i, 0u, kTagMscInit << 24, sg.word_id), ks);
    const uint32_t r = fdiv(i, fLx), x = i - r * Lx;
    const uint32_t zz = fdiv(r, sg.fLy), y = r - zz * (uint32_t)sg.Ly;
    const int c = (int)((x + y + zz) & 1u);
    sg.cls[c][r * (uint32_t)sg.Hx + (x >> 1)] = w.x;
  }
  (void)nseg;
}

// Unpack / pack one replica lane in site order.
__global__ void msc_get(const MscSeg sg, uint32_t lane, int8_t* __restrict__ out) {
  const uint32_t Lx = 2u * (uint32_t)sg.Hx, n = 2u * sg.n_c;
  const FastDiv fLx = sg.fLx;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t r = fdiv(i, fLx), x = i - r * Lx;
    const uint32_t zz = fdiv(r, sg.fLy), y = r - zz * (uint32_t)sg.Ly;
    const int c = (int)((x + y + zz) & 1u);
    out[i] = (sg.cls[c][r * (uint32_t)sg.Hx + (x >> 1)] >> lane) & 1u ? 1 : -1;
  }
}

__global__ void msc_set(const MscSeg sg, uint32_t lane, const int8_t* __restrict__ in, int* flag) {
  const uint32_t Lx = 2u * (uint32_t)sg.Hx, n = 2u * sg.n_c;
  const FastDiv fLx = sg.fLx;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int8_t v = in[i];
    if (v != 1 && v != -1) atomicOr(flag, 1);
    const uint32_t r = fdiv(i, fLx), x = i - r * Lx;
    const uint32_t zz = fdiv(r, sg.fLy), y = r - zz * (uint32_t)sg.Ly;
    const int c = (int)((x + y + zz) & 1u);
    uint32_t* p = &sg.cls[c][r * (uint32_t)sg.Hx + (x >> 1)];
    if (v > 0) atomicOr(p, 1u << lane);
    else atomicAnd(p, ~(1u << lane));
  }
}

struct GroupHost {
  vg_lattice_desc lat;
  int n_rep, z, nd, dn[4], seg0, rep_off;
  long long n;
  std::vector<double> temps;
  double* d_beta = nullptr;
  unsigned long long* d_thr = nullptr;
  int* d_tau = nullptr;
  int* d_rep_at = nullptr;
  unsigned long long* d_acc = nullptr;
  unsigned long long* d_att = nullptr;
};

}  // namespace

struct vg_batch {
  int device = 0;
  vg_batch_tuning tune{256, 4, 1};
  cudaStream_t own_stream = nullptr, stream = nullptr;
  double J = 1.0;
  uint64_t seed = 0;
  KeySchedule ks{};
  int every = 10, exchange = 1, total_rep = 0;
  std::vector<GroupHost> groups;
  std::vector<MscSeg> segs;
  MscSeg* d_segs = nullptr;
  std::vector<int2> blocks;
  int2* d_blocks = nullptr;
  uint32_t* d_tabs = nullptr;
  MscGroupDev* d_groups = nullptr;
  MscDev* d_dev = nullptr;
  uint32_t* d_spins = nullptr;
  unsigned long long* d_obs = nullptr;
  int* d_tau_ring = nullptr;
  size_t ring_cap = 0;
  uint64_t last_rounds = 0;
  uint64_t sweep = 0;
  uint32_t round = 0;
  cudaGraphExec_t graph = nullptr;
  int* d_flag = nullptr;
  int8_t* d_stage = nullptr;
  long long stage_n = 0;
  long long replica_sites = 0;
  std::string err;
};

extern "C" void vg_internal_set_last_error(const char* msg);

namespace {

int bfail(vg_batch* b, int code, const std::string& m) {
  if (b) b->err = m;
  vg_internal_set_last_error(m.c_str());
  return code;
}

#define VG_BCUDA(b, expr)                                                                          \
  do {                                                                                             \
    cudaError_t _e = (expr);                                                                       \
    if (_e != cudaSuccess)                                                                         \
      return bfail((b), _e == cudaErrorMemoryAllocation ? VG_ERR_OOM : VG_ERR_CUDA,                \
                   std::string(#expr) + ": " + cudaGetErrorString(_e));                            \
  } while (0)

template <typename T>
int balloc(vg_batch* b, T** p, size_t count) {
  VG_BCUDA(b, cudaMalloc((void**)p, std::max<size_t>(count, 1) * sizeof(T)));
  return VG_OK;
}

void bdestroy(vg_batch* b) {
  if (!b) return;
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->graph) cudaGraphExecDestroy(b->graph);
  for (auto& g : b->groups) {
    cudaFree(g.d_beta);
    cudaFree(g.d_thr);
    cudaFree(g.d_tau);
    cudaFree(g.d_rep_at);
    cudaFree(g.d_acc);
    cudaFree(g.d_att);
  }
  cudaFree(b->d_segs);
  cudaFree(b->d_blocks);
  cudaFree(b->d_tabs);
  cudaFree(b->d_groups);
  cudaFree(b->d_dev);
  cudaFree(b->d_spins);
  cudaFree(b->d_obs);
  cudaFree(b->d_tau_ring);
  cudaFree(b->d_flag);
  cudaFree(b->d_stage);
  if (b->own_stream) cudaStreamDestroy(b->own_stream);
  delete b;
}

using MscPassFn = void (*)(const MscSeg*, const int2*, const uint32_t*, const MscDev*, uint32_t, KeySchedule, int,
                           int, unsigned long long*);

template <int C, int TPB, bool MEAS>
MscPassFn msc_pass_wpt(int wpt, int wif) {
  if (wpt == 2) return wif == 2 ? msc_pass<C, TPB, 2, 2, MEAS> : msc_pass<C, TPB, 2, 1, MEAS>;
  if (wpt == 4) return wif == 2 ? msc_pass<C, TPB, 4, 2, MEAS> : msc_pass<C, TPB, 4, 1, MEAS>;
  return wif == 2 ? msc_pass<C, TPB, 8, 2, MEAS> : msc_pass<C, TPB, 8, 1, MEAS>;
}

template <int C, bool MEAS = false>
MscPassFn msc_pass_fn(const vg_batch_tuning& t) {
  return t.threads_per_block == 128 ? msc_pass_wpt<C, 128, MEAS>(t.words_per_thread, t.words_in_flight)
                                    : msc_pass_wpt<C, 256, MEAS>(t.words_per_thread, t.words_in_flight);
}

bool tuning_supported(const vg_batch_tuning& t) {
  return (t.threads_per_block == 128 || t.threads_per_block == 256) &&
         (t.words_per_thread == 2 || t.words_per_thread == 4 || t.words_per_thread == 8) &&
         (t.words_in_flight == 1 || t.words_in_flight == 2);
}

// Block table for the current launch shape: (segment, first word) per block.
int build_blocks(vg_batch* b) {
  const int per = b->tune.threads_per_block * b->tune.words_per_thread;
  b->blocks.clear();
  for (size_t k = 0; k < b->segs.size(); ++k) {
    const int nbl = (int)((b->segs[k].n_c + per - 1) / per);
    for (int i = 0; i < nbl; ++i) b->blocks.push_back(make_int2((int)k, i * per));
  }
  cudaFree(b->d_blocks);
  b->d_blocks = nullptr;
  int rc = balloc(b, &b->d_blocks, b->blocks.size());
  if (rc) return rc;
  VG_BCUDA(b, cudaMemcpy(b->d_blocks, b->blocks.data(), sizeof(int2) * b->blocks.size(), cudaMemcpyHostToDevice));
  return VG_OK;
}

// One round on the stream: sweeps, measurement, exchange, advance.
int enqueue_round(vg_batch* b) {
  const int nb = (int)b->blocks.size();
  const MscPassFn p0 = msc_pass_fn<0>(b->tune), p1 = msc_pass_fn<1>(b->tune), p1m = msc_pass_fn<1, true>(b->tune);
  const dim3 tpb((unsigned)b->tune.threads_per_block);
  for (int t = 0; t < b->every; ++t) {
    const int jsign = b->J > 0.0 ? 1 : b->J < 0.0 ? -1 : 0;
    VG_BCUDA(b, launch_pdl_ex(p0, dim3(nb), tpb, 0, b->stream, (const MscSeg*)b->d_segs, (const int2*)b->d_blocks,
                           (const uint32_t*)b->d_tabs, (const MscDev*)b->d_dev, (uint32_t)t, b->ks, jsign,
                           b->total_rep, b->d_obs));
    // the round's last sweep measures its final state
    VG_BCUDA(b, launch_pdl_ex(t + 1 == b->every ? p1m : p1, dim3(nb), tpb, 0, b->stream, (const MscSeg*)b->d_segs,
                           (const int2*)b->d_blocks, (const uint32_t*)b->d_tabs, (const MscDev*)b->d_dev,
                           (uint32_t)t, b->ks, jsign, b->total_rep, b->d_obs));
  }
  int maxrep = 0;
  for (auto& g : b->groups) maxrep = std::max(maxrep, g.n_rep);
  msc_exchange<<<(int)b->groups.size(), 256, sizeof(double) * maxrep, b->stream>>>(
      b->d_groups, b->d_segs, b->d_tabs, b->d_dev, b->total_rep, b->d_obs, b->d_tau_ring, b->exchange, b->ks);
  VG_BCUDA(b, cudaGetLastError());
  msc_advance<<<1, 1, 0, b->stream>>>(b->d_dev, (uint32_t)b->every);
  VG_BCUDA(b, cudaGetLastError());
  return VG_OK;
}

// The per-round ring buffers are baked into the captured graph: growing them
// drops the graph, which is captured again with the new pointers.
int ensure_ring(vg_batch* b, uint64_t rounds) {
  if (rounds <= b->ring_cap) return VG_OK;
  rounds = std::max<uint64_t>(rounds, std::max<uint64_t>(64, 2 * b->ring_cap));
  VG_BCUDA(b, cudaStreamSynchronize(b->stream));
  if (b->graph) {
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  cudaFree(b->d_obs);
  cudaFree(b->d_tau_ring);
  b->d_obs = nullptr;
  b->d_tau_ring = nullptr;
  int rc;
  if ((rc = balloc(b, &b->d_obs, (size_t)rounds * b->total_rep * 2))) return rc;
  if ((rc = balloc(b, &b->d_tau_ring, (size_t)rounds * b->total_rep))) return rc;
  b->ring_cap = rounds;
  return VG_OK;
}

int find_replica(vg_batch* b, int g, int r, MscSeg* sg, uint32_t* lane) {
  if (g < 0 || g >= (int)b->groups.size()) return bfail(b, VG_ERR_INVALID_ARG, "group index out of range");
  const GroupHost& G = b->groups[g];
  if (r < 0 || r >= G.n_rep) return bfail(b, VG_ERR_INVALID_ARG, "replica index out of range");
  *sg = b->segs[G.seg0 + r / 32];
  *lane = (uint32_t)(r % 32);
  return VG_OK;
}

int ensure_stage(vg_batch* b, long long n) {
  if (n <= b->stage_n) return VG_OK;
  cudaFree(b->d_stage);
  b->d_stage = nullptr;
  int rc = balloc(b, &b->d_stage, (size_t)n);
  if (rc) return rc;
  b->stage_n = n;
  return VG_OK;
}

}  // namespace

extern "C" {

int vg_batch_create(const vg_replica_group* groups, int32_t n_groups, double J, uint64_t seed,
                    int32_t sweeps_per_round, int32_t replica_exchange, vg_batch** out) {
  if (!out || !groups || n_groups < 1) return bfail(nullptr, VG_ERR_INVALID_ARG, "no replica groups");
  *out = nullptr;
  if (sweeps_per_round < 1) return bfail(nullptr, VG_ERR_INVALID_ARG, "sweeps_per_round must be >= 1");
  if (!std::isfinite(J)) return bfail(nullptr, VG_ERR_INVALID_ARG, "exchange constant must be finite");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    return bfail(nullptr, VG_ERR_NO_DEVICE, "no CUDA device is visible");
  vg_batch* b = new (std::nothrow) vg_batch();
  if (!b) return bfail(nullptr, VG_ERR_OOM, "host allocation failed");
  cudaGetDevice(&b->device);
  b->J = J;
  b->seed = seed;
  b->ks = make_key_schedule((uint32_t)seed, (uint32_t)(seed >> 32));
  b->every = sweeps_per_round;
  b->exchange = replica_exchange != 0;
  if (cudaStreamCreateWithFlags(&b->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
    bdestroy(b);
    return bfail(nullptr, VG_ERR_CUDA, "stream creation failed");
  }
  b->stream = b->own_stream;

  // validate groups, lay out replica words
  size_t words_total = 0;
  int seg = 0, rep = 0;
  for (int g = 0; g < n_groups; ++g) {
    const vg_replica_group& rg = groups[g];
    const vg_lattice_desc& L = rg.lattice;
    const bool is3d = L.pbc_x && L.pbc_y && L.pbc_z;
    const bool is2d = L.pbc_x && L.pbc_y && !L.pbc_z && L.nz == 1;
    if (L.cell != VG_CELL_SC || !(is3d || is2d) || L.nx < 2 || L.ny < 2 || L.nx % 2 || L.ny % 2 ||
        (is3d && (L.nz < 2 || L.nz % 2))) {
      bdestroy(b);
      return bfail(nullptr, VG_ERR_UNSUPPORTED,
                   "batched groups need an sc lattice with even extents >= 2, periodic on every axis or 2D "
                   "(nz = 1, open z)");
    }
    if (rg.n_replicas < 32 || rg.n_replicas % 32 || rg.n_replicas > 1024 || !rg.temperatures) {
      bdestroy(b);
      return bfail(nullptr, VG_ERR_INVALID_ARG, "n_replicas must be a multiple of 32 in [32, 1024] with temperatures");
    }
    const double n = (double)L.nx * L.ny * L.nz;
    if (n > 2147483647.0) {
      bdestroy(b);
      return bfail(nullptr, VG_ERR_UNSUPPORTED, "lattice has more than 2^31-1 sites");
    }
    GroupHost G;
    G.lat = L;
    G.n_rep = rg.n_replicas;
    G.n = (long long)L.nx * L.ny * L.nz;
    G.z = is3d ? 6 : 4;
    G.seg0 = seg;
    G.rep_off = rep;
    G.temps.assign(rg.temperatures, rg.temperatures + rg.n_replicas);
    for (double t : G.temps)
      if (!(t > 0.0) || !std::isfinite(t)) {
        bdestroy(b);
        return bfail(nullptr, VG_ERR_INVALID_ARG, "temperatures must be positive and finite");
      }
    G.nd = 0;
    for (int na = 0; na <= G.z; ++na)
      if (2.0 * J * (double)(G.z - 2 * na) > 0.0 && G.nd < 4) G.dn[G.nd++] = na;
    b->groups.push_back(G);
    seg += G.n_rep / 32;
    rep += G.n_rep;
    words_total += (size_t)(G.n_rep / 32) * (size_t)G.n;
    b->replica_sites += (long long)G.n_rep * G.n;
  }
  b->total_rep = rep;
  int rc = balloc(b, &b->d_spins, words_total);
  size_t off = 0;
  for (auto& G : b->groups) {
    const uint32_t nc = (uint32_t)(G.n / 2);
    for (int w = 0; w < G.n_rep / 32 && !rc; ++w) {
      MscSeg s{};
      s.cls[0] = b->d_spins + off;
      s.cls[1] = b->d_spins + off + nc;
      off += 2 * (size_t)nc;
      s.n_c = nc;
      s.Hx = G.lat.nx / 2;
      s.Ly = G.lat.ny;
      s.Lz = G.lat.nz;
      s.dim3 = G.z == 6;
      s.fHx = make_fastdiv((uint32_t)s.Hx);
      s.fLy = make_fastdiv((uint32_t)s.Ly);
      s.plane = s.Ly * s.Hx;
      s.zwrap = (s.Lz - 1) * s.plane;
      s.fLx = make_fastdiv((uint32_t)G.lat.nx);
      s.word_id = (uint32_t)b->segs.size();
      s.group = (int)(&G - &b->groups[0]);
      s.nd = G.nd;
      for (int q = 0; q < 4; ++q) s.dn[q] = q < G.nd ? G.dn[q] : 0;
      s.rep0 = G.rep_off + 32 * w;
      b->segs.push_back(s);
    }
  }
  if (!rc) rc = balloc(b, &b->d_segs, b->segs.size());
  if (!rc) rc = build_blocks(b);
  if (!rc) rc = balloc(b, &b->d_tabs, b->segs.size() * kTabWords);
  if (!rc) rc = balloc(b, &b->d_groups, b->groups.size());
  if (!rc) rc = balloc(b, &b->d_dev, 1);
  if (!rc) rc = balloc(b, &b->d_flag, 1);
  std::vector<MscGroupDev> gdev;
  for (auto& G : b->groups) {
    if (rc) break;
    if ((rc = balloc(b, &G.d_beta, G.n_rep))) break;
    if ((rc = balloc(b, &G.d_thr, (size_t)G.n_rep * (G.z + 1)))) break;
    if ((rc = balloc(b, &G.d_tau, G.n_rep))) break;
    if ((rc = balloc(b, &G.d_rep_at, G.n_rep))) break;
    if ((rc = balloc(b, &G.d_acc, G.n_rep))) break;
    if ((rc = balloc(b, &G.d_att, G.n_rep))) break;
    std::vector<double> beta(G.n_rep);
    std::vector<unsigned long long> thr((size_t)G.n_rep * (G.z + 1));
    std::vector<int> ident(G.n_rep);
    for (int i = 0; i < G.n_rep; ++i) {
      const double T = std::max(G.temps[i], 2.220446049250313e-16);
      beta[i] = 1.0 / G.temps[i];
      ident[i] = i;
      for (int na = 0; na <= G.z; ++na) {
        // the Ising threshold rule for dE = 2 J (z - 2 n_anti)
        const double de = 2.0 * J * (double)(G.z - 2 * na);
        unsigned long long th;
        if (de <= 0.0) {
          th = 1ull << 32;
        } else {
          const double x = std::ceil(std::exp(-de / T) * 4294967296.0);
          th = x >= 4294967296.0 ? (1ull << 32) : x <= 0.0 ? 0ull : (unsigned long long)x;
        }
        thr[(size_t)i * (G.z + 1) + na] = th;
      }
    }
    cudaMemcpy(G.d_beta, beta.data(), sizeof(double) * G.n_rep, cudaMemcpyHostToDevice);
    cudaMemcpy(G.d_thr, thr.data(), sizeof(unsigned long long) * thr.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(G.d_tau, ident.data(), sizeof(int) * G.n_rep, cudaMemcpyHostToDevice);
    cudaMemcpy(G.d_rep_at, ident.data(), sizeof(int) * G.n_rep, cudaMemcpyHostToDevice);
    cudaMemset(G.d_acc, 0, sizeof(unsigned long long) * G.n_rep);
    cudaMemset(G.d_att, 0, sizeof(unsigned long long) * G.n_rep);
    MscGroupDev d{};
    d.n_rep = G.n_rep;
    d.rep_off = G.rep_off;
    d.seg0 = G.seg0;
    d.z = G.z;
    d.J = J;
    d.nbonds = (double)G.z * (double)G.n / 2.0;
    d.beta = G.d_beta;
    d.thr = G.d_thr;
    d.tau = G.d_tau;
    d.rep_at = G.d_rep_at;
    d.accepted = G.d_acc;
    d.attempted = G.d_att;
    gdev.push_back(d);
  }
  if (rc) {
    const std::string e = b->err;
    bdestroy(b);
    return bfail(nullptr, rc, e);
  }
  cudaMemcpy(b->d_segs, b->segs.data(), sizeof(MscSeg) * b->segs.size(), cudaMemcpyHostToDevice);
  cudaMemcpy(b->d_groups, gdev.data(), sizeof(MscGroupDev) * gdev.size(), cudaMemcpyHostToDevice);
  MscDev d0{0, 0, 0, 0};
  cudaMemcpy(b->d_dev, &d0, sizeof(d0), cudaMemcpyHostToDevice);
  cudaMemset(b->d_spins, 0xFF, sizeof(uint32_t) * words_total);  // all up until initialised
  msc_tabs_kernel<<<(int)b->groups.size(), 256, 0, b->stream>>>(b->d_groups, b->d_segs, b->d_tabs);
  const cudaError_t e = cudaStreamSynchronize(b->stream);
  if (e != cudaSuccess) {
    bdestroy(b);
    return bfail(nullptr, VG_ERR_CUDA, std::string("batch set-up: ") + cudaGetErrorString(e));
  }
  *out = b;
  return VG_OK;
}

int vg_batch_destroy(vg_batch* b) {
  if (!b) return VG_ERR_INVALID_ARG;
  bdestroy(b);
  return VG_OK;
}

const char* vg_batch_last_error(const vg_batch* b) { return b ? b->err.c_str() : ""; }

int vg_batch_get_info(const vg_batch* b, vg_batch_info* o) {
  if (!b || !o) return VG_ERR_INVALID_ARG;
  o->n_groups = (int32_t)b->groups.size();
  o->total_replicas = b->total_rep;
  o->replica_words = (int32_t)b->segs.size();
  o->replica_sites = b->replica_sites;
  o->sweeps_per_round = b->every;
  o->sweep_index = b->sweep;
  o->round_index = b->round;
  o->graph = b->graph != nullptr;
  return VG_OK;
}

int vg_batch_get_stream(const vg_batch* b, void** s) {
  if (!b || !s) return VG_ERR_INVALID_ARG;
  *s = (void*)b->stream;
  return VG_OK;
}

int vg_batch_init_random(vg_batch* b) {
  if (!b) return VG_ERR_INVALID_ARG;
  VG_BCUDA(b, cudaSetDevice(b->device));
  msc_init<<<dim3(64, (unsigned)b->segs.size()), 256, 0, b->stream>>>(b->d_segs, (int)b->segs.size(), b->ks);
  VG_BCUDA(b, cudaGetLastError());
  VG_BCUDA(b, cudaStreamSynchronize(b->stream));
  return VG_OK;
}

int vg_batch_run_async(vg_batch* b, uint64_t rounds) {
  if (!b) return VG_ERR_INVALID_ARG;
  if (rounds > kSweepLimit || !sweep_range_ok(b->sweep, rounds * (uint64_t)b->every))
    return bfail(b, VG_ERR_INVALID_ARG, "the run passes sweep index 2^32 (the 32-bit sweep word of the Philox counter)");
  VG_BCUDA(b, cudaSetDevice(b->device));
  int rc = ensure_ring(b, std::max<uint64_t>(rounds, 1));
  if (rc) return rc;
  VG_BCUDA(b, cudaMemsetAsync(b->d_obs, 0, sizeof(unsigned long long) * rounds * b->total_rep * 2, b->stream));
  MscDev d{(uint32_t)b->sweep, b->round, b->round, 0};
  VG_BCUDA(b, cudaMemcpyAsync(b->d_dev, &d, sizeof(d), cudaMemcpyHostToDevice, b->stream));
  if (!b->graph) {  // capture one round once
    cudaGraph_t g = nullptr;
    bool ok = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
    if (ok) {
      const int erc = enqueue_round(b);
      ok = cudaStreamEndCapture(b->stream, &g) == cudaSuccess && erc == VG_OK;
    }
    if (ok && cudaGraphInstantiate(&b->graph, g, 0) != cudaSuccess) {
      b->graph = nullptr;
      ok = false;
    }
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();  // a failed capture falls back to direct launches
  }
  for (uint64_t r = 0; r < rounds; ++r) {
    if (b->graph) {
      VG_BCUDA(b, cudaGraphLaunch(b->graph, b->stream));
    } else {
      if ((rc = enqueue_round(b))) return rc;
    }
  }
  b->sweep += rounds * (uint64_t)b->every;
  b->round += (uint32_t)rounds;
  b->last_rounds = rounds;
  return VG_OK;
}

int vg_batch_synchronize(vg_batch* b) {
  if (!b) return VG_ERR_INVALID_ARG;
  VG_BCUDA(b, cudaStreamSynchronize(b->stream));
  return VG_OK;
}

int vg_batch_run(vg_batch* b, uint64_t rounds) {
  int rc = vg_batch_run_async(b, rounds);
  if (rc) return rc;
  return vg_batch_synchronize(b);
}

int vg_batch_observables(vg_batch* b, uint64_t round, int64_t* counts, int32_t* tau) {
  if (!b) return VG_ERR_INVALID_ARG;
  if (round >= b->last_rounds) return bfail(b, VG_ERR_INVALID_ARG, "round not in the last run");
  VG_BCUDA(b, cudaStreamSynchronize(b->stream));
  if (counts)
    VG_BCUDA(b, cudaMemcpy(counts, b->d_obs + (size_t)round * b->total_rep * 2, sizeof(int64_t) * b->total_rep * 2,
                           cudaMemcpyDeviceToHost));
  if (tau)
    VG_BCUDA(b, cudaMemcpy(tau, b->d_tau_ring + (size_t)round * b->total_rep, sizeof(int32_t) * b->total_rep,
                           cudaMemcpyDeviceToHost));
  return VG_OK;
}

int vg_batch_ladder(vg_batch* b, int32_t group, int32_t* tau) {
  if (!b || !tau || group < 0 || group >= (int)b->groups.size()) return VG_ERR_INVALID_ARG;
  VG_BCUDA(b, cudaStreamSynchronize(b->stream));
  const GroupHost& G = b->groups[group];
  VG_BCUDA(b, cudaMemcpy(tau, G.d_tau, sizeof(int) * G.n_rep, cudaMemcpyDeviceToHost));
  return VG_OK;
}

int vg_batch_swap_stats(vg_batch* b, int32_t group, int64_t* accepted, int64_t* attempted) {
  if (!b || group < 0 || group >= (int)b->groups.size()) return VG_ERR_INVALID_ARG;
  VG_BCUDA(b, cudaStreamSynchronize(b->stream));
  const GroupHost& G = b->groups[group];
  if (accepted) VG_BCUDA(b, cudaMemcpy(accepted, G.d_acc, sizeof(int64_t) * G.n_rep, cudaMemcpyDeviceToHost));
  if (attempted) VG_BCUDA(b, cudaMemcpy(attempted, G.d_att, sizeof(int64_t) * G.n_rep, cudaMemcpyDeviceToHost));
  return VG_OK;
}

int vg_batch_get_tuning(const vg_batch* b, vg_batch_tuning* t) {
  if (!b || !t) return VG_ERR_INVALID_ARG;
  *t = b->tune;
  return VG_OK;
}

int vg_batch_set_tuning(vg_batch* b, const vg_batch_tuning* t) {
  if (!b || !t) return VG_ERR_INVALID_ARG;
  if (!tuning_supported(*t))
    return bfail(b, VG_ERR_UNSUPPORTED, "tuning: threads_per_block 128 or 256, words_per_thread 2, 4 or 8, "
                                        "words_in_flight 1 or 2");
  VG_BCUDA(b, cudaSetDevice(b->device));
  VG_BCUDA(b, cudaStreamSynchronize(b->stream));
  if (b->graph) {  // the captured round holds the old launch shape
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  b->tune = *t;
  return build_blocks(b);
}

int vg_batch_autotune(vg_batch* b, uint32_t rounds, vg_batch_tuning* best, double* best_ms) {
  if (!b || rounds == 0) return VG_ERR_INVALID_ARG;
  VG_BCUDA(b, cudaSetDevice(b->device));
  VG_BCUDA(b, cudaStreamSynchronize(b->stream));
  int rc;
  // The candidates run real rounds; everything they change is saved first
  // and restored afterwards, so the batch continues as if never tuned.
  size_t words = 0;
  for (const auto& sg : b->segs) words += 2 * (size_t)sg.n_c;
  const size_t tabs = b->segs.size() * kTabWords;
  const size_t ring_obs = (size_t)b->last_rounds * b->total_rep * 2, ring_tau = (size_t)b->last_rounds * b->total_rep;
  uint32_t* sv_spins = nullptr;
  uint32_t* sv_tabs = nullptr;
  unsigned long long* sv_obs = nullptr;
  int* sv_ring = nullptr;
  std::vector<int*> sv_int;
  std::vector<unsigned long long*> sv_cnt;
  auto release = [&]() {
    cudaFree(sv_spins);
    cudaFree(sv_tabs);
    cudaFree(sv_obs);
    cudaFree(sv_ring);
    for (auto* p : sv_int) cudaFree(p);
    for (auto* p : sv_cnt) cudaFree(p);
  };
  bool ok = cudaMalloc((void**)&sv_spins, words * 4) == cudaSuccess &&
            cudaMalloc((void**)&sv_tabs, tabs * 4) == cudaSuccess &&
            cudaMalloc((void**)&sv_obs, std::max<size_t>(ring_obs, 1) * 8) == cudaSuccess &&
            cudaMalloc((void**)&sv_ring, std::max<size_t>(ring_tau, 1) * 4) == cudaSuccess;
  for (auto& G : b->groups) {
    int* a = nullptr;
    unsigned long long* c = nullptr;
    ok = ok && cudaMalloc((void**)&a, sizeof(int) * 2 * G.n_rep) == cudaSuccess;
    sv_int.push_back(a);
    ok = ok && cudaMalloc((void**)&c, sizeof(unsigned long long) * 2 * G.n_rep) == cudaSuccess;
    sv_cnt.push_back(c);
  }
  if (!ok) {
    release();
    cudaGetLastError();
    return bfail(b, VG_ERR_OOM, "autotune: no device memory for the saved state");
  }
  auto copy_state = [&](bool save) -> cudaError_t {
    const cudaMemcpyKind k = cudaMemcpyDeviceToDevice;
    cudaError_t e = save ? cudaMemcpyAsync(sv_spins, b->d_spins, words * 4, k, b->stream)
                         : cudaMemcpyAsync(b->d_spins, sv_spins, words * 4, k, b->stream);
    if (e == cudaSuccess)
      e = save ? cudaMemcpyAsync(sv_tabs, b->d_tabs, tabs * 4, k, b->stream)
               : cudaMemcpyAsync(b->d_tabs, sv_tabs, tabs * 4, k, b->stream);
    if (e == cudaSuccess && ring_obs)
      e = save ? cudaMemcpyAsync(sv_obs, b->d_obs, ring_obs * 8, k, b->stream)
               : cudaMemcpyAsync(b->d_obs, sv_obs, ring_obs * 8, k, b->stream);
    if (e == cudaSuccess && ring_tau)
      e = save ? cudaMemcpyAsync(sv_ring, b->d_tau_ring, ring_tau * 4, k, b->stream)
               : cudaMemcpyAsync(b->d_tau_ring, sv_ring, ring_tau * 4, k, b->stream);
    for (size_t g = 0; g < b->groups.size() && e == cudaSuccess; ++g) {
      GroupHost& G = b->groups[g];
      const size_t n = (size_t)G.n_rep;
      int* a = sv_int[g];
      unsigned long long* c = sv_cnt[g];
      if (save) {
        e = cudaMemcpyAsync(a, G.d_tau, n * 4, k, b->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(a + n, G.d_rep_at, n * 4, k, b->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(c, G.d_acc, n * 8, k, b->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(c + n, G.d_att, n * 8, k, b->stream);
      } else {
        e = cudaMemcpyAsync(G.d_tau, a, n * 4, k, b->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(G.d_rep_at, a + n, n * 4, k, b->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(G.d_acc, c, n * 8, k, b->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(G.d_att, c + n, n * 8, k, b->stream);
      }
    }
    return e;
  };
  cudaError_t e = copy_state(true);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  if (e == cudaSuccess && (rc = ensure_ring(b, rounds + 1))) {  // after the saved copy: growing drops the ring
    release();
    return rc;
  }
  const vg_batch_tuning keep = b->tune;
  vg_batch_tuning top = keep;
  double top_ms = 1e300;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  if (b->graph) {
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  static const int kTpb[2] = {128, 256}, kWpt[3] = {2, 4, 8}, kWif[2] = {1, 2};
  for (int it = 0; it < 2 && e == cudaSuccess && !rc; ++it)
    for (int iw = 0; iw < 3 && e == cudaSuccess && !rc; ++iw)
      for (int ii = 0; ii < 2 && e == cudaSuccess && !rc; ++ii) {
        b->tune = vg_batch_tuning{kTpb[it], kWpt[iw], kWif[ii]};
        if ((rc = build_blocks(b))) break;
        const MscDev d{(uint32_t)b->sweep, b->round, b->round, 0};
        e = cudaMemcpyAsync(b->d_dev, &d, sizeof(d), cudaMemcpyHostToDevice, b->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
        if (e == cudaSuccess && (rc = enqueue_round(b))) break;  // warm-up round
        if (e == cudaSuccess) e = cudaEventRecord(e0, b->stream);
        for (uint32_t r = 0; r < rounds && e == cudaSuccess && !rc; ++r) rc = enqueue_round(b);
        if (e == cudaSuccess) e = cudaEventRecord(e1, b->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
        float ms = 0.f;
        if (e == cudaSuccess && !rc) e = cudaEventElapsedTime(&ms, e0, e1);
        if (e == cudaSuccess && !rc && ms / rounds < top_ms) {
          top_ms = ms / rounds;
          top = b->tune;
        }
      }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  // restore the state and the counters, keep the fastest shape
  b->tune = (e == cudaSuccess && !rc) ? top : keep;
  int rc2 = build_blocks(b);
  const MscDev d{(uint32_t)b->sweep, b->round, b->round - (uint32_t)b->last_rounds, 0};
  cudaError_t e2 = copy_state(false);
  if (e2 == cudaSuccess) e2 = cudaMemcpyAsync(b->d_dev, &d, sizeof(d), cudaMemcpyHostToDevice, b->stream);
  if (e2 == cudaSuccess) e2 = cudaStreamSynchronize(b->stream);
  release();
  if (rc) return rc;
  if (e != cudaSuccess) return bfail(b, VG_ERR_CUDA, std::string("autotune: ") + cudaGetErrorString(e));
  if (rc2) return rc2;
  if (e2 != cudaSuccess) return bfail(b, VG_ERR_CUDA, std::string("autotune restore: ") + cudaGetErrorString(e2));
  if (best) *best = top;
  if (best_ms) *best_ms = top_ms;
  return VG_OK;
}

int vg_batch_get_replica(vg_batch* b, int32_t group, int32_t replica, int8_t* spins) {
  if (!b || !spins) return VG_ERR_INVALID_ARG;
  MscSeg sg;
  uint32_t lane;
  int rc = find_replica(b, group, replica, &sg, &lane);
  if (rc) return rc;
  const long long n = 2LL * sg.n_c;
  if ((rc = ensure_stage(b, n))) return rc;
  msc_get<<<256, 256, 0, b->stream>>>(sg, lane, b->d_stage);
  VG_BCUDA(b, cudaGetLastError());
  VG_BCUDA(b, cudaMemcpyAsync(spins, b->d_stage, (size_t)n, cudaMemcpyDeviceToHost, b->stream));
  VG_BCUDA(b, cudaStreamSynchronize(b->stream));
  return VG_OK;
}

int vg_batch_set_replica(vg_batch* b, int32_t group, int32_t replica, const int8_t* spins) {
  if (!b || !spins) return VG_ERR_INVALID_ARG;
  MscSeg sg;
  uint32_t lane;
  int rc = find_replica(b, group, replica, &sg, &lane);
  if (rc) return rc;
  const long long n = 2LL * sg.n_c;
  if ((rc = ensure_stage(b, n))) return rc;
  VG_BCUDA(b, cudaMemcpyAsync(b->d_stage, spins, (size_t)n, cudaMemcpyHostToDevice, b->stream));
  VG_BCUDA(b, cudaMemsetAsync(b->d_flag, 0, sizeof(int), b->stream));
  msc_set<<<256, 256, 0, b->stream>>>(sg, lane, b->d_stage, b->d_flag);
  VG_BCUDA(b, cudaGetLastError());
  int flag = 0;
  VG_BCUDA(b, cudaMemcpyAsync(&flag, b->d_flag, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
  VG_BCUDA(b, cudaStreamSynchronize(b->stream));
  if (flag) return bfail(b, VG_ERR_INVALID_ARG, "Ising spins must be +1 or -1");
  return VG_OK;
}

}  // extern "C"
