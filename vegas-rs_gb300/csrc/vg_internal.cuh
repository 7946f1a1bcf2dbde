// vg_internal.cuh -- shared device helpers and kernel argument blocks of the
// vegas GB300 engine.  Nothing here is part of the public C ABI.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <cstring>

#include <utility>

#include "vegas_gpu.h"

namespace vg {

// Programmatic dependent launch: a colour pass lets the next one launch
// while it drains, and every pass waits for its predecessor's writes
// (griddepcontrol.wait) before touching spins or partial sums.  Both are
// no-ops for kernels launched without the PDL attribute.
__device__ __forceinline__ void pdl_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// Launch with programmatic stream serialization (kernels that call pdl_wait
// before reading what their predecessor wrote).
template <typename... P, typename... A>
cudaError_t launch_pdl_ex(void (*kern)(P...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, A&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, std::forward<A>(args)...);
}
template <typename... P, typename... A>
cudaError_t launch_pdl(void (*kern)(P...), int grid, int tpb, cudaStream_t s, A&&... args) {
  return launch_pdl_ex(kern, dim3(grid), dim3(tpb), 0, s, std::forward<A>(args)...);
}

constexpr int kMaxZ = 12;          // fcc coordination
constexpr int kMaxColours = 16;
constexpr int kIsingGroup = 16;    // class entries sharing one Philox block
constexpr int kNumSums = 8;        // members of vg_sums
// The sweep index is Philox counter word 1 (32 bits): a run may use sweep
// indices up to 2^32 - 1, and entry points refuse runs that would go past.
constexpr unsigned long long kSweepLimit = 1ull << 32;
inline bool sweep_range_ok(unsigned long long first, unsigned long long n) {
  return first < kSweepLimit && n <= kSweepLimit - first;
}

// Philox rounds of the Heisenberg update draws (proposal and acceptance, one
// block per site): Salmon et al., "Parallel random numbers: as easy as 1, 2,
// 3" (SC'11), report Philox4x32 passing TestU01's Crush batteries from 7
// rounds on and take 10 as the default for a safety margin of 3 rounds.  The
// per-site block was about a fifth of the FP32 update's instructions.
// Initial states and the Ising draws keep 10 rounds.
constexpr int kHeisRounds = 7;

// Draw-stream tags (bits 24..31 of Philox counter word 2).
enum : uint32_t {
  kTagIsingAccept = 1,
  kTagIsingPropose = 2,
  kTagHeis = 3,
  kTagInitIsing = 4,
  kTagInitHeis = 5
};

// ------------------------------------------------------------ Philox4x32-10
// Salmon et al., "Parallel random numbers: as easy as 1, 2, 3" (SC'11).
// Each round: two 32x32->64 multiplies (one wide multiply each) and two
// three-input XORs with the round key.
__host__ __device__ __forceinline__ uint4 philox(uint4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    if (r) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    const unsigned long long p0 = (unsigned long long)0xD2511F53u * c.x;
    const unsigned long long p1 = (unsigned long long)0xCD9E8D57u * c.z;
    c = make_uint4((uint32_t)(p1 >> 32) ^ c.y ^ k0, (uint32_t)p1, (uint32_t)(p0 >> 32) ^ c.w ^ k1, (uint32_t)p0);
  }
  return c;
}

// Round keys precomputed on the host; passed as kernel parameters they are
// read straight from the constant bank by the XORs.
struct KeySchedule {
  uint32_t k0[10], k1[10];
};

inline KeySchedule make_key_schedule(uint32_t k0, uint32_t k1) {
  KeySchedule s;
  for (int r = 0; r < 10; ++r) {
    s.k0[r] = k0 + (uint32_t)r * 0x9E3779B9u;
    s.k1[r] = k1 + (uint32_t)r * 0xBB67AE85u;
  }
  return s;
}

// ROUNDS < 10: the first ROUNDS rounds of the same schedule (Philox4x32-R).
template <int ROUNDS = 10>
__device__ __forceinline__ uint4 philox_ks(uint4 c, const KeySchedule& ks) {
  static_assert(ROUNDS >= 1 && ROUNDS <= 10, "the key schedule holds 10 rounds");
#pragma unroll
  for (int r = 0; r < ROUNDS; ++r) {
    const unsigned long long p0 = (unsigned long long)0xD2511F53u * c.x;
    const unsigned long long p1 = (unsigned long long)0xCD9E8D57u * c.z;
    c = make_uint4((uint32_t)(p1 >> 32) ^ c.y ^ ks.k0[r], (uint32_t)p1, (uint32_t)(p0 >> 32) ^ c.w ^ ks.k1[r],
                   (uint32_t)p0);
  }
  return c;
}

__device__ __forceinline__ uint32_t blk_byte(const uint4& b, int k) {
  const uint32_t w = (k >> 2) == 0 ? b.x : (k >> 2) == 1 ? b.y : (k >> 2) == 2 ? b.z : b.w;
  return (w >> (8 * (k & 3))) & 0xFFu;
}

// Division by a runtime constant d for dividends n < 2^31: one multiply-high,
// one add, one shift (q = (umulhi(n, m) + n) >> s with s = ceil(log2 d),
// m = floor(2^32 (2^s - d) / d) + 1).
struct FastDiv {
  uint32_t d, m, s;
};

inline FastDiv make_fastdiv(uint32_t d) {
  FastDiv f;
  f.d = d;
  f.s = 0;
  while ((1ull << f.s) < d) ++f.s;
  f.m = (uint32_t)((((1ull << 32) * ((1ull << f.s) - d)) / d) + 1);
  return f;
}

__device__ __forceinline__ uint32_t fdiv(uint32_t n, const FastDiv& f) { return (__umulhi(n, f.m) + n) >> f.s; }

// Ising acceptance table: index s*(2z+1) + nsum + z, value = threshold on a
// 32-bit uniform (accept iff U < thr); thr >= 2^32 means always.
// For lattices where every site has zeff existing neighbours (zeff < 0
// otherwise), byte tables indexed by the up-neighbour count n_up in
// [0, zeff]: top[s][.] holds the most significant byte of thr(s, n_up)
// (0xFF where the move always accepts); [0] = entries 0..3, [1] = 4..7.
struct IsingTable {
  unsigned long long thr[2 * (2 * kMaxZ + 1)];
  uint32_t top[2][2];
  int zeff;
};

// The acceptance table of the reference's rule (dE < 0 accepts, otherwise
// accept iff u < exp(-dE/T), src/integrator.rs:113-137) for the Ising site
// energy E_i(s) = -J s nsum + hz s (src/energy.rs:147-152, :194-206) with z
// neighbours at most, built in FP64 on the host: thr = ceil(exp(-dE/T) 2^32),
// 2^32 where the move always accepts.  sc: the lattice uses the checkerboard
// kernels, whose byte tables need every site to have the same number of
// existing neighbours (each axis periodic, or open with extent 1); zeeman
// sign, |B| and the field orientation are folded into hz by the caller.
inline IsingTable make_ising_table(double J, double hz, double T, int z, bool sc, const int ext[3],
                                   const int per[3]) {
  IsingTable t;
  std::memset(&t, 0, sizeof(t));
  const int W = 2 * z + 1;
  for (int s01 = 0; s01 < 2; ++s01)
    for (int ns = -z; ns <= z; ++ns) {
      const double s = s01 ? 1.0 : -1.0;
      const double e_old = -J * s * (double)ns + hz * s;
      const double e_new = -J * (-s) * (double)ns + hz * (-s);
      const double de = e_new - e_old;
      unsigned long long thr;
      if (de <= 0.0) {
        thr = 1ull << 32;
      } else {
        const double x = std::ceil(std::exp(-de / T) * 4294967296.0);
        thr = x >= 4294967296.0 ? (1ull << 32) : x <= 0.0 ? 0ull : (unsigned long long)x;
      }
      t.thr[s01 * W + ns + z] = thr;
    }
  t.zeff = -1;
  if (!sc) return t;
  int zeff = 0;
  bool uniform = true;
  for (int a = 0; a < 3; ++a) {
    if (per[a]) zeff += 2;
    else if (ext[a] > 1) uniform = false;
  }
  if (!uniform) return t;
  t.zeff = zeff;
  uint8_t top[2][8] = {};
  for (int s01 = 0; s01 < 2; ++s01)
    for (int nu = 0; nu <= zeff; ++nu) {
      const unsigned long long thr = t.thr[s01 * W + 2 * nu - zeff + z];
      top[s01][nu] = thr >= (1ull << 32) ? 0xFF : (uint8_t)(thr >> 24);
    }
  for (int s01 = 0; s01 < 2; ++s01)
    for (int h = 0; h < 2; ++h)
      t.top[s01][h] = (uint32_t)top[s01][4 * h] | ((uint32_t)top[s01][4 * h + 1] << 8) |
                      ((uint32_t)top[s01][4 * h + 2] << 16) | ((uint32_t)top[s01][4 * h + 3] << 24);
  return t;
}

struct RngKey {
  uint32_t k0, k1, replica, sweep;
  KeySchedule ks;
};

// ------------------------------------------------------------ kernel args
struct IsingScArgs {          // sc checkerboard, class-separated uint8 0/1
  uint8_t* cls[2];
  uint32_t groups;            // 16-site groups per class
  int Hx, Ly, Lz, G;          // Hx = Lx/2, G = Hx/16
  int pbx, pby, pbz;
  FastDiv fG, fLy;
  // byte offsets within a class (a class holds fewer than 2^31 sites): a
  // z plane, and the wrap-around jumps along y and z
  uint32_t plane, ywrap, zwrap;
};

// The offsets of IsingScArgs from its extents (set after Hx, Ly, Lz).
inline void set_sc_offsets(IsingScArgs& a) {
  a.plane = (uint32_t)a.Ly * (uint32_t)a.Hx;
  a.ywrap = (uint32_t)(a.Ly - 1) * (uint32_t)a.Hx;
  a.zwrap = (uint32_t)(a.Lz - 1) * a.plane;
}

// Basis positions in half lattice constants: bcc (0,0,0) (1,1,1); fcc
// (0,0,0) (1,1,0) (1,0,1) (0,1,1) -- the order of Lattice::bcc / fcc.  The
// neighbours of basis b on basis q sit in the cells c + sum over the axes a
// where the two positions differ of {0, +1 if b is at the half position on
// a else -1} e_a.
template <int NB>
__host__ __device__ constexpr int half_pos(int b, int a) {
  return NB == 2 ? (b == 1 ? 1 : 0) : (((b == 1 && a != 2) || (b == 2 && a != 1) || (b == 3 && a != 0)) ? 1 : 0);
}

struct IsingSubArgs {         // bcc / fcc: one uint8 0/1 array per sublattice, [class][cell]
  uint8_t* base;              // class q at base + q * ncell, cell = (z ny + y) nx + x
  uint32_t ncell, groups;     // cells per class, 16-cell runs per class (nx a multiple of 16)
  int nx, ny, nz, z;          // z: coordination (8 or 12)
  int pbx, pby, pbz;
  FastDiv fnx, fny;
};

struct IsingGenArgs {         // any lattice: natural order uint8 0/1 + ELL
  uint8_t* spin;
  const int32_t* sites;       // class entry -> site
  const int32_t* nbr;         // [z][n_c] neighbour sites (-1 absent)
  const uint32_t* lowmask;    // bit k: neighbour k has a lower colour
  long long n_c;
  int z;
  const double* jb;           // [z][n_c] per-bond exchange constants, or null (uniform J, table thresholds)
  double hz;                  // per-bond path: per-site Zeeman coefficient (field orientation folded in)
  double T;                   // per-bond path: temperature (clamped)
};

// One Ising sweep per launch on a fully periodic sc checkerboard lattice
// (vg_tiled.cu): both classes of a tile of whole x rows staged in shared
// memory with halos; a sweep reads the class arrays `in` and writes `out`.
struct IsingTileArgs {
  const uint8_t* in[2];
  uint8_t* out[2];
  int Hx, Ly, Lz, G;          // Hx = Lx/2 bytes per class row, G = Hx/16 (even)
  int nyt, nzt;               // tiles along y and z (grid = nyt x nzt blocks)
  int TY, TZm;                // the tiles' y extent (nyt divides Ly), the largest z extent
  FastDiv fG2, fny0, fny;     // by G/2, TY + 2 (the class-0 box), TY
  int* err;                   // set to 1 if a block's staging wait ran out (then it writes nothing)
};
constexpr size_t kTileSmemMax = 200 * 1024;  // dynamic shared memory per block

template <typename R>
struct HeisScArgs {           // sc checkerboard, class-separated SoA
  R* x[2];
  R* y[2];
  R* z[2];
  uint32_t n_c;               // sites per class
  int Hx, Ly, Lz;
  int pbx, pby, pbz;
  FastDiv fHx, fLy;
};

template <typename R>
struct HeisSubArgs {          // bcc / fcc: SoA planes per sublattice, [class][xyz][cell]
  R* spin;
  uint32_t ncell;             // cells per class (3 x classes x ncell < 2^32)
  int nx, ny, nz;
  int pbx, pby, pbz;
  uint32_t runs;              // ncell / W
  FastDiv frow;               // run index -> row (runs per row = nx / W)
  FastDiv fny;
  int rpr;                    // runs per row
};

template <typename R>
struct HeisGenArgs {          // any lattice: natural order SoA + ELL
  R* x;
  R* y;
  R* z;
  const int32_t* sites;
  const int32_t* nbr;
  const uint32_t* lowmask;
  long long n_c;
  int zc;
  const R* jb;                // [zc][n_c] per-bond exchange constants (then P.J = 1), or null
};

template <typename R>
struct HeisParams {
  R J, K, ax, ay, az, hz, bx, by, bz, Kc, beta;
  R T;
};

// ------------------------------------------------------------ launchers
// Each launcher enqueues one colour pass; part (may be null) receives one
// row of kNumSums partials per block (int64 for Ising, double for
// Heisenberg).  update = false only measures.
cudaError_t launch_ising_sc(const IsingScArgs& a, const IsingTable& tab, RngKey key, int colour,
                            int proposal, bool update, long long* part, int grid, int tpb, cudaStream_t s);
int ising_sc_blocks_per_sm(const IsingScArgs& a, const IsingTable& tab, int tpb);
// Wolff cluster steps on natural-order int8 +-1 spins, one block.
size_t ising_wolff_smem(int n);
// The same steps in one block for lattices whose spins and cluster marks fit
// its shared memory as bits (ising_wolff_mid_smem(n) bytes); q: the cluster
// queue in global memory, n entries.
size_t ising_wolff_mid_smem(int n);
cudaError_t launch_ising_wolff_mid(int8_t* spins, int n, int z, const int32_t* nbr, const uint8_t* occ,
                                   unsigned long long thr, RngKey key, uint32_t n_steps, double* sums, int32_t* q,
                                   cudaStream_t s);
// The same steps over the whole grid (one cooperative launch) for lattices
// beyond one block: spins, stamps (mark, n words) and queue (q, n entries)
// in global memory; g is zeroed by the launcher, and g->abort_flag != 0
// after the launch means a grid barrier gave up.
constexpr int kWolffGridTpb = 512;
struct WolffGrid {
  unsigned int cnt[3];                // appends of level L go to cnt[L % 3]
  unsigned int bar_count;             // grid barrier: arrivals
  unsigned int abort_flag;
  unsigned long long bar_word;        // grid barrier: generation << 32 | handed value
  unsigned long long cut;             // this step's sum of boundary spins (two's complement)
  unsigned long long bond0, ups0;     // sums of the incoming state
};
// One grid barrier over `blocks` blocks of 32 threads (a cooperative launch)
// where block `skip` (none if skip < 0) never arrives; g->abort_flag tells
// whether a wait ran out.
cudaError_t launch_wolff_barrier_probe(WolffGrid* g, int blocks, int skip, cudaStream_t s);
cudaError_t launch_ising_wolff_grid(int8_t* spins, int n, int z, const int32_t* nbr, const uint8_t* occ,
                                    unsigned long long thr, RngKey key, uint32_t n_steps, double* sums,
                                    uint32_t* mark, int32_t* q, WolffGrid* g, int sm_count, cudaStream_t s);
cudaError_t launch_ising_wolff(int8_t* spins, int n, int z, const int32_t* nbr, const uint8_t* occ,
                               unsigned long long thr, RngKey key, uint32_t n_steps, double* sums, cudaStream_t s);
// Per-site energies and single-site energy changes on natural-order copies
// of the state (int8 +-1, or [n][3] doubles); jnat (may be null): per-bond
// constants in neighbour-table layout [n][z].
struct SiteTerms {
  int has_exchange, has_anisotropy, has_zeeman, has_gauge, has_cubic;
  double J, K, axis[3], hz, b[3], gauge, Kc;
  double axis_sign, field_sign;  // Ising: the z signs of the axis and the field
};
cudaError_t launch_site_energies(bool ising, const void* spins, int64_t n, int z, const int32_t* nbr,
                                 const double* jnat, const SiteTerms& t, double* out, cudaStream_t s);
template <typename R>
cudaError_t launch_heis_delta(const double* spins, const double* prop, int64_t n, int z, const int32_t* nbr,
                              const double* jnat, const HeisParams<R>& P, double* out, cudaStream_t s);
// One colour (sublattice) pass of a bcc / fcc Ising lattice.
cudaError_t launch_ising_sub(const IsingSubArgs& a, int nb, const IsingTable& tab, RngKey key, int colour,
                             int proposal, bool update, long long* part, int grid, int tpb, cudaStream_t s);
size_t ising_resident_smem(const IsingScArgs& a);
// The tiled sweep kernel: its tiling for a lattice (false if none fits), its
// dynamic shared memory, the per-device opt-in, and one sweep (part: one row
// of sums per tile, or null).
bool ising_tile_plan(int Hx, int Ly, int Lz, int sm_count, IsingTileArgs* a);
size_t ising_tile_smem(int Hx, int TY, int TZm);
cudaError_t ising_tile_prepare();
cudaError_t launch_ising_tile_sweep(const IsingTileArgs& a, const IsingTable& tab, RngKey key, int proposal,
                                    long long* part, cudaStream_t s);
cudaError_t launch_ising_resident(const IsingScArgs& a, const IsingTable& tab, RngKey key, int proposal,
                                  uint32_t n_sweeps, double* sums, int tpb, cudaStream_t s);
cudaError_t launch_ising_gen(const IsingGenArgs& a, const IsingTable& tab, RngKey key, int colour,
                             int proposal, bool update, long long* part, int grid, int tpb,
                             cudaStream_t s);
template <typename R>
cudaError_t launch_heis_sc(const HeisScArgs<R>& a, const HeisParams<R>& p, RngKey key, int colour,
                           int proposal, bool update, double* part, int grid, int tpb,
                           cudaStream_t s);
// bcc / fcc sublattice pass; nb = basis size, W = cells per run (4 when nx
// is a multiple of 4, else 1).
template <typename R>
cudaError_t launch_heis_sub(const HeisSubArgs<R>& a, int nb, int W, const HeisParams<R>& p, RngKey key, int colour,
                            int proposal, bool update, double* part, int grid, int tpb, cudaStream_t s);
template <typename R>
cudaError_t launch_heis_gen(const HeisGenArgs<R>& a, const HeisParams<R>& p, RngKey key, int colour,
                            int proposal, bool update, double* part, int grid, int tpb,
                            cudaStream_t s);

// ------------------------------------------------------------ reductions
// Block-wide sum of kNumSums values into row `out` (thread 0 writes).
template <typename T>
__device__ __forceinline__ void block_sum_store(T (&v)[kNumSums], T* out) {
  __shared__ T red[32][kNumSums];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < kNumSums; ++i) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[i] += __shfl_down_sync(0xffffffffu, v[i], o);
  }
  if (lane == 0) {
#pragma unroll
    for (int i = 0; i < kNumSums; ++i) red[warp][i] = v[i];
  }
  __syncthreads();
  if (warp == 0) {
    const int nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int i = 0; i < kNumSums; ++i) {
      T t = lane < nw ? red[lane][i] : T(0);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
      if (lane == 0) out[i] = t;
    }
  }
}

}  // namespace vg
