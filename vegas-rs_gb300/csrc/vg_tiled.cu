// vg_tiled.cu -- one launch per Ising sweep: both colour passes of a fully
// periodic sc checkerboard lattice inside shared-memory tiles with halos.
//
// Replaces the two colour passes of MetropolisFlipIntegrator::step /
// MetropolisIntegrator::step for IsingSpin (src/integrator.rs:66-137) with
// the same decisions as the per-pass kernels (vg_ising.cu): the same Philox
// blocks per 16-site group (counter: group index within the class, sweep,
// tag << 24 | colour << 8 | digit, replica), the same byte-parallel first-digit
// compare and the same tie resolution, so results are bit-identical.
//
// A block owns a tile of whole x rows, y in [y0, y1) and z in [z0, z1) (the
// tiles partition the y-z plane of rows).  It copies class 1 over the tile
// grown by two rows in y and z and class 0 over the tile grown by one into
// shared memory, runs colour 0 on the grown class-0 box -- the ring around
// the tile is computed redundantly: the neighbouring tiles compute the same
// sites from the same inputs and draws and get the same spins -- then colour
// 1 on the tile, whose class-0 neighbours are all in the box and updated,
// and writes both classes of the tile.  Blocks read halo rows that other
// blocks rewrite in the same launch, so a sweep reads one buffer of a pair
// and writes the other (the context alternates them).  Against two passes
// per sweep this removes one launch boundary per sweep (its fill, drain and
// wait) and serves every neighbour load from shared memory instead of L2.
#include <cuda_runtime.h>

#include <algorithm>

#include "vg_ising_bytes.cuh"

namespace vg {

namespace {

constexpr int kTileThreads = 1024;
constexpr int kTileQueue = 64;  // per-warp tie queue

struct TileGeom {  // one block's tile
  int y0, z0, TY, TZ;
};

__device__ __forceinline__ TileGeom tile_of(const IsingTileArgs& a) {
  const int ty = (int)(blockIdx.x % (unsigned)a.nyt), tz = (int)(blockIdx.x / (unsigned)a.nyt);
  TileGeom t;
  t.y0 = ty * a.Ly / a.nyt;
  t.z0 = tz * a.Lz / a.nzt;
  t.TY = (ty + 1) * a.Ly / a.nyt - t.y0;
  t.TZ = (tz + 1) * a.Lz / a.nzt - t.z0;
  return t;
}

// FastDiv (vg_internal.cuh) formed on the device, for divisors that differ
// between blocks.
__device__ __forceinline__ FastDiv fastdiv_dev(uint32_t d) {
  FastDiv f;
  f.d = d;
  f.s = d > 1u ? 32u - (uint32_t)__clz(d - 1u) : 0u;
  f.m = (uint32_t)((((1ull << 32) * ((1ull << f.s) - d)) / d) + 1ull);
  return f;
}

__device__ __forceinline__ int wrap(int v, int n) { return v < 0 ? v + n : (v >= n ? v - n : v); }

// Byte offsets of box rows in shared memory: class 1 over [-2, T + 2),
// class 0 over [-1, T + 1), rows [z][y] with the largest tile's y stride.
__device__ __forceinline__ uint32_t row1(const IsingTileArgs& a, int dy, int dz) {
  return (uint32_t)((dz + 2) * (a.TYm + 4) + (dy + 2)) * (uint32_t)a.Hx;
}
__device__ __forceinline__ uint32_t row0(const IsingTileArgs& a, int dy, int dz) {
  return (uint32_t)((dz + 1) * (a.TYm + 2) + (dy + 1)) * (uint32_t)a.Hx;
}

// Copy box rows [lo, TY + hi) x [lo, TZ + hi) of class c between global
// memory and shared memory (load: global -> shared; else shared -> global
// for the tile's own rows, lo = hi = 0).
template <bool LOAD>
__device__ __forceinline__ void copy_rows(const IsingTileArgs& a, const TileGeom& t, int c, int lo, int hi,
                                          uint8_t* sm) {
  const int ny = t.TY + hi - lo, nz = t.TZ + hi - lo;
  const uint32_t per_row = (uint32_t)a.G;  // 16-byte words per row
  const uint32_t items = (uint32_t)(ny * nz) * per_row;
  const FastDiv fny = fastdiv_dev((uint32_t)ny);
  for (uint32_t i = threadIdx.x; i < items; i += blockDim.x) {
    const uint32_t r = fdiv(i, a.fG), w = i - r * per_row;
    const int bz = (int)fdiv(r, fny), by = (int)r - bz * ny;
    const int dy = by + lo, dz = bz + lo;
    const uint32_t gy = (uint32_t)wrap(t.y0 + dy, a.Ly), gz = (uint32_t)wrap(t.z0 + dz, a.Lz);
    const uint32_t goff = (gz * (uint32_t)a.Ly + gy) * (uint32_t)a.Hx + 16u * w;
    const uint32_t soff = (c ? row1(a, dy, dz) : row0(a, dy, dz)) + 16u * w;
    if (LOAD) {
      *reinterpret_cast<uint4*>(sm + soff) = __ldg(reinterpret_cast<const uint4*>(a.in[c] + goff));
    } else {
      *reinterpret_cast<uint4*>(a.out[c] + goff) = *reinterpret_cast<const uint4*>(sm + soff);
    }
  }
}

// One colour pass over the box rows [lo, TY + hi) x [lo, TZ + hi) of class C
// (own rows in `own`, neighbour rows in `oth`, both in shared memory);
// measures the tile's own rows.  Decisions as sc1_range (vg_ising.cu):
// uniform coordination 6, byte-parallel first digit, ties queued per warp.
template <int C, bool MEASURE, int PROP>
__device__ __forceinline__ void tile_pass(const IsingTileArgs& a, const TileGeom& t, int lo, int hi, uint8_t* own,
                                          const uint8_t* oth, const IsingTable& tab, const RngKey& key,
                                          const unsigned long long* s_thr, uint2 (*s_q)[kTileQueue], int& bond,
                                          int& ups, int& nacc) {
  constexpr int Z = 6;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int ny = t.TY + hi - lo, nz = t.TZ + hi - lo;
  const uint32_t G = (uint32_t)a.G;
  const uint32_t items = (uint32_t)(ny * nz) * G;
  const FastDiv fny = fastdiv_dev((uint32_t)ny);
  int qn = 0;  // warp-uniform queue length

  // decide the first n queued ties (one per lane), then drop them
  auto drain = [&](int n) {
    __syncwarp();
    if (lane < n) {
      const uint2 e = s_q[warp][lane];
      const int k = (int)(e.y & 15u);
      const uint32_t s01 = (e.y >> 4) & 1u, nu = (e.y >> 5) & 7u, inner = (e.y >> 8) & 1u;
      if (resolve_tie(e.x >> 0, k, s01, nu, Z, C, s_thr, key)) {
        own[(e.y >> 9) * 16u + (uint32_t)k] = (uint8_t)(s01 ^ 1u);
        if (MEASURE && inner) {
          ups += 1 - 2 * (int)s01;
          nacc += 1;
          if (C == 1) bond -= 2 * (2 * (int)s01 - 1) * (2 * (int)nu - Z);
        }
      }
    }
    __syncwarp();
    const int rest = qn - n;
    uint2 mv = make_uint2(0, 0);
    if (lane < rest) mv = s_q[warp][n + lane];
    __syncwarp();
    if (lane < rest) s_q[warp][lane] = mv;
    __syncwarp();
    qn = rest;
  };

  // whole warps walk the items (the queue needs every lane at its ballots)
  const uint32_t first = threadIdx.x & ~31u, step = blockDim.x;
  for (uint32_t base = first; base < items; base += step) {
    const uint32_t i = base + (uint32_t)lane;
    const bool active = i < items;
    uint32_t tm = 0, sgrp = 0, gid = 0;
    uint32_t S[4] = {0, 0, 0, 0}, A[4] = {0, 0, 0, 0};
    bool inner = false;
    if (active) {
      const uint32_t r = fdiv(i, a.fG), g = i - r * G;
      const int bz = (int)fdiv(r, fny), by = (int)r - bz * ny;
      const int dy = by + lo, dz = bz + lo;
      inner = dy >= 0 && dy < t.TY && dz >= 0 && dz < t.TZ;
      const int gy = wrap(t.y0 + dy, a.Ly), gz = wrap(t.z0 + dz, a.Lz);
      const int p = (gy + gz + C) & 1;  // x parity of this row's class-C sites
      gid = ((uint32_t)gz * (uint32_t)a.Ly + (uint32_t)gy) * G + g;
      const uint32_t h0 = 16u * g;
      const uint32_t ro = (C ? row1(a, dy, dz) : row0(a, dy, dz));
      sgrp = (ro + h0) >> 4;
      auto orow = [&](int y, int z) { return C ? row0(a, y, z) : row1(a, y, z); };
      const uint32_t rx = orow(dy, dz);
      const uint4 Sv = *reinterpret_cast<const uint4*>(own + ro + h0);
      const uint4 X0 = *reinterpret_cast<const uint4*>(oth + rx + h0);
      const uint32_t e = p == 0 ? oth[rx + (h0 == 0 ? (uint32_t)a.Hx - 1u : h0 - 1u)]
                                : oth[rx + (h0 + 16u == (uint32_t)a.Hx ? 0u : h0 + 16u)];
      uint32_t X1[4];
      if (p == 0) {
        X1[0] = __byte_perm(e << 24, X0.x, 0x6543);
        X1[1] = __byte_perm(X0.x, X0.y, 0x6543);
        X1[2] = __byte_perm(X0.y, X0.z, 0x6543);
        X1[3] = __byte_perm(X0.z, X0.w, 0x6543);
      } else {
        X1[0] = __byte_perm(X0.x, X0.y, 0x4321);
        X1[1] = __byte_perm(X0.y, X0.z, 0x4321);
        X1[2] = __byte_perm(X0.z, X0.w, 0x4321);
        X1[3] = __byte_perm(X0.w, e, 0x4321);
      }
      const uint4 Ym = *reinterpret_cast<const uint4*>(oth + orow(dy - 1, dz) + h0);
      const uint4 Yp = *reinterpret_cast<const uint4*>(oth + orow(dy + 1, dz) + h0);
      const uint4 Zm = *reinterpret_cast<const uint4*>(oth + orow(dy, dz - 1) + h0);
      const uint4 Zp = *reinterpret_cast<const uint4*>(oth + orow(dy, dz + 1) + h0);
      S[0] = Sv.x;
      S[1] = Sv.y;
      S[2] = Sv.z;
      S[3] = Sv.w;
      A[0] = X0.x + X1[0] + Ym.x + Yp.x + Zm.x + Zp.x;
      A[1] = X0.y + X1[1] + Ym.y + Yp.y + Zm.y + Zp.y;
      A[2] = X0.z + X1[2] + Ym.z + Yp.z + Zm.z + Zp.z;
      A[3] = X0.w + X1[3] + Ym.w + Yp.w + Zm.w + Zp.w;

      uint32_t cand[4] = {0x01010101u, 0x01010101u, 0x01010101u, 0x01010101u};
      if (PROP == VG_PROPOSE_RANDOM) {
        const uint4 b = philox_ks(make_uint4(gid, key.sweep, (kTagIsingPropose << 24) | ((uint32_t)C << 8), key.replica),
                                  key.ks);
        const uint32_t w[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
        for (int j = 0; j < 4; ++j) cand[j] = ((~w[j] >> 7) & 0x01010101u) ^ S[j];
      }
      const uint4 b = philox_ks(make_uint4(gid, key.sweep, (kTagIsingAccept << 24) | ((uint32_t)C << 8), key.replica),
                                key.ks);
      const uint32_t R[4] = {b.x, b.y, b.z, b.w};
      uint32_t F[4], anytie = 0;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const uint32_t sel = nibble_selector(A[j]);
        const uint32_t sm = S[j] * 0xFFu;
        const uint32_t thr = (__byte_perm(tab.top[1][0], tab.top[1][1], sel) & sm) |
                             (__byte_perm(tab.top[0][0], tab.top[0][1], sel) & ~sm);
        F[j] = (bytes_gt80(thr, R[j]) >> 7) & cand[j];
        const uint32_t x = R[j] ^ thr;
        anytie |= (x - 0x01010101u) & ~x & 0x80808080u;  // nonzero iff some byte of x is zero
        if (anytie) tm |= gather4(bytes_zero(x) & cand[j]) << (4 * j);
      }
      uint32_t Sn[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) Sn[j] = S[j] ^ F[j];
      if ((F[0] | F[1] | F[2] | F[3]) != 0u)
        *reinterpret_cast<uint4*>(own + ro + h0) = make_uint4(Sn[0], Sn[1], Sn[2], Sn[3]);
      if (MEASURE && inner) {
        unsigned su = 0, sf = 0;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          su = __dp4a(Sn[j], 0x01010101u, su);
          sf = __dp4a(F[j], 0x01010101u, sf);
        }
        ups += (int)su;
        nacc += (int)sf;
        if (C == 1) {  // every neighbour of class 1 has the lower colour: all bonds counted here
          unsigned sm = 0, m = 0;
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const uint32_t M = 2u * A[j];  // neighbour sum + Z per byte
            sm = __dp4a(Sn[j], M, sm);
            m = __dp4a(M, 0x01010101u, m);
          }
          bond += 2 * (int)sm - (int)m - Z * (2 * (int)su - 16);
        }
      }
    }
    // queue this round's ties, one site per lane per round
    unsigned lanes = __ballot_sync(0xffffffffu, tm != 0u);
    while (lanes) {
      if (qn + 32 > kTileQueue) drain(32 < qn ? 32 : qn);
      const int pos = qn + __popc(lanes & ((1u << lane) - 1u));
      if (tm) {
        const int k = __ffs(tm) - 1;
        tm &= tm - 1u;
        const uint32_t sk = byte_at(S[0], S[1], S[2], S[3], k);
        const uint32_t nk = byte_at(A[0], A[1], A[2], A[3], k);
        s_q[warp][pos] = make_uint2(gid, (uint32_t)k | (sk << 4) | (nk << 5) | ((uint32_t)inner << 8) | (sgrp << 9));
      }
      qn += __popc(lanes);
      if (qn >= 32) drain(32);
      lanes = __ballot_sync(0xffffffffu, tm != 0u);
    }
  }
  if (qn > 0) drain(qn);
}

template <bool MEASURE, int PROP>
__global__ void __launch_bounds__(kTileThreads, 1) ising_tile_sweep_kernel(const IsingTileArgs a, const IsingTable tab,
                                                                           const RngKey key, long long* __restrict__ part) {
  extern __shared__ __align__(16) uint8_t s_spin[];  // class-1 box, then class-0 box
  __shared__ unsigned long long s_thr[2 * 13];
  __shared__ uint2 s_q[kTileThreads / 32][kTileQueue];
  uint8_t* s1 = s_spin;
  uint8_t* s0 = s_spin + (size_t)(a.TZm + 4) * (a.TYm + 4) * a.Hx;
  pdl_launch_dependents();
  for (int i = threadIdx.x; i < 2 * 13; i += blockDim.x) s_thr[i] = tab.thr[i];
  const TileGeom t = tile_of(a);
  pdl_wait();  // the previous sweep's writes (and its reads of our output buffer) are complete
  copy_rows<true>(a, t, 1, -2, 2, s1);
  copy_rows<true>(a, t, 0, -1, 1, s0);
  __syncthreads();
  int bond = 0, ups = 0, nacc = 0;
  tile_pass<0, MEASURE, PROP>(a, t, -1, 1, s0, s1, tab, key, s_thr, s_q, bond, ups, nacc);
  __syncthreads();
  tile_pass<1, MEASURE, PROP>(a, t, 0, 0, s1, s0, tab, key, s_thr, s_q, bond, ups, nacc);
  __syncthreads();
  copy_rows<false>(a, t, 0, 0, 0, s0);
  copy_rows<false>(a, t, 1, 0, 0, s1);
  if (MEASURE) block_sum3_store(bond, ups, nacc, part + (size_t)blockIdx.x * kNumSums);
}

template <bool M, int P>
cudaError_t tile_launch(const IsingTileArgs& a, const IsingTable& tab, const RngKey& key, long long* part,
                        size_t smem, cudaStream_t s) {
  return launch_pdl_ex(ising_tile_sweep_kernel<M, P>, dim3((unsigned)(a.nyt * a.nzt)), dim3(kTileThreads), smem, s,
                       a, tab, key, part);
}

}  // namespace

// Opt the sweep kernels in to kTileSmemMax bytes of dynamic shared memory on
// the current device (once per device, before the first launch).
cudaError_t ising_tile_prepare() {
  const int bytes = (int)kTileSmemMax;
  cudaError_t e = cudaFuncSetAttribute(ising_tile_sweep_kernel<true, VG_PROPOSE_FLIP>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(ising_tile_sweep_kernel<false, VG_PROPOSE_FLIP>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(ising_tile_sweep_kernel<true, VG_PROPOSE_RANDOM>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(ising_tile_sweep_kernel<false, VG_PROPOSE_RANDOM>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  return e;
}

size_t ising_tile_smem(int Hx, int TYm, int TZm) {
  return (size_t)((TZm + 4) * (TYm + 4) + (TZm + 2) * (TYm + 2)) * (size_t)Hx;
}

// The tiling of a lattice's y-z plane of rows: nearly equal tiles (extents
// differ by at most one row), as few waves of one block per SM as the
// shared memory allows, then the least grown-box work per wave.  Returns
// false when no tiling fits (rows too long for shared memory).
bool ising_tile_plan(int Hx, int Ly, int Lz, int sm_count, IsingTileArgs* a) {
  double best = 1e300;
  bool found = false;
  for (int nyt = 1; nyt <= Ly; ++nyt) {
    const int TYm = (Ly + nyt - 1) / nyt;
    for (int nzt = 1; nzt <= Lz; ++nzt) {
      const int TZm = (Lz + nzt - 1) / nzt;
      if (ising_tile_smem(Hx, TYm, TZm) > kTileSmemMax) continue;
      const long long tiles = (long long)nyt * nzt;
      const long long waves = (tiles + sm_count - 1) / sm_count;
      // per wave: colour 0 on the grown box, colour 1 on the tile, loads of
      // both boxes and stores of the tile (weights: relative costs per row)
      const double work = 1.0 * (TYm + 2) * (TZm + 2) + 1.0 * TYm * TZm + 0.35 * ((TYm + 4) * (TZm + 4) +
                          (TYm + 2) * (TZm + 2) + 2 * TYm * TZm) + 40.0;
      const double cost = (double)waves * work;
      if (cost < best) {
        best = cost;
        found = true;
        a->nyt = nyt;
        a->nzt = nzt;
        a->TYm = TYm;
        a->TZm = TZm;
      }
    }
  }
  return found;
}

cudaError_t launch_ising_tile_sweep(const IsingTileArgs& a, const IsingTable& tab, RngKey key, int proposal,
                                    long long* part, cudaStream_t s) {
  const size_t smem = ising_tile_smem(a.Hx, a.TYm, a.TZm);
  if (proposal == VG_PROPOSE_FLIP)
    return part ? tile_launch<true, VG_PROPOSE_FLIP>(a, tab, key, part, smem, s)
                : tile_launch<false, VG_PROPOSE_FLIP>(a, tab, key, part, smem, s);
  return part ? tile_launch<true, VG_PROPOSE_RANDOM>(a, tab, key, part, smem, s)
              : tile_launch<false, VG_PROPOSE_RANDOM>(a, tab, key, part, smem, s);
}

}  // namespace vg
