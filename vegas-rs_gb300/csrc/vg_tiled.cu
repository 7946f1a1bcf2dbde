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
// A block owns a tile of whole x rows, y in [y0, y0 + TY) and z in
// [z0, z0 + TZ) (the tiles partition the y-z plane of rows).  It stages
// class 1 over the tile grown by two rows in y and z and class 0 over the
// tile grown by one in shared memory (bulk asynchronous copies, one or two
// per z plane, completing on an mbarrier), runs colour 0 on the grown
// class-0 box -- the ring around the tile is computed redundantly: the
// neighbouring tiles compute the same sites from the same inputs and draws
// and get the same spins -- then colour 1 on the tile, whose class-0
// neighbours are all in the box and updated, and writes both classes of the
// tile back with bulk copies.  Blocks read halo rows that other blocks
// rewrite in the same launch, so a sweep reads one buffer of a pair and
// writes the other (the context alternates them).  Against two passes per
// sweep this removes one launch boundary per sweep and serves every
// neighbour load from shared memory instead of L2.
//
// A thread takes two consecutive 16-site groups of a row at a time (rows
// hold an even number of groups), as the pair kernel of the per-pass path:
// index arithmetic, row offsets and the x-edge byte are shared by the pair.
#include <cuda_runtime.h>

#include <algorithm>

#include "vg_ising_bytes.cuh"

namespace vg {

namespace {

constexpr int kTileThreads = 768;          // 24 warps; 80 registers each (the pair state)
constexpr int kTileQueue = 64;             // per-warp tie queue
constexpr unsigned kWaitTries = 1u << 22;  // bound on the mbarrier polls of the staging wait

struct TileGeom {  // one block's tile
  int y0, z0, TZ;
};

__device__ __forceinline__ TileGeom tile_of(const IsingTileArgs& a) {
  const int ty = (int)(blockIdx.x % (unsigned)a.nyt), tz = (int)(blockIdx.x / (unsigned)a.nyt);
  TileGeom t;
  t.y0 = ty * a.TY;
  t.z0 = tz * a.Lz / a.nzt;
  t.TZ = (tz + 1) * a.Lz / a.nzt - t.z0;
  return t;
}

__device__ __forceinline__ int wrap(int v, int n) { return v < 0 ? v + n : (v >= n ? v - n : v); }

// Byte offsets of box rows in shared memory: class 1 over [-2, T + 2),
// class 0 over [-1, T + 1), rows [z][y].
__device__ __forceinline__ uint32_t row1(const IsingTileArgs& a, int dy, int dz) {
  return (uint32_t)((dz + 2) * (a.TY + 4) + (dy + 2)) * (uint32_t)a.Hx;
}
__device__ __forceinline__ uint32_t row0(const IsingTileArgs& a, int dy, int dz) {
  return (uint32_t)((dz + 1) * (a.TY + 2) + (dy + 1)) * (uint32_t)a.Hx;
}

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// A bulk copy between a class array and a box: byte offsets in both, length.
struct Copy {
  uint32_t goff, soff, bytes;
};

// The copies of one z plane of the box rows [lo, TY + hi) of class c: the
// plane's rows are contiguous in both places except where y wraps around,
// which splits them -- in three when one tile spans all of y (the range
// [-2, Ly + 2) wraps at both ends; Ly >= 4 keeps it below 2 Ly).
__device__ __forceinline__ int plane_copies(const IsingTileArgs& a, const TileGeom& t, int c, int lo, int hi, int dz,
                                            Copy (&out)[3]) {
  const int gz = wrap(t.z0 + dz, a.Lz);
  const int ylo = t.y0 + lo, yhi = t.y0 + a.TY + hi;  // global y range (may leave [0, Ly))
  const uint32_t plane = (uint32_t)gz * (uint32_t)a.Ly;
  int n = 0;
  for (int y = ylo; y < yhi && n < 3;) {
    const int gy = wrap(y, a.Ly);
    const int run = min(yhi - y, a.Ly - gy);  // rows until the end of the range or the wrap
    out[n].goff = (plane + (uint32_t)gy) * (uint32_t)a.Hx;
    out[n].soff = c ? row1(a, y - t.y0, dz) : row0(a, y - t.y0, dz);
    out[n].bytes = (uint32_t)run * (uint32_t)a.Hx;
    ++n;
    y += run;
  }
  return n;
}

// The class-0 box planes [-1, -1 + P) that the first round of colour-0
// items can touch (a round is one item per thread), and with them class-1
// planes [-2, P): the first of the two staging chunks.
__device__ __forceinline__ int first_chunk_planes(const IsingTileArgs& a, const TileGeom& t) {
  const int per_plane = (a.TY + 2) * (a.G >> 1);  // colour-0 items per box plane
  return min(t.TZ + 2, ((int)blockDim.x + per_plane - 1) / per_plane);
}

// Stage both boxes in two chunks, each completing on its own mbarrier:
// thread 0 registers each chunk's bytes, then lane k of warp 0 issues the
// copies of planes k, k + 32, ... (first chunk first).
__device__ __forceinline__ void stage_boxes(const IsingTileArgs& a, const TileGeom& t, uint8_t* s1, uint8_t* s0,
                                            uint64_t* mbar) {
  const int n1 = t.TZ + 4, n0 = t.TZ + 2;
  const int P = first_chunk_planes(a, t);
  // chunk 0: class-1 planes [-2, P), class-0 planes [-1, -1 + P); chunk 1: the rest
  const int c1a = P + 2, c0a = P;
  if (threadIdx.x == 0) {
    const uint32_t b0 = (uint32_t)((a.TY + 4) * c1a + (a.TY + 2) * c0a) * (uint32_t)a.Hx;
    const uint32_t b1 = (uint32_t)((a.TY + 4) * (n1 - c1a) + (a.TY + 2) * (n0 - c0a)) * (uint32_t)a.Hx;
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_addr(mbar)), "r"(b0)
                 : "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_addr(mbar + 1)), "r"(b1)
                 : "memory");
  }
  __syncwarp();
  if (threadIdx.x < 32) {
    for (int k = (int)threadIdx.x; k < n1 + n0; k += 32) {
      // planes in the order chunk 0 (class 1, class 0), chunk 1 (class 1, class 0)
      int c, dz, chunk;
      if (k < c1a) { c = 1; dz = k - 2; chunk = 0; }
      else if (k < c1a + c0a) { c = 0; dz = k - c1a - 1; chunk = 0; }
      else if (k < n1 + c0a) { c = 1; dz = k - c0a - 2; chunk = 1; }
      else { c = 0; dz = k - n1 - 1; chunk = 1; }
      Copy cp[3];
      const int m = plane_copies(a, t, c, c ? -2 : -1, c ? 2 : 1, dz, cp);
      uint8_t* sm = c ? s1 : s0;
      for (int j = 0; j < m; ++j)
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                smem_addr(sm + cp[j].soff)),
            "l"(a.in[c] + cp[j].goff), "r"(cp[j].bytes), "r"(smem_addr(mbar + chunk))
            : "memory");
    }
  }
}

// Wait for phase 0 of the mbarrier with a bound; false if it ran out.
__device__ __forceinline__ bool wait_staged(uint64_t* mbar) {
  const uint32_t addr = smem_addr(mbar);
  for (unsigned it = 0; it < kWaitTries; ++it) {
    uint32_t done = 0;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(addr)
        : "memory");
    if (done) return true;
  }
  return false;
}

// Write the tile's own rows of class c back (one bulk copy per z plane:
// its rows y0 .. y0 + TY - 1 do not wrap).  Every thread fenced its shared
// writes for the async proxy before the barrier that precedes this.
__device__ __forceinline__ void store_tile(const IsingTileArgs& a, const TileGeom& t, int c, const uint8_t* sm) {
  if (threadIdx.x < 32) {
    for (int dz = (int)threadIdx.x; dz < t.TZ; dz += 32) {
      const uint32_t goff = ((uint32_t)(t.z0 + dz) * (uint32_t)a.Ly + (uint32_t)t.y0) * (uint32_t)a.Hx;
      const uint32_t soff = c ? row1(a, 0, dz) : row0(a, 0, dz);
      asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;\n" ::"l"(a.out[c] + goff),
                   "r"(smem_addr(sm + soff)), "r"((uint32_t)a.TY * (uint32_t)a.Hx)
                   : "memory");
    }
    asm volatile("cp.async.bulk.commit_group;\n" ::: "memory");
  }
}

// One colour pass over the box rows [lo, TY + hi) x [lo, TZ + hi) of class C
// (own rows in `own`, neighbour rows in `oth`, both in shared memory); a
// thread takes groups q and q + G/2 of one row per item (so that the lanes of
// a warp read consecutive 16-byte words: no bank conflicts).  Measures the
// tile's own rows.  Decisions as the pair kernel (vg_ising.cu): uniform
// coordination 6, byte-parallel first digit, ties queued per warp.  For
// colour 0, the first round of items waits for the first staging chunk only
// (*staged_all is the wait for both, done once before the second round).
template <int C, bool MEASURE, int PROP>
__device__ __forceinline__ void tile_pass(const IsingTileArgs& a, const TileGeom& t, int lo, int hi,
                                          const FastDiv& fny, uint8_t* own, const uint8_t* oth, const IsingTable& tab,
                                          const RngKey& key, const unsigned long long* s_thr,
                                          uint2 (*s_q)[kTileQueue], uint64_t* mbar, int& bond, int& ups,
                                          int& nacc) {
  constexpr int Z = 6;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int ny = a.TY + hi - lo, nz = t.TZ + hi - lo;
  const uint32_t G2 = (uint32_t)(a.G >> 1);
  const uint32_t items = (uint32_t)(ny * nz) * G2;
  int qn = 0;  // warp-uniform queue length

  // decide the first n queued ties (one per lane), then drop them
  auto drain = [&](int n) {
    __syncwarp();
    if (lane < n) {
      const uint2 e = s_q[warp][lane];
      const int k = (int)(e.y & 15u);
      const uint32_t s01 = (e.y >> 4) & 1u, nu = (e.y >> 5) & 7u, inner = (e.y >> 8) & 1u;
      if (resolve_tie(e.x, k, s01, nu, Z, C, s_thr, key)) {
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
  for (uint32_t base = threadIdx.x & ~31u; base < items; base += blockDim.x) {
    if (C == 0 && base >= blockDim.x && base < 2u * blockDim.x) wait_staged(mbar + 1);  // the second chunk
    const uint32_t i = base + (uint32_t)lane;
    uint32_t tm = 0, sgrp = 0, gid0 = 0;  // tied sites: bit k -> group gid0 + (k >> 4) * G/2, site k & 15
    bool inner = false;
    uint32_t S[8], A[8];
#pragma unroll
    for (int w = 0; w < 8; ++w) S[w] = A[w] = 0u;
    if (i < items) {
      const uint32_t r = fdiv(i, a.fG2), q = i - r * G2;
      const int bz = (int)fdiv(r, fny), by = (int)r - bz * ny;
      const int dy = by + lo, dz = bz + lo;
      inner = dy >= 0 && dy < a.TY && dz >= 0 && dz < t.TZ;
      const int gy = wrap(t.y0 + dy, a.Ly), gz = wrap(t.z0 + dz, a.Lz);
      const int p = (gy + gz + C) & 1;  // x parity of this row's class-C sites
      gid0 = ((uint32_t)gz * (uint32_t)a.Ly + (uint32_t)gy) * (uint32_t)a.G + q;
      const uint32_t ha = 16u * q, hb = ha + 8u * (uint32_t)a.G;  // the pair: groups q and q + G/2
      const uint32_t ro = C ? row1(a, dy, dz) : row0(a, dy, dz);
      sgrp = (ro + ha) >> 4;
      const uint32_t ystep = (uint32_t)a.Hx, zstep = (uint32_t)((C ? a.TY + 2 : a.TY + 4) * a.Hx);
      const uint32_t rx = C ? row0(a, dy, dz) : row1(a, dy, dz);  // the other class, same row
      const uint4 Sa = *reinterpret_cast<const uint4*>(own + ro + ha);
      const uint4 Sb = *reinterpret_cast<const uint4*>(own + ro + hb);
      const uint4 Xa = *reinterpret_cast<const uint4*>(oth + rx + ha);
      const uint4 Xb = *reinterpret_cast<const uint4*>(oth + rx + hb);
      // the x neighbours outside each group's 16 bytes: byte h - 1 (p = 0) or h + 16 (p = 1), cyclic in the row
      const uint32_t Hx = (uint32_t)a.Hx;
      const uint32_t ea = p == 0 ? oth[rx + (ha == 0 ? Hx - 1u : ha - 1u)] : oth[rx + ha + 16u];
      const uint32_t eb = p == 0 ? oth[rx + hb - 1u] : oth[rx + (hb + 16u == Hx ? 0u : hb + 16u)];
      const uint32_t X0[8] = {Xa.x, Xa.y, Xa.z, Xa.w, Xb.x, Xb.y, Xb.z, Xb.w};
      uint32_t X1[8];
      if (p == 0) {
        X1[0] = __byte_perm(ea << 24, X0[0], 0x6543);
        X1[4] = __byte_perm(eb << 24, X0[4], 0x6543);
#pragma unroll
        for (int w = 1; w < 4; ++w) {
          X1[w] = __byte_perm(X0[w - 1], X0[w], 0x6543);
          X1[w + 4] = __byte_perm(X0[w + 3], X0[w + 4], 0x6543);
        }
      } else {
#pragma unroll
        for (int w = 0; w < 3; ++w) {
          X1[w] = __byte_perm(X0[w], X0[w + 1], 0x4321);
          X1[w + 4] = __byte_perm(X0[w + 4], X0[w + 5], 0x4321);
        }
        X1[3] = __byte_perm(X0[3], ea, 0x4321);
        X1[7] = __byte_perm(X0[7], eb, 0x4321);
      }
      auto ld2 = [&](uint32_t off, uint32_t (&v)[8]) {
        const uint4 u0 = *reinterpret_cast<const uint4*>(oth + off + ha);
        const uint4 u1 = *reinterpret_cast<const uint4*>(oth + off + hb);
        v[0] = u0.x; v[1] = u0.y; v[2] = u0.z; v[3] = u0.w;
        v[4] = u1.x; v[5] = u1.y; v[6] = u1.z; v[7] = u1.w;
      };
      uint32_t Ym[8], Yp[8], Zm[8], Zp[8];
      ld2(rx - ystep, Ym);
      ld2(rx + ystep, Yp);
      ld2(rx - zstep, Zm);
      ld2(rx + zstep, Zp);
      S[0] = Sa.x; S[1] = Sa.y; S[2] = Sa.z; S[3] = Sa.w;
      S[4] = Sb.x; S[5] = Sb.y; S[6] = Sb.z; S[7] = Sb.w;
#pragma unroll
      for (int w = 0; w < 8; ++w) A[w] = X0[w] + X1[w] + Ym[w] + Yp[w] + Zm[w] + Zp[w];

      uint32_t F[8];
#pragma unroll
      for (int g = 0; g < 2; ++g) {
        const uint32_t gid = gid0 + (uint32_t)g * G2;
        uint32_t cand[4] = {0x01010101u, 0x01010101u, 0x01010101u, 0x01010101u};
        if (PROP == VG_PROPOSE_RANDOM) {
          const uint4 b = philox_ks(
              make_uint4(gid, key.sweep, (kTagIsingPropose << 24) | ((uint32_t)C << 8), key.replica), key.ks);
          const uint32_t w4[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
          for (int j = 0; j < 4; ++j) cand[j] = ((~w4[j] >> 7) & 0x01010101u) ^ S[4 * g + j];
        }
        const uint4 b = philox_ks(
            make_uint4(gid, key.sweep, (kTagIsingAccept << 24) | ((uint32_t)C << 8), key.replica), key.ks);
        const uint32_t R[4] = {b.x, b.y, b.z, b.w};
        uint32_t thr[4], anytie = 0;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int w = 4 * g + j;
          const uint32_t sel = nibble_selector(A[w]);
          const uint32_t sm = S[w] * 0xFFu;
          thr[j] = (__byte_perm(tab.top[1][0], tab.top[1][1], sel) & sm) |
                   (__byte_perm(tab.top[0][0], tab.top[0][1], sel) & ~sm);
          F[w] = (bytes_gt80(thr[j], R[j]) >> 7) & cand[j];
          const uint32_t x = R[j] ^ thr[j];
          anytie |= (x - 0x01010101u) & ~x & 0x80808080u;  // nonzero iff some byte of x is zero
        }
        if (anytie) {
#pragma unroll
          for (int j = 0; j < 4; ++j) tm |= gather4(bytes_zero(R[j] ^ thr[j]) & cand[j]) << (16 * g + 4 * j);
        }
      }
      uint32_t Sn[8], anyf = 0;
#pragma unroll
      for (int w = 0; w < 8; ++w) {
        Sn[w] = S[w] ^ F[w];
        anyf |= F[w];
      }
      if (anyf) {
        *reinterpret_cast<uint4*>(own + ro + ha) = make_uint4(Sn[0], Sn[1], Sn[2], Sn[3]);
        *reinterpret_cast<uint4*>(own + ro + hb) = make_uint4(Sn[4], Sn[5], Sn[6], Sn[7]);
      }
      if (MEASURE && inner) {
        unsigned su = 0, sf = 0;
#pragma unroll
        for (int w = 0; w < 8; ++w) {
          su = __dp4a(Sn[w], 0x01010101u, su);
          sf = __dp4a(F[w], 0x01010101u, sf);
        }
        ups += (int)su;
        nacc += (int)sf;
        if (C == 1) {  // every neighbour of class 1 has the lower colour: all bonds counted here
          unsigned sm = 0, m = 0;
#pragma unroll
          for (int w = 0; w < 8; ++w) {
            const uint32_t M = 2u * A[w];  // neighbour sum + Z per byte (all six neighbours exist)
            sm = __dp4a(Sn[w], M, sm);
            m = __dp4a(M, 0x01010101u, m);
          }
          bond += 2 * (int)sm - (int)m - Z * (2 * (int)su - 32);
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
        const int wi = k >> 2;
        uint32_t sw = 0, aw = 0;  // S[wi], A[wi] by selects: a dynamic index would put S, A on the stack
#pragma unroll
        for (int w = 0; w < 8; ++w) {
          sw = w == wi ? S[w] : sw;
          aw = w == wi ? A[w] : aw;
        }
        const uint32_t sk = (sw >> (8 * (k & 3))) & 0xFFu;
        const uint32_t nk = (aw >> (8 * (k & 3))) & 0xFFu;
        const uint32_t half = (uint32_t)(k >> 4) * G2;  // the pair's second group lies G/2 groups on
        s_q[warp][pos] = make_uint2(gid0 + half, (uint32_t)(k & 15) | (sk << 4) | (nk << 5) |
                                                     ((uint32_t)inner << 8) | ((sgrp + half) << 9));
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
  extern __shared__ __align__(128) uint8_t s_spin[];  // class-1 box, then class-0 box
  __shared__ unsigned long long s_thr[2 * 13];
  __shared__ uint2 s_q[kTileThreads / 32][kTileQueue];
  __shared__ __align__(8) uint64_t s_mbar[2];  // the two staging chunks
  __shared__ int s_ok;
  uint8_t* s1 = s_spin;
  uint8_t* s0 = s_spin + (size_t)(a.TZm + 4) * (a.TY + 4) * a.Hx;
  pdl_launch_dependents();
  for (int i = threadIdx.x; i < 2 * 13; i += blockDim.x) s_thr[i] = tab.thr[i];
  const TileGeom t = tile_of(a);
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_addr(&s_mbar[0])) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_addr(&s_mbar[1])) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  __syncthreads();
  pdl_wait();  // the previous sweep's writes (and its reads of our output buffer) are complete
  stage_boxes(a, t, s1, s0, s_mbar);
  // the first chunk, then (inside the colour-0 pass, before its second round
  // of items) the second; thread 0 checks both with a bound before the pass
  // results are used
  bool staged = wait_staged(&s_mbar[0]);
  if (threadIdx.x == 0) s_ok = staged ? 1 : 0;
  __syncthreads();
  if (!s_ok) {  // a staging wait ran out (never expected): report it, write nothing, and give the
                // copies still in flight a second bounded wait before the block's shared memory goes
    if (threadIdx.x == 0) {
      atomicExch(a.err, 1);
      wait_staged(&s_mbar[0]);
      wait_staged(&s_mbar[1]);
    }
    return;
  }
  int bond = 0, ups = 0, nacc = 0;
  tile_pass<0, MEASURE, PROP>(a, t, -1, 1, a.fny0, s0, s1, tab, key, s_thr, s_q, s_mbar, bond, ups, nacc);
  staged = wait_staged(&s_mbar[1]);  // already complete unless the pass had a single round
  if (threadIdx.x == 0) s_ok = staged ? 1 : 0;
  __syncthreads();
  if (!s_ok) {
    if (threadIdx.x == 0) {
      atomicExch(a.err, 1);
      wait_staged(&s_mbar[1]);
    }
    return;
  }
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");  // class 0 for the bulk store
  __syncthreads();
  store_tile(a, t, 0, s0);  // class 0 is final: its store overlaps the class-1 pass
  tile_pass<1, MEASURE, PROP>(a, t, 0, 0, a.fny, s1, s0, tab, key, s_thr, s_q, s_mbar, bond, ups, nacc);
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
  __syncthreads();
  store_tile(a, t, 1, s1);
  if (MEASURE) block_sum3_store(bond, ups, nacc, part + (size_t)blockIdx.x * kNumSums);
  if (threadIdx.x < 32) asm volatile("cp.async.bulk.wait_group 0;\n" ::: "memory");  // both stores complete
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

size_t ising_tile_smem(int Hx, int TY, int TZm) {
  return (size_t)((TZm + 4) * (TY + 4) + (TZm + 2) * (TY + 2)) * (size_t)Hx;
}

// The tiling of a lattice's y-z plane of rows: y in nyt equal tiles (nyt
// divides Ly), z in nzt nearly equal ones (extents differ by at most one);
// one block per tile, as few waves of one block per SM as shared memory
// allows, then the fewest rounds of pair items per wave (colour 0 on the
// grown box, colour 1 on the tile) plus the staged and stored rows.  Rows
// must hold an even number of groups.  Returns false when no tiling fits.
bool ising_tile_plan(int Hx, int Ly, int Lz, int sm_count, IsingTileArgs* a) {
  const int G = Hx / kIsingGroup;
  if (G < 2 || G % 2) return false;
  double best = 1e300;
  bool found = false;
  for (int nyt = 1; nyt <= Ly; ++nyt) {
    if (Ly % nyt) continue;
    const int TY = Ly / nyt;
    for (int nzt = 1; nzt <= Lz; ++nzt) {
      const int TZm = (Lz + nzt - 1) / nzt;
      if (ising_tile_smem(Hx, TY, TZm) > kTileSmemMax) continue;
      const long long tiles = (long long)nyt * nzt;
      const long long waves = (tiles + sm_count - 1) / sm_count;
      const long long p0 = (long long)(TY + 2) * (TZm + 2) * (G / 2), p1 = (long long)TY * TZm * (G / 2);
      const double rounds = (double)((p0 + kTileThreads - 1) / kTileThreads + (p1 + kTileThreads - 1) / kTileThreads);
      // staged and stored rows, in units of a round of pair items
      const double copies = 0.05 * ((TY + 4) * (TZm + 4) + (TY + 2) * (TZm + 2) + 2.0 * TY * TZm) * G / kTileThreads;
      const double cost = (double)waves * (rounds + copies + 0.5);
      if (cost < best) {
        best = cost;
        found = true;
        a->nyt = nyt;
        a->nzt = nzt;
        a->TY = TY;
        a->TZm = TZm;
      }
    }
  }
  if (found) {
    a->fny0 = make_fastdiv((uint32_t)(a->TY + 2));
    a->fny = make_fastdiv((uint32_t)a->TY);
    a->fG2 = make_fastdiv((uint32_t)(G / 2));
  }
  return found;
}

cudaError_t launch_ising_tile_sweep(const IsingTileArgs& a, const IsingTable& tab, RngKey key, int proposal,
                                    long long* part, cudaStream_t s) {
  const size_t smem = ising_tile_smem(a.Hx, a.TY, a.TZm);
  if (proposal == VG_PROPOSE_FLIP)
    return part ? tile_launch<true, VG_PROPOSE_FLIP>(a, tab, key, part, smem, s)
                : tile_launch<false, VG_PROPOSE_FLIP>(a, tab, key, part, smem, s);
  return part ? tile_launch<true, VG_PROPOSE_RANDOM>(a, tab, key, part, smem, s)
              : tile_launch<false, VG_PROPOSE_RANDOM>(a, tab, key, part, smem, s);
}

}  // namespace vg
