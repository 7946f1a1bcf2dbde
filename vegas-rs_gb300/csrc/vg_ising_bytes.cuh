// vg_ising_bytes.cuh -- byte-parallel helpers of the Ising checkerboard
// kernels (a 32-bit word carries four sites, one 0/1 byte each), the block
// sum of the per-pass Ising partials and the resolution of first-digit ties.
// Shared by the per-pass kernels (vg_ising.cu) and the tiled sweep kernel
// (vg_tiled.cu), which must decide every site identically.
#pragma once

#include "vg_internal.cuh"

namespace vg {

// 4 bits -> 4 bytes of 0/1 and back.
__device__ __forceinline__ uint32_t spread4(uint32_t m) { return ((m & 0xFu) * 0x00204081u) & 0x01010101u; }
__device__ __forceinline__ uint32_t gather4(uint32_t x) { return (((x & 0x01010101u) * 0x01020408u) >> 24) & 0xFu; }

// ------------------------------------------------------------------ sc
// Byte-parallel helpers: a 32-bit word carries 4 sites, one byte each.
// PRMT selector from 4 bytes in [0, 7].
__device__ __forceinline__ uint32_t nibble_selector(uint32_t a) {
  const uint32_t y = (a | (a >> 4)) & 0x00770077u;
  return (y | (y >> 8)) & 0x7777u;
}
// 0x80 in each byte where t > r (unsigned): the carry out of each byte of
// t + ~r (= 255 + t - r), a majority of bit 7 of t, bit 7 of ~r and the
// carry into bit 7 (bit 7 of the 7-bit partial sums, which cannot overflow
// into the next byte).
__device__ __forceinline__ uint32_t bytes_gt80(uint32_t t, uint32_t r) {
  const uint32_t nr = ~r;
  const uint32_t s = (t & 0x7F7F7F7Fu) + (nr & 0x7F7F7F7Fu);
  return ((t & nr) | ((t | nr) & s)) & 0x80808080u;
}
// 0x01 in each byte of x that is zero
__device__ __forceinline__ uint32_t bytes_zero(uint32_t x) {
  const uint32_t t = (x & 0x7F7F7F7Fu) + 0x7F7F7F7Fu;
  return (~(t | x) >> 7) & 0x01010101u;
}
__device__ __forceinline__ uint32_t byte_at(uint32_t w0, uint32_t w1, uint32_t w2, uint32_t w3, int k) {
  const uint32_t lo = (k & 4) ? w1 : w0, hi = (k & 4) ? w3 : w2;
  return (((k & 8) ? hi : lo) >> (8 * (k & 3))) & 0xFFu;
}

// Block sum of the three live Ising partials (bond, up spins, accepted) into
// one kNumSums row.
__device__ __forceinline__ void block_sum3_store(int a, int b, int c, long long* out) {
  __shared__ int red[3][32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  a = __reduce_add_sync(0xffffffffu, a);
  b = __reduce_add_sync(0xffffffffu, b);
  c = __reduce_add_sync(0xffffffffu, c);
  if (lane == 0) {
    red[0][warp] = a;
    red[1][warp] = b;
    red[2][warp] = c;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    long long sa = 0, sb = 0, sc = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      sa += red[0][w];
      sb += red[1][w];
      sc += red[2][w];
    }
    out[0] = sa;
    out[1] = out[2] = out[3] = out[4] = out[5] = 0;
    out[6] = sb;
    out[7] = sc;
  }
}

// Resolution of ties deferred to whole warps: a queued site (group gid,
// site k, spin s, up-neighbour count nu) tied with its threshold on digit 0;
// digits 1..3 decide it exactly as the in-line rule would.  Returns whether
// the move is accepted.
__device__ __forceinline__ bool resolve_tie(uint32_t gid, int k, uint32_t s01, uint32_t nu, int zeff, int colour,
                                            const unsigned long long* s_thr, const RngKey& key) {
  constexpr int Z = 6, W = 2 * Z + 1;
  const unsigned long long th = s_thr[s01 * W + 2 * nu - zeff + Z];
  if (th >= (1ull << 32)) return true;
  for (int d = 1; d < 4; ++d) {
    const uint4 bd = philox_ks(
        make_uint4(gid, key.sweep, (kTagIsingAccept << 24) | ((uint32_t)colour << 8) | (uint32_t)d, key.replica),
        key.ks);
    const uint32_t ub = byte_at(bd.x, bd.y, bd.z, bd.w, k);
    const uint32_t tb = ((uint32_t)th >> (24 - 8 * d)) & 0xFFu;
    if (ub != tb) return ub < tb;
  }
  return false;  // U == thr: not below the threshold
}

}  // namespace vg
