// vg_ising.cu -- Ising colour-class Metropolis passes.
//
// Replaces MetropolisFlipIntegrator::step / MetropolisIntegrator::step for
// IsingSpin (src/integrator.rs:66-137) with the reference's accept rule:
// dE < 0 accepts; otherwise accept iff u < exp(-dE/T).  dE is an integer
// function of (s, sum of neighbour spins), so the rule is a table of 32-bit
// thresholds built on the host in FP64 (accept iff U < thr for the site's
// 32-bit uniform U).  U is drawn byte-serially: byte (j & 15) of Philox
// block d = 0..3 of the 16-site group j >> 4 is digit d (most significant
// first), and a later block is generated only while some site of the group
// still ties with its threshold -- usually one block per 16 sites.
//
// Two kernel families, identical results:
//  * ising_sc_kernel: sc lattice in a checkerboard, class-separated layout
//    (class c holds sites with (x+y+z)&1 == c, row-major [z][y][x/2]); one
//    thread owns 16 consecutive sites of a row as one uint4 of 0/1 bytes and
//    adds its six neighbour vectors with plain 32-bit adds (bytes <= 6).
//  * ising_gen_kernel: any lattice via an ELL neighbour table per colour
//    class of a greedy colouring (natural-order spins).
#include <utility>

#include "vg_ising_bytes.cuh"

namespace vg {

// Decide 16 candidate sites given their 64-bit thresholds; returns the
// accepted mask.  Site k of group g uses byte k of the group's blocks.
__device__ __forceinline__ uint32_t decide16(const unsigned long long (&t)[16], uint32_t cand,
                                             const RngKey& key, uint32_t g, int colour) {
  uint32_t thr32[16];
  uint32_t acc = 0, und = 0;
#pragma unroll
  for (int k = 0; k < 16; ++k) {
    thr32[k] = (uint32_t)t[k];
    const bool c = (cand >> k) & 1u;
    if (c && t[k] >= (1ull << 32)) acc |= 1u << k;
    if (c && t[k] > 0ull && t[k] < (1ull << 32)) und |= 1u << k;
  }
#pragma unroll 1
  for (int d = 0; d < 4 && und; ++d) {
    const uint4 b = philox_ks(make_uint4(g, key.sweep, (kTagIsingAccept << 24) | ((uint32_t)colour << 8) | (uint32_t)d,
                                         key.replica),
                              key.ks);
    const uint32_t w[4] = {b.x, b.y, b.z, b.w};
    const int sh = 24 - 8 * d;
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      const uint32_t bit = 1u << k;
      const uint32_t ub = (w[k >> 2] >> (8 * (k & 3))) & 0xFFu;
      const uint32_t tb = (thr32[k] >> sh) & 0xFFu;
      if (und & bit) {
        if (ub < tb) {
          acc |= bit;
          und &= ~bit;
        } else if (ub > tb) {
          und &= ~bit;
        }
      }
    }
  }
  return acc;
}

// UNIFORM: every site has the same number zeff of existing neighbours (each
// axis periodic, or open with extent 1), so the up-neighbour count n_up in
// [0, zeff] indexes 8-entry byte tables and four sites are decided per
// word: the threshold's top byte comes from a PRMT lookup (0xFF for moves
// that always accept), the first random digit is compared byte-parallel, and
// sites whose digit ties with the threshold digit (probability 1/256) are
// queued per warp and resolved 32 at a time.  Otherwise the scalar
// decide16 path runs in line.  Both give the decisions of "accept iff U < thr".
constexpr int kScQueue = 64;  // per-warp tie queue

// The 16-site groups base + lane for base in [first, end) step `step` (base
// a multiple of 32 apart from `first`), adding the pass's sums to bond / ups
// / nacc.  Every tie is resolved before returning.
template <int C, bool UNIFORM, bool MEASURE, bool UPDATE, int PROP>
__device__ __forceinline__ void sc1_range(const IsingScArgs& a, const IsingTable& tab, const RngKey& key,
                                          const unsigned long long* s_thr, uint2 (*s_q)[kScQueue], uint32_t first,
                                          uint32_t end, uint32_t step, int& bond, int& ups, int& nacc) {
  constexpr int Z = 6, W = 2 * Z + 1;
  constexpr int kQ = kScQueue;
  uint8_t* __restrict__ own = a.cls[C];
  const uint8_t* __restrict__ oth = a.cls[C ^ 1];
  const int zoff = Z - tab.zeff;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int qn = 0;  // warp-uniform queue length

  // apply the first n queued ties (one per lane), then drop them
  auto drain = [&](int n) {
    __syncwarp();
    if (lane < n) {
      const uint2 e = s_q[warp][lane];
      const int k = (int)(e.y & 15u);
      const uint32_t s01 = (e.y >> 4) & 1u, nu = e.y >> 5;
      if (resolve_tie(e.x, k, s01, nu, tab.zeff, C, s_thr, key)) {
        own[(size_t)e.x * 16 + k] = (uint8_t)(s01 ^ 1u);
        ups += 1 - 2 * (int)s01;
        nacc += 1;
        if (C == 1) bond -= 2 * (2 * (int)s01 - 1) * (2 * (int)nu - tab.zeff);
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

  for (uint32_t base = first; base < end; base += step) {
    const uint32_t gid = base + lane;
    const bool active = gid < end;
    uint32_t tm = 0;  // sites of this group whose first digit tied
    uint32_t S[4] = {0, 0, 0, 0}, A[4] = {0, 0, 0, 0};
    if (active) {
      const int row = (int)fdiv(gid, a.fG);
      const int h0 = (int)(gid - (uint32_t)row * a.G) << 4;
      const int z = (int)fdiv((uint32_t)row, a.fLy);
      const int y = row - z * a.Ly;
      const int p = (y + z + C) & 1;  // x parity of this row's class-C sites
      const int rb = row * a.Hx;

      const uint4 Sv = *reinterpret_cast<const uint4*>(own + rb + h0);
      const uint4 X0 = __ldg(reinterpret_cast<const uint4*>(oth + rb + h0));
      // x-neighbour not shared with X0: h0-1 (p = 0) or h0+16 (p = 1)
      uint32_t e = 0;
      bool xmiss = false;
      if (p == 0) {
        if (h0 > 0) e = __ldg(oth + rb + h0 - 1);
        else if (a.pbx) e = __ldg(oth + rb + a.Hx - 1);
        else xmiss = true;
      } else {
        if (h0 + 16 < a.Hx) e = __ldg(oth + rb + h0 + 16);
        else if (a.pbx) e = __ldg(oth + rb);
        else xmiss = true;
      }
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
      const int rym = y > 0 ? row - 1 : (a.pby ? row + a.Ly - 1 : -1);
      const int ryp = y < a.Ly - 1 ? row + 1 : (a.pby ? row - (a.Ly - 1) : -1);
      const int rzm = z > 0 ? row - a.Ly : (a.pbz ? row + (a.Lz - 1) * a.Ly : -1);
      const int rzp = z < a.Lz - 1 ? row + a.Ly : (a.pbz ? row - (a.Lz - 1) * a.Ly : -1);
      const uint4 zero4 = make_uint4(0, 0, 0, 0);
      const uint4 Ym = rym >= 0 ? __ldg(reinterpret_cast<const uint4*>(oth + (uint32_t)rym * (uint32_t)a.Hx + h0)) : zero4;
      const uint4 Yp = ryp >= 0 ? __ldg(reinterpret_cast<const uint4*>(oth + (uint32_t)ryp * (uint32_t)a.Hx + h0)) : zero4;
      const uint4 Zm = rzm >= 0 ? __ldg(reinterpret_cast<const uint4*>(oth + (uint32_t)rzm * (uint32_t)a.Hx + h0)) : zero4;
      const uint4 Zp = rzp >= 0 ? __ldg(reinterpret_cast<const uint4*>(oth + (uint32_t)rzp * (uint32_t)a.Hx + h0)) : zero4;

      S[0] = Sv.x;
      S[1] = Sv.y;
      S[2] = Sv.z;
      S[3] = Sv.w;
      A[0] = X0.x + X1[0] + Ym.x + Yp.x + Zm.x + Zp.x;
      A[1] = X0.y + X1[1] + Ym.y + Yp.y + Zm.y + Zp.y;
      A[2] = X0.z + X1[2] + Ym.z + Yp.z + Zm.z + Zp.z;
      A[3] = X0.w + X1[3] + Ym.w + Yp.w + Zm.w + Zp.w;
      // M = 2A + (Z - Zc) per byte, where Zc counts existing neighbours; the
      // neighbour sum of site k is M_k - Z.
      uint32_t M[4];
      if (UNIFORM) {
#pragma unroll
        for (int i = 0; i < 4; ++i) M[i] = 2u * A[i] + (uint32_t)zoff * 0x01010101u;
      } else {
        const uint32_t zmiss = (uint32_t)((rym < 0) + (ryp < 0) + (rzm < 0) + (rzp < 0));
#pragma unroll
        for (int i = 0; i < 4; ++i) M[i] = 2u * A[i] + zmiss * 0x01010101u;
        if (xmiss) {
          if (p == 0) M[0] += 1u;
          else M[3] += 1u << 24;
        }
      }

      uint32_t F[4] = {0, 0, 0, 0};  // 0x01 bytes: sites that flip
      if (UPDATE) {
        uint32_t cand[4] = {0x01010101u, 0x01010101u, 0x01010101u, 0x01010101u};
        if (PROP == VG_PROPOSE_RANDOM) {
          const uint4 b = philox_ks(make_uint4(gid, key.sweep, (kTagIsingPropose << 24) | ((uint32_t)C << 8), key.replica),
                                    key.ks);
          const uint32_t w[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
          for (int i = 0; i < 4; ++i) cand[i] = ((~w[i] >> 7) & 0x01010101u) ^ S[i];
        }
        if (UNIFORM) {
          const uint4 b = philox_ks(make_uint4(gid, key.sweep, (kTagIsingAccept << 24) | ((uint32_t)C << 8), key.replica),
                                    key.ks);
          const uint32_t R[4] = {b.x, b.y, b.z, b.w};
          uint32_t thr[4], anytie = 0;
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const uint32_t sel = nibble_selector(A[i]);
            const uint32_t sm = S[i] * 0xFFu;
            thr[i] = (__byte_perm(tab.top[1][0], tab.top[1][1], sel) & sm) |
                     (__byte_perm(tab.top[0][0], tab.top[0][1], sel) & ~sm);
            F[i] = (bytes_gt80(thr[i], R[i]) >> 7) & cand[i];
            const uint32_t x = R[i] ^ thr[i];
            anytie |= (x - 0x01010101u) & ~x & 0x80808080u;  // nonzero iff some byte of x is zero
          }
          if (anytie) {
#pragma unroll
            for (int i = 0; i < 4; ++i) tm |= gather4(bytes_zero(R[i] ^ thr[i]) & cand[i]) << (4 * i);
          }
        } else {
          uint32_t cm = 0;
#pragma unroll
          for (int i = 0; i < 4; ++i) cm |= gather4(cand[i]) << (4 * i);
          unsigned long long t[16];
#pragma unroll
          for (int k = 0; k < 16; ++k) {
            const uint32_t idx = ((S[k >> 2] * (uint32_t)W + M[k >> 2]) >> (8 * (k & 3))) & 0xFFu;
            t[k] = s_thr[idx];
          }
          const uint32_t flip = decide16(t, cm, key, gid, C) & cm;
#pragma unroll
          for (int i = 0; i < 4; ++i) F[i] = spread4(flip >> (4 * i));
        }
      }
      uint32_t Sn[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) Sn[i] = S[i] ^ F[i];
      if ((F[0] | F[1] | F[2] | F[3]) != 0u)
        *reinterpret_cast<uint4*>(own + rb + h0) = make_uint4(Sn[0], Sn[1], Sn[2], Sn[3]);

      if (MEASURE) {
        int u = 0, f = 0;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          u += __popc(Sn[i]);
          f += __popc(F[i]);
        }
        ups += u;
        nacc += f;
        if (C == 1) {  // every neighbour of class 1 has the lower colour: all bonds counted here
          unsigned sm = 0, m = 0;
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            sm = __dp4a(Sn[i], M[i], sm);
            m = __dp4a(M[i], 0x01010101u, m);
          }
          bond += 2 * (int)sm - (int)m - Z * (2 * u - 16);
        }
      }
    }
    if (UNIFORM && UPDATE) {
      // queue this iteration's ties, one site per lane per round
      unsigned lanes = __ballot_sync(0xffffffffu, tm != 0u);
      while (lanes) {
        if (qn + 32 > kQ) drain(32 < qn ? 32 : qn);
        const int pos = qn + __popc(lanes & ((1u << lane) - 1u));
        if (tm) {
          const int k = __ffs(tm) - 1;
          tm &= tm - 1u;
          const uint32_t sk = byte_at(S[0], S[1], S[2], S[3], k);
          const uint32_t nk = byte_at(A[0], A[1], A[2], A[3], k);
          s_q[warp][pos] = make_uint2(gid, (uint32_t)k | (sk << 4) | (nk << 5));
        }
        qn += __popc(lanes);
        if (qn >= 32) drain(32);
        lanes = __ballot_sync(0xffffffffu, tm != 0u);
      }
    }
  }
  if (UNIFORM && UPDATE && qn > 0) drain(qn);
}

template <int C, bool UNIFORM, bool MEASURE, bool UPDATE, int PROP>
__global__ void __launch_bounds__(256, UNIFORM ? 4 : 2) ising_sc_kernel(const IsingScArgs a, const IsingTable tab, const RngKey key,
                                                          long long* __restrict__ part) {
  constexpr int W = 13;
  __shared__ unsigned long long s_thr[2 * W];
  __shared__ uint2 s_q[8][kScQueue];
  pdl_launch_dependents();
  for (int i = threadIdx.x; i < 2 * W; i += blockDim.x) s_thr[i] = tab.thr[i];
  __syncthreads();
  pdl_wait();
  int bond = 0, ups = 0, nacc = 0;
  sc1_range<C, UNIFORM, MEASURE, UPDATE, PROP>(a, tab, key, s_thr, s_q, blockIdx.x * blockDim.x + (threadIdx.x & ~31u),
                                               a.groups, gridDim.x * blockDim.x, bond, ups, nacc);
  if (MEASURE) block_sum3_store(bond, ups, nacc, part + (size_t)blockIdx.x * kNumSums);
}

// Two 16-site groups per thread (32 consecutive class sites of a row; rows
// hold an even number of groups), uniform coordination only.  Index
// arithmetic, neighbour rows and the x-edge byte are shared by the pair;
// every group draws and decides exactly as in ising_sc_kernel (same Philox
// blocks, same tie resolution), so results are identical.  ALLPER: all axes
// periodic, no missing rows.
// 80 registers: the pair state stays in registers (four blocks per SM at 64
// registers spilled ~100 bytes a thread and ran 256^3 at 708 flips/ns, 804 so)
constexpr int kSc2MinBlocks = 3;
// Ties on the first digit (1/256 of the candidate sites, so that a warp
// meets one in most rounds of pairs) are queued per block and decided after
// the block's pairs; entries past the queue's end are decided in line.
// Timing builds put tie handling at about 30 % of the pass at 256^3 (one
// that ignored ties ran 1,128 flips/ns against 790), and the work in the
// pair loop, which runs in most rounds whatever the queue, dominates it:
// a per-warp queue, this block queue, deferring whole groups to the end of
// the block, a per-warp ring of tied groups drained 32 at a time, and
// deciding a tied group's ties in line from its second-digit Philox block
// (byte-parallel against the thresholds' second bytes) all ran between 739
// and 802 flips/ns.  The kernel is latency-bound (43 % of issue
// slots used), so serial work on a tie lengthens its warp's path.
constexpr int kSc2BlockQueue = 512;

// S[w] and A[w] byte k & 3 of word w = k >> 2 (bit k of a pair's tie mask),
// by selects: a dynamic index would put S and A on the stack.
__device__ __forceinline__ void pair_site(const uint32_t (&S)[8], const uint32_t (&A)[8], int k, uint32_t& s01,
                                          uint32_t& nu) {
  const int wi = k >> 2;
  uint32_t sw = 0, aw = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    sw = i == wi ? S[i] : sw;
    aw = i == wi ? A[i] : aw;
  }
  s01 = (sw >> (8 * (k & 3))) & 0xFFu;
  nu = (aw >> (8 * (k & 3))) & 0xFFu;
}

// The pairs base + lane for base in [first, end) step `step` (base a
// multiple of 32 apart from `first`), adding the pass's sums to bond / ups /
// nacc.  Ties go to the block queue s_tq / s_tn (decided by sc2_ties after
// the block's pairs, every thread of the block taking part).
template <int C, bool MEASURE, bool UPDATE, int PROP, bool ALLPER>
__device__ __forceinline__ void sc2_range(const IsingScArgs& a, const FastDiv& fG2, const IsingTable& tab,
                                          const RngKey& key, const unsigned long long* s_thr, uint2* s_tq, int* s_tn,
                                          uint32_t first, uint32_t end, uint32_t step, int& bond, int& ups,
                                          int& nacc) {
  constexpr int Z = 6;
  uint8_t* __restrict__ own = a.cls[C];
  const uint8_t* __restrict__ oth = a.cls[C ^ 1];
  const uint32_t zoff = (uint32_t)(Z - tab.zeff) * 0x01010101u;
  const int lane = threadIdx.x & 31;
  const int G2 = a.G >> 1;
  const uint32_t pairs = end;

  for (uint32_t base = first; base < pairs; base += step) {
    const uint32_t q = base + lane;
    const bool active = q < pairs;
    uint32_t tm = 0;  // tied sites: bit k -> group 2q + (k >> 4), site k & 15
    uint32_t S[8], A[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) S[i] = A[i] = 0u;
    if (active) {
      const int row = (int)fdiv(q, fG2);
      const int h0 = (int)(q - (uint32_t)row * (uint32_t)G2) << 5;
      const int z = (int)fdiv((uint32_t)row, a.fLy);
      const int y = row - z * a.Ly;
      const int p = (y + z + C) & 1;
      const uint32_t rb = (uint32_t)row * (uint32_t)a.Hx;  // 32-bit: no wide multiply beside Philox's

      const uint4 Sa = *reinterpret_cast<const uint4*>(own + rb + h0);
      const uint4 Sb = *reinterpret_cast<const uint4*>(own + rb + h0 + 16);
      const uint4 Xa = __ldg(reinterpret_cast<const uint4*>(oth + rb + h0));
      const uint4 Xb = __ldg(reinterpret_cast<const uint4*>(oth + rb + h0 + 16));
      uint32_t e = 0;
      if (p == 0) {
        if (h0 > 0) e = __ldg(oth + rb + h0 - 1);
        else if (ALLPER || a.pbx) e = __ldg(oth + rb + a.Hx - 1);
      } else {
        if (h0 + 32 < a.Hx) e = __ldg(oth + rb + h0 + 32);
        else if (ALLPER || a.pbx) e = __ldg(oth + rb);
      }
      const uint32_t X0[8] = {Xa.x, Xa.y, Xa.z, Xa.w, Xb.x, Xb.y, Xb.z, Xb.w};
      uint32_t X1[8];
      if (p == 0) {
        X1[0] = __byte_perm(e << 24, X0[0], 0x6543);
#pragma unroll
        for (int i = 1; i < 8; ++i) X1[i] = __byte_perm(X0[i - 1], X0[i], 0x6543);
      } else {
#pragma unroll
        for (int i = 0; i < 7; ++i) X1[i] = __byte_perm(X0[i], X0[i + 1], 0x4321);
        X1[7] = __byte_perm(X0[7], e, 0x4321);
      }
      uint32_t oym, oyp, ozm, ozp;  // neighbour row offsets
      bool hym = true, hyp = true, hzm = true, hzp = true;
      oym = y > 0 ? rb - (uint32_t)a.Hx : rb + a.ywrap;
      oyp = y < a.Ly - 1 ? rb + (uint32_t)a.Hx : rb - a.ywrap;
      ozm = z > 0 ? rb - a.plane : rb + a.zwrap;
      ozp = z < a.Lz - 1 ? rb + a.plane : rb - a.zwrap;
      if (!ALLPER) {
        hym = y > 0 || a.pby;
        hyp = y < a.Ly - 1 || a.pby;
        hzm = z > 0 || a.pbz;
        hzp = z < a.Lz - 1 || a.pbz;
      }
      const uint4 zero4 = make_uint4(0, 0, 0, 0);
      auto ld2 = [&](bool has, uint32_t off, uint32_t (&v)[8]) {
        const uint4 u0 = has ? __ldg(reinterpret_cast<const uint4*>(oth + off + h0)) : zero4;
        const uint4 u1 = has ? __ldg(reinterpret_cast<const uint4*>(oth + off + h0 + 16)) : zero4;
        v[0] = u0.x; v[1] = u0.y; v[2] = u0.z; v[3] = u0.w;
        v[4] = u1.x; v[5] = u1.y; v[6] = u1.z; v[7] = u1.w;
      };
      uint32_t Ym[8], Yp[8], Zm[8], Zp[8];
      ld2(hym, oym, Ym);
      ld2(hyp, oyp, Yp);
      ld2(hzm, ozm, Zm);
      ld2(hzp, ozp, Zp);
      S[0] = Sa.x; S[1] = Sa.y; S[2] = Sa.z; S[3] = Sa.w;
      S[4] = Sb.x; S[5] = Sb.y; S[6] = Sb.z; S[7] = Sb.w;
#pragma unroll
      for (int i = 0; i < 8; ++i) A[i] = X0[i] + X1[i] + Ym[i] + Yp[i] + Zm[i] + Zp[i];

      uint32_t F[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) F[i] = 0u;
      if (UPDATE) {
#pragma unroll
        for (int g = 0; g < 2; ++g) {
          const uint32_t gid = 2u * q + (uint32_t)g;
          uint32_t cand[4] = {0x01010101u, 0x01010101u, 0x01010101u, 0x01010101u};
          if (PROP == VG_PROPOSE_RANDOM) {
            const uint4 b = philox_ks(
                make_uint4(gid, key.sweep, (kTagIsingPropose << 24) | ((uint32_t)C << 8), key.replica), key.ks);
            const uint32_t w[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
            for (int i = 0; i < 4; ++i) cand[i] = ((~w[i] >> 7) & 0x01010101u) ^ S[4 * g + i];
          }
          const uint4 b = philox_ks(
              make_uint4(gid, key.sweep, (kTagIsingAccept << 24) | ((uint32_t)C << 8), key.replica), key.ks);
          const uint32_t R[4] = {b.x, b.y, b.z, b.w};
          uint32_t thr[4], anytie = 0;
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const int wi = 4 * g + i;
            const uint32_t sel = nibble_selector(A[wi]);
            const uint32_t sm = S[wi] * 0xFFu;
            thr[i] = (__byte_perm(tab.top[1][0], tab.top[1][1], sel) & sm) |
                     (__byte_perm(tab.top[0][0], tab.top[0][1], sel) & ~sm);
            F[wi] = (bytes_gt80(thr[i], R[i]) >> 7) & cand[i];
            const uint32_t x = R[i] ^ thr[i];
            anytie |= (x - 0x01010101u) & ~x & 0x80808080u;  // nonzero iff some byte of x is zero
          }
          if (anytie) {
#pragma unroll
            for (int i = 0; i < 4; ++i) tm |= gather4(bytes_zero(R[i] ^ thr[i]) & cand[i]) << (16 * g + 4 * i);
          }
        }
        if (tm) {  // sites whose first digit tied with their threshold's: to the block queue
          for (uint32_t m = tm; m; m &= m - 1u) {
            const int k = __ffs(m) - 1;
            const int slot = atomicAdd(s_tn, 1);
            if (slot < kSc2BlockQueue) {
              uint32_t s01, nu;
              pair_site(S, A, k, s01, nu);
              s_tq[slot] = make_uint2(2u * q + (uint32_t)(k >> 4), (uint32_t)(k & 15) | (s01 << 4) | (nu << 5));
              tm &= ~(1u << k);
            }
          }
          for (uint32_t m = tm; m; m &= m - 1u) {  // no room left in the queue: decided here
            const int k = __ffs(m) - 1;
            uint32_t s01, nu;
            pair_site(S, A, k, s01, nu);
            if (resolve_tie(2u * q + (uint32_t)(k >> 4), k & 15, s01, nu, tab.zeff, C, s_thr, key)) {
              const uint32_t bit = 1u << (8 * (k & 3));
#pragma unroll
              for (int i = 0; i < 8; ++i)
                if (i == (k >> 2)) F[i] |= bit;
            }
          }
        }
      }
      uint32_t Sn[8], anyf = 0;
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        Sn[i] = S[i] ^ F[i];
        anyf |= F[i];
      }
      if (anyf) {
        *reinterpret_cast<uint4*>(own + rb + h0) = make_uint4(Sn[0], Sn[1], Sn[2], Sn[3]);
        *reinterpret_cast<uint4*>(own + rb + h0 + 16) = make_uint4(Sn[4], Sn[5], Sn[6], Sn[7]);
      }
      if (MEASURE) {
        // byte-wise sums over the eight words stay below 256 (Sn and F bytes
        // are 0/1, M bytes at most 2 Z), then one byte dot product each
        // byte sums as dot products: the ALU pipe is the busier one here
        unsigned su = 0, sf = 0;
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          su = __dp4a(Sn[i], 0x01010101u, su);
          sf = __dp4a(F[i], 0x01010101u, sf);
        }
        const int u = (int)su;
        ups += u;
        nacc += (int)sf;
        if (C == 1) {  // every neighbour of class 1 has the lower colour: all bonds counted here
          unsigned sm = 0, m = 0;
#pragma unroll
          for (int i = 0; i < 8; ++i) {
            const uint32_t M = 2u * A[i] + zoff;  // neighbour sum + Z per byte
            sm = __dp4a(Sn[i], M, sm);
            m = __dp4a(M, 0x01010101u, m);
          }
          bond += 2 * (int)sm - (int)m - Z * (2 * u - 32);
        }
      }
    }
  }
}

// The block's queued ties (sc2_range), one per thread, after every pair of
// the block has been stored: the flips and their changes to the sums.
template <int C, bool MEASURE>
__device__ __forceinline__ void sc2_ties(const IsingScArgs& a, const IsingTable& tab, const RngKey& key,
                                         const unsigned long long* s_thr, const uint2* s_tq, int n, int& bond,
                                         int& ups, int& nacc) {
  uint8_t* __restrict__ own = a.cls[C];
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const uint2 e = s_tq[i];
    const int k = (int)(e.y & 15u);
    const uint32_t s01 = (e.y >> 4) & 1u, nu = e.y >> 5;
    if (resolve_tie(e.x, k, s01, nu, tab.zeff, C, s_thr, key)) {
      own[(size_t)e.x * 16 + k] = (uint8_t)(s01 ^ 1u);
      if (MEASURE) {
        ups += 1 - 2 * (int)s01;
        nacc += 1;
        if (C == 1) bond -= 2 * (2 * (int)s01 - 1) * (2 * (int)nu - tab.zeff);
      }
    }
  }
}

template <int C, bool MEASURE, bool UPDATE, int PROP, bool ALLPER>
__global__ void __launch_bounds__(256, kSc2MinBlocks) ising_sc2_kernel(const IsingScArgs a, const FastDiv fG2,
                                                                       const IsingTable tab, const RngKey key,
                                                                       long long* __restrict__ part) {
  constexpr int W = 13;
  __shared__ unsigned long long s_thr[2 * W];
  __shared__ uint2 s_q[8][kScQueue];         // one group per thread: per-warp tie queues
  __shared__ uint2 s_tq[kSc2BlockQueue];     // pairs: the block's tie queue
  __shared__ int s_tn;
  pdl_launch_dependents();
  if (threadIdx.x == 0) s_tn = 0;
  for (int i = threadIdx.x; i < 2 * W; i += blockDim.x) s_thr[i] = tab.thr[i];
  __syncthreads();
  pdl_wait();
  int bond = 0, ups = 0, nacc = 0;
  // A class with no more groups than the grid has threads runs one group per
  // thread (twice the threads of pairs; 128^3: 5.4 -> 4.1 us per pass).
  // Larger classes run pairs: dealing the pairs left over after whole rounds
  // out as single groups, evenly over the SMs, was slower at 192^3 - 512^3
  // (256^3: 9.8 -> 10.4 us) than letting a quarter of the blocks run one
  // more pair round on issue slots the others have freed, and so were a
  // few leftover pairs for every warp (256^3: 805 -> 707 flips/ns) and one
  // contiguous range of pairs per block (805 -> 774; 512^3 1,085 -> 1,038).
  const uint32_t T = gridDim.x * blockDim.x;
  const uint32_t first = blockIdx.x * blockDim.x + (threadIdx.x & ~31u);
  if (a.groups <= T) {
    sc1_range<C, true, MEASURE, UPDATE, PROP>(a, tab, key, s_thr, s_q, first, a.groups, T, bond, ups, nacc);
  } else {
    sc2_range<C, MEASURE, UPDATE, PROP, ALLPER>(a, fG2, tab, key, s_thr, s_tq, &s_tn, first, a.groups >> 1, T,
                                                bond, ups, nacc);
    if (UPDATE) {
      __syncthreads();  // every pair of the block is stored
      sc2_ties<C, MEASURE>(a, tab, key, s_thr, s_tq, min(s_tn, kSc2BlockQueue), bond, ups, nacc);
    }
  }
  if (MEASURE) block_sum3_store(bond, ups, nacc, part + (size_t)blockIdx.x * kNumSums);
}

// ------------------------------------------------------------- generic
// Class entries dealt out per thread of a grid stride (entry j of the class:
// site sites[j]), so that a class of a few hundred thousand sites still fills
// the GPU.  Entry j draws
// byte (j & 15) of the blocks of group j >> 4, exactly as the 16-entry
// kernels do: the sixteen lanes of a half warp compute their group's block
// together (the same instructions, no extra issue).

// Acceptance of "U < th" with the first digit ub0 already drawn; later
// digits only on a tie (probability 1/256).
__device__ __forceinline__ bool decide1(unsigned long long th, uint32_t ub0, const RngKey& key, uint32_t g, int k,
                                        int colour) {
  if (th >= (1ull << 32)) return true;
  if (th == 0ull) return false;
  uint32_t tb = ((uint32_t)th >> 24) & 0xFFu;
  if (ub0 != tb) return ub0 < tb;
  for (int d = 1; d < 4; ++d) {
    const uint4 b = philox_ks(
        make_uint4(g, key.sweep, (kTagIsingAccept << 24) | ((uint32_t)colour << 8) | (uint32_t)d, key.replica),
        key.ks);
    const uint32_t ub = blk_byte(b, k);
    tb = ((uint32_t)th >> (24 - 8 * d)) & 0xFFu;
    if (ub != tb) return ub < tb;
  }
  return false;  // U == th: not below the threshold
}

// The first-digit byte of entry j and, for random proposals, whether its
// proposal differs from s (byte < 128 proposes Up).
template <bool UPDATE, int PROP>
__device__ __forceinline__ void draw1(const RngKey& key, uint32_t g, int k, int colour, uint32_t& ub0,
                                      uint32_t& prop_up) {
  ub0 = 0u;
  prop_up = 0u;
  if (!UPDATE) return;
  ub0 = blk_byte(
      philox_ks(make_uint4(g, key.sweep, (kTagIsingAccept << 24) | ((uint32_t)colour << 8), key.replica), key.ks),
      k);
  if (PROP == VG_PROPOSE_RANDOM)
    prop_up = blk_byte(philox_ks(make_uint4(g, key.sweep, (kTagIsingPropose << 24) | ((uint32_t)colour << 8),
                                            key.replica),
                                 key.ks),
                       k) < 128u
                  ? 1u
                  : 0u;
}

// NI class entries per thread at a time (j, j + stride, ...), every load of
// the NI entries issued before any store: a pass writes only its own class
// and reads only the others, so the loads of later entries never depend on
// the stores of earlier ones, but the compiler cannot know that across loop
// iterations.  One entry per iteration left the kernel waiting on two levels
// of dependent loads (index, then spin) per entry (bcc 128^3: 28.3 -> 40.4
// flips/ns, sc 255^3: 33.7 -> 53.0 with NI = 4).  Classes with no more
// entries than the grid has threads run NI = 1 (the batch's extra loads made
// sc 64^3 28 % slower).
template <int ZT, int NI, bool MEASURE, bool UPDATE, int PROP>
__global__ void __launch_bounds__(256, 4) ising_gen_kernel(const IsingGenArgs a, const IsingTable tab, const RngKey key,
                                                         const int colour, long long* __restrict__ part) {
  constexpr int W = 2 * ZT + 1;
  __shared__ unsigned long long s_thr[2 * W];
  const int z = a.z;
  const int Wz = 2 * z + 1;
  pdl_launch_dependents();
  for (int i = threadIdx.x; i < 2 * Wz; i += blockDim.x) s_thr[i] = tab.thr[i];
  __syncthreads();
  pdl_wait();

  int bond = 0, ups = 0, nacc = 0;  // per thread: a few entries of at most +-z each
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long j0 = (long long)blockIdx.x * blockDim.x + threadIdx.x; j0 < a.n_c; j0 += NI * stride) {
    int site[NI], s[NI], nsum[NI], nlow[NI];
    uint32_t lm[NI];
    bool live[NI];
#pragma unroll
    for (int b = 0; b < NI; ++b) {
      const long long j = j0 + b * stride;
      live[b] = j < a.n_c;
      // an entry past the class's end loads entry j0's data and is dropped:
      // unconditional loads let the compiler issue all of them up front
      const long long jj = live[b] ? j : j0;
      site[b] = __ldg(a.sites + jj);
      lm[b] = __ldg(a.lowmask + jj);
      nsum[b] = 0;
      nlow[b] = 0;
    }
#pragma unroll
    for (int b = 0; b < NI; ++b) s[b] = a.spin[site[b]];
#pragma unroll
    for (int q = 0; q < ZT; ++q) {
      if (q < z) {
#pragma unroll
        for (int b = 0; b < NI; ++b) {
          const long long jj = live[b] ? j0 + b * stride : j0;
          const int t = __ldg(a.nbr + ((uint32_t)q * (uint32_t)a.n_c + (uint32_t)jj));
          if (t >= 0) {
            const int v = 2 * (int)a.spin[t] - 1;
            nsum[b] += v;
            if ((lm[b] >> q) & 1u) nlow[b] += v;
          }
        }
      }
    }
#pragma unroll
    for (int b = 0; b < NI; ++b) {
      if (!live[b]) continue;
      const long long j = j0 + b * stride;
      const uint32_t g = (uint32_t)(j >> 4);
      const int k = (int)(j & 15);
      uint32_t ub0, up;
      draw1<UPDATE, PROP>(key, g, k, colour, ub0, up);
      bool acc = false;
      if (UPDATE && (PROP == VG_PROPOSE_FLIP || up != (uint32_t)s[b]))
        acc = decide1(s_thr[s[b] * Wz + nsum[b] + z], ub0, key, g, k, colour);
      const int sn = s[b] ^ (int)acc;
      if (acc) a.spin[site[b]] = (uint8_t)sn;
      if (MEASURE) {
        ups += sn;
        bond += sn ? nlow[b] : -nlow[b];
        nacc += acc;
      }
    }
  }
  if (MEASURE) block_sum3_store(bond, ups, nacc, part + (size_t)blockIdx.x * kNumSums);
}

template <int ZT, int NI, bool MEASURE, bool UPDATE, int PROP>
__global__ void __launch_bounds__(256) ising_bond_kernel(const IsingGenArgs a, const RngKey key, const int colour,
                                                         double* __restrict__ part) {
  // NI entries per thread at a time, loads before stores (as ising_gen_kernel)
  pdl_launch_dependents();
  pdl_wait();
  double bond = 0.0, ups = 0.0, nacc = 0.0;
  const int z = a.z;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long j0 = (long long)blockIdx.x * blockDim.x + threadIdx.x; j0 < a.n_c; j0 += NI * stride) {
    int site[NI];
    uint32_t s01[NI], lm[NI];
    double hj[NI], hlow[NI];
    bool live[NI];
#pragma unroll
    for (int b = 0; b < NI; ++b) {
      const long long j = j0 + b * stride;
      live[b] = j < a.n_c;
      const long long jj = live[b] ? j : j0;  // past the class's end: entry j0's data, dropped
      site[b] = __ldg(a.sites + jj);
      lm[b] = __ldg(a.lowmask + jj);
      hj[b] = 0.0;
      hlow[b] = 0.0;
    }
#pragma unroll
    for (int b = 0; b < NI; ++b) s01[b] = a.spin[site[b]];
#pragma unroll
    for (int q = 0; q < ZT; ++q) {
      if (q < z) {
#pragma unroll
        for (int b = 0; b < NI; ++b) {
          const long long jj = live[b] ? j0 + b * stride : j0;
          const uint32_t e = (uint32_t)q * (uint32_t)a.n_c + (uint32_t)jj;
          const int nb = __ldg(a.nbr + e);
          if (nb >= 0) {
            const double v = __ldg(a.jb + e) * (double)(2 * (int)a.spin[nb] - 1);
            hj[b] += v;
            if ((lm[b] >> q) & 1u) hlow[b] += v;
          }
        }
      }
    }
#pragma unroll
    for (int b = 0; b < NI; ++b) {
      if (!live[b]) continue;
      const long long j = j0 + b * stride;
      const uint32_t g = (uint32_t)(j >> 4);
      const int k = (int)(j & 15);
      uint32_t ub0, up;
      draw1<UPDATE, PROP>(key, g, k, colour, ub0, up);
      bool acc = false;
      if (UPDATE && (PROP == VG_PROPOSE_FLIP || up != s01[b])) {
        const double sd = s01[b] ? 1.0 : -1.0;
        const double e_old = -sd * hj[b] + a.hz * sd;
        const double e_new = -(-sd) * hj[b] + a.hz * (-sd);
        const double de = e_new - e_old;
        unsigned long long th;
        if (de <= 0.0) {
          th = 1ull << 32;
        } else {
          const double x = ceil(exp(-de / a.T) * 4294967296.0);
          th = x >= 4294967296.0 ? (1ull << 32) : x <= 0.0 ? 0ull : (unsigned long long)x;
        }
        acc = decide1(th, ub0, key, g, k, colour);
      }
      const int sn = (int)s01[b] ^ (int)acc;
      if (acc) a.spin[site[b]] = (uint8_t)sn;
      if (MEASURE) {
        ups += (double)sn;
        bond += sn ? hlow[b] : -hlow[b];
        nacc += acc ? 1.0 : 0.0;
      }
    }
  }
  if (MEASURE) {
    double v[kNumSums] = {bond, 0.0, 0.0, 0.0, 0.0, 0.0, ups, nacc};
    block_sum_store(v, part + (long long)blockIdx.x * kNumSums);
  }
}

// ------------------------------------------------------------ sublattice
// bcc / fcc Ising with one array per sublattice (the greedy colouring's
// classes; entry = cell index): a thread takes a run of 16 cells along x of
// class CLS.  Its neighbours on class Q are the runs of Q at the cells
// c + {0, d} e_a along the axes a where the two basis positions differ:
// whole 16-byte rows along y and z, and along x the same row shifted by one
// cell (its 16 bytes and the byte at the run's edge).  Entry j draws byte
// j & 15 of group j >> 4, so results equal the generic path's.
//
// Decisions are byte-parallel as in the sc pair kernel: every entry of a run
// has the same number nbe of existing neighbours (open y / z boundaries drop
// whole rows), except the edge entry when its x neighbour lies across an
// open boundary.  A shared table per (nbe, spin) holds the thresholds' top
// bytes for up-neighbour counts 0..15, looked up with two PRMTs per word;
// the first random digit is compared byte-parallel.  The rare ties (and the
// odd edge entry) go to a block queue that the whole block decides from the
// full thresholds after its runs (a warp would otherwise diverge into one
// more Philox block for one or two lanes in most rounds); their flips and
// sum changes are applied then.  Entries the queue has no room for are
// decided in line.
constexpr int kSubQueue = 512;  // tie entries per block

// Top bytes of the thresholds of 16 entries packed 4 per word (nu = up
// neighbours per byte, s = 0/1 spin per byte), from the 16-byte tables of
// the two spin values.
__device__ __forceinline__ uint32_t sub_top(uint32_t nu, uint32_t s, const uint4& t0, const uint4& t1) {
  const uint32_t sel = nibble_selector(nu);
  const uint32_t hm = ((nu >> 3) & 0x01010101u) * 0xFFu;
  const uint32_t sm = s * 0xFFu;
  const uint32_t a0 = (__byte_perm(t0.z, t0.w, sel) & hm) | (__byte_perm(t0.x, t0.y, sel) & ~hm);
  const uint32_t a1 = (__byte_perm(t1.z, t1.w, sel) & hm) | (__byte_perm(t1.x, t1.y, sel) & ~hm);
  return (a1 & sm) | (a0 & ~sm);
}

template <int NB, int CLS, bool MEASURE, bool UPDATE, int PROP>
__global__ void __launch_bounds__(256, 4) ising_sub_kernel(const IsingSubArgs a, const IsingTable tab, const RngKey key,
                                                           long long* __restrict__ part) {
  constexpr int ZC = NB == 2 ? 8 : 12;  // coordination
  constexpr int W = 2 * ZC + 1;
  constexpr int dx = half_pos<NB>(CLS, 0) ? 1 : -1, dy = half_pos<NB>(CLS, 1) ? 1 : -1,
                dz = half_pos<NB>(CLS, 2) ? 1 : -1;
  constexpr int edge = dx < 0 ? 0 : 15;        // the entry whose x neighbour lies outside the run
  constexpr int ZL = (NB == 2 ? 8 : 4) * CLS;  // bonds to lower classes per entry
  constexpr bool ALL_LOW = CLS == NB - 1;      // every neighbour class is lower
  __shared__ unsigned long long s_thr[2 * W];
  __shared__ uint4 s_top[ZC + 1][2];           // [nbe][spin]: top byte for nu = 0..15
  // tie queue: (group, k | s01 << 4 | first << 5 | nu << 6 | ne << 10 | nl << 14 | lk << 18)
  __shared__ uint2 s_tq[UPDATE ? kSubQueue : 1];
  __shared__ int s_tn;
  pdl_launch_dependents();
  if (threadIdx.x == 0) s_tn = 0;
  for (int i = threadIdx.x; i < 2 * W; i += blockDim.x) s_thr[i] = tab.thr[i];
  for (int i = threadIdx.x; i < (ZC + 1) * 32; i += blockDim.x) {
    const int nbe = i >> 5, s01 = (i >> 4) & 1, nu = i & 15;
    uint32_t top = 0u;
    if (nu <= nbe) {
      const unsigned long long t = tab.thr[s01 * W + 2 * nu - nbe + ZC];
      top = t >= (1ull << 32) ? 0xFFu : (uint32_t)(t >> 24);
    }
    reinterpret_cast<uint8_t*>(&s_top[nbe][s01])[nu] = (uint8_t)top;
  }
  __syncthreads();
  pdl_wait();
  uint8_t* __restrict__ own = a.base + (size_t)CLS * a.ncell;
  int bond = 0, ups = 0, nacc = 0;
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < a.groups; g += stride) {
    const uint32_t cell0 = g << 4;
    const uint32_t row = fdiv(cell0, a.fnx);
    const int x0 = (int)(cell0 - row * (uint32_t)a.nx);
    const int z = (int)fdiv(row, a.fny);
    const int y = (int)row - z * a.ny;
    int ys = y + dy, zs = z + dz, xe = dx < 0 ? x0 - 1 : x0 + 16;
    bool yok = true, zok = true, xok = true;
    if (ys < 0 || ys >= a.ny) {
      ys = ys < 0 ? a.ny - 1 : 0;
      yok = a.pby;
    }
    if (zs < 0 || zs >= a.nz) {
      zs = zs < 0 ? a.nz - 1 : 0;
      zok = a.pbz;
    }
    if (xe < 0 || xe >= a.nx) {
      xe = xe < 0 ? a.nx - 1 : 0;
      xok = a.pbx;
    }
    uint32_t A[4] = {0u, 0u, 0u, 0u}, Lo[4] = {0u, 0u, 0u, 0u};  // up neighbours per byte: all, lower classes
    int miss = 0, missL = 0, emiss = 0, emissL = 0;  // dropped bonds of every entry, and of the edge entry
#pragma unroll
    for (int q = 0; q < NB; ++q) {
      if (q == CLS) continue;
      const bool Dx = half_pos<NB>(q, 0) != half_pos<NB>(CLS, 0);
      const bool Dy = half_pos<NB>(q, 1) != half_pos<NB>(CLS, 1);
      const bool Dz = half_pos<NB>(q, 2) != half_pos<NB>(CLS, 2);
      const bool low = q < CLS && !ALL_LOW;
      const uint8_t* __restrict__ oq = a.base + (size_t)q * a.ncell;
#pragma unroll
      for (int iz = 0; iz < 2; ++iz) {
        if (iz && !Dz) continue;
#pragma unroll
        for (int iy = 0; iy < 2; ++iy) {
          if (iy && !Dy) continue;
          const int per = Dx ? 2 : 1;  // bonds this row carries per entry
          if ((iz && !zok) || (iy && !yok)) {
            miss += per;
            if (q < CLS) missL += per;
            continue;
          }
          const uint32_t r = ((uint32_t)(iz ? zs : z) * (uint32_t)a.ny + (uint32_t)(iy ? ys : y)) * (uint32_t)a.nx;
          const uint4 v = __ldg(reinterpret_cast<const uint4*>(oq + r + (uint32_t)x0));
          const uint32_t w[4] = {v.x, v.y, v.z, v.w};
          uint32_t X1[4] = {0u, 0u, 0u, 0u};
          if (Dx) {
            uint32_t e = 0u;
            if (xok) e = __ldg(oq + r + (uint32_t)xe);
            else {
              emiss += 1;
              if (q < CLS) emissL += 1;
            }
            if (dx < 0) {
              X1[0] = __byte_perm(e << 24, w[0], 0x6543);
#pragma unroll
              for (int i = 1; i < 4; ++i) X1[i] = __byte_perm(w[i - 1], w[i], 0x6543);
            } else {
#pragma unroll
              for (int i = 0; i < 3; ++i) X1[i] = __byte_perm(w[i], w[i + 1], 0x4321);
              X1[3] = __byte_perm(w[3], e, 0x4321);
            }
          }
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const uint32_t add = w[i] + X1[i];
            A[i] += add;
            if (low) Lo[i] += add;
          }
        }
      }
    }
    if (ALL_LOW) {
#pragma unroll
      for (int i = 0; i < 4; ++i) Lo[i] = A[i];
    }
    const uint4 Sv = *reinterpret_cast<const uint4*>(own + cell0);
    const uint32_t S[4] = {Sv.x, Sv.y, Sv.z, Sv.w};
    const int nbe = ZC - miss;
    uint32_t F[4] = {0u, 0u, 0u, 0u};
    if (UPDATE) {
      uint32_t cand[4] = {0x01010101u, 0x01010101u, 0x01010101u, 0x01010101u};
      if (PROP == VG_PROPOSE_RANDOM) {
        const uint4 pb =
            philox_ks(make_uint4(g, key.sweep, (kTagIsingPropose << 24) | ((uint32_t)CLS << 8), key.replica), key.ks);
        const uint32_t w[4] = {pb.x, pb.y, pb.z, pb.w};
#pragma unroll
        for (int i = 0; i < 4; ++i) cand[i] = ((~w[i] >> 7) & 0x01010101u) ^ S[i];
      }
      const uint32_t ecand = (cand[edge >> 2] >> (8 * (edge & 3))) & 1u;
      if (emiss) cand[edge >> 2] &= ~(0xFFu << (8 * (edge & 3)));  // decided below from its own threshold
      const uint4 b = philox_ks(make_uint4(g, key.sweep, (kTagIsingAccept << 24) | ((uint32_t)CLS << 8), key.replica),
                                key.ks);
      const uint32_t R[4] = {b.x, b.y, b.z, b.w};
      const uint4 t0 = s_top[nbe][0], t1 = s_top[nbe][1];
      uint32_t tm = 0u;  // entries tied with their threshold on the first digit
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const uint32_t thr = sub_top(A[i], S[i], t0, t1);
        F[i] = (bytes_gt80(thr, R[i]) >> 7) & cand[i];
        tm |= gather4(bytes_zero(R[i] ^ thr) & cand[i]) << (4 * i);
      }
      if (emiss && ecand) tm |= 1u << edge;  // the edge entry starts at the first digit
      for (uint32_t m = tm; m; m &= m - 1u) {
        const int k = __ffs(m) - 1;
        const int slot = atomicAdd(&s_tn, 1);
        if (slot < kSubQueue) {
          const uint32_t s01 = byte_at(S[0], S[1], S[2], S[3], k);
          const uint32_t nu = byte_at(A[0], A[1], A[2], A[3], k);
          const uint32_t nl = byte_at(Lo[0], Lo[1], Lo[2], Lo[3], k);
          const bool ek = k == edge && emiss;
          const uint32_t ne = (uint32_t)(nbe - (ek ? emiss : 0));
          const uint32_t lk = (uint32_t)(ZL - missL - (ek ? emissL : 0));
          s_tq[slot] = make_uint2(g, (uint32_t)k | (s01 << 4) | ((uint32_t)ek << 5) | (nu << 6) | (ne << 10) |
                                         (nl << 14) | (lk << 18));
          tm &= ~(1u << k);
        }
      }
      if (tm) {  // no room left in the queue
        const uint32_t nbe_e = (uint32_t)(nbe - emiss);
        uint32_t acc = 0u;
        for (int d = 0; d < 4 && tm; ++d) {
          uint4 bd = b;
          if (d > 0)
            bd = philox_ks(make_uint4(g, key.sweep, (kTagIsingAccept << 24) | ((uint32_t)CLS << 8) | (uint32_t)d,
                                      key.replica),
                           key.ks);
          for (uint32_t m = tm; m; m &= m - 1u) {
            const int k = __ffs(m) - 1;
            const uint32_t s01 = byte_at(S[0], S[1], S[2], S[3], k);
            const uint32_t nu = byte_at(A[0], A[1], A[2], A[3], k);
            const int ne = k == edge ? (int)nbe_e : nbe;
            const unsigned long long th = s_thr[s01 * W + 2 * (int)nu - ne + ZC];
            const uint32_t bit = 1u << k;
            if (th >= (1ull << 32)) {
              acc |= bit;
              tm &= ~bit;
              continue;
            }
            const bool first = k == edge && emiss && d == 0;  // not compared byte-parallel
            if (d == 0 && !first) continue;                 // tied on digit 0 already
            const uint32_t ub = blk_byte(bd, k);
            const uint32_t tb = ((uint32_t)th >> (24 - 8 * d)) & 0xFFu;
            if (ub < tb) {
              acc |= bit;
              tm &= ~bit;
            } else if (ub > tb) {
              tm &= ~bit;
            }
          }
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) F[i] |= spread4(acc >> (4 * i));
      }
    }
    uint32_t Sn[4], anyf = 0u;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      Sn[i] = S[i] ^ F[i];
      anyf |= F[i];
    }
    if (anyf) *reinterpret_cast<uint4*>(own + cell0) = make_uint4(Sn[0], Sn[1], Sn[2], Sn[3]);
    if (MEASURE) {
      unsigned su = 0u, sf = 0u;
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        su = __dp4a(Sn[i], 0x01010101u, su);
        sf = __dp4a(F[i], 0x01010101u, sf);
      }
      ups += (int)su;
      nacc += (int)sf;
      if (CLS > 0) {
        // sum_k (2 s_k - 1)(2 nl_k - L_k), L_k = L but L - emissL for the edge entry
        const int L = ZL - missL;
        unsigned snl = 0u, nls = 0u;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          snl = __dp4a(Sn[i], Lo[i], snl);
          nls = __dp4a(Lo[i], 0x01010101u, nls);
        }
        const int se = (int)((Sn[edge >> 2] >> (8 * (edge & 3))) & 1u);
        bond += 4 * (int)snl - 2 * (L * (int)su - emissL * se) - 2 * (int)nls + 16 * L - emissL;
      }
    }
  }
  if (UPDATE) {  // the queued entries, one per thread
    __syncthreads();
    const int nq = s_tn < kSubQueue ? s_tn : kSubQueue;
    for (int i = threadIdx.x; i < nq; i += blockDim.x) {
      const uint2 e = s_tq[i];
      const int k = (int)(e.y & 15u);
      const uint32_t s01 = (e.y >> 4) & 1u, first = (e.y >> 5) & 1u, nu = (e.y >> 6) & 15u, ne = (e.y >> 10) & 15u;
      const unsigned long long th = s_thr[s01 * W + 2 * (int)nu - (int)ne + ZC];
      bool acc = th >= (1ull << 32), done = acc;
      for (int d = first ? 0 : 1; d < 4 && !done; ++d) {
        const uint4 bd = philox_ks(
            make_uint4(e.x, key.sweep, (kTagIsingAccept << 24) | ((uint32_t)CLS << 8) | (uint32_t)d, key.replica),
            key.ks);
        const uint32_t ub = blk_byte(bd, k), tb = ((uint32_t)th >> (24 - 8 * d)) & 0xFFu;
        if (ub != tb) {
          acc = ub < tb;
          done = true;
        }
      }
      if (acc) {  // U < thr; a tie on every digit (U == thr) rejects
        own[(size_t)e.x * 16 + k] = (uint8_t)(s01 ^ 1u);
        if (MEASURE) {
          ups += 1 - 2 * (int)s01;
          nacc += 1;
          if (CLS > 0) {
            const int nl = (int)((e.y >> 14) & 15u), lk = (int)((e.y >> 18) & 15u);
            bond -= 2 * (2 * (int)s01 - 1) * (2 * nl - lk);
          }
        }
      }
    }
  }
  if (MEASURE) block_sum3_store(bond, ups, nacc, part + (size_t)blockIdx.x * kNumSums);
}

// ------------------------------------------------------------ dispatch
template <int C, bool UNIFORM>
static cudaError_t sc_dispatch(const IsingScArgs& a, const IsingTable& tab, RngKey key, int proposal, bool update,
                               long long* part, int grid, int tpb, cudaStream_t s) {
  const bool m = part != nullptr;
  if (!update) return launch_pdl(ising_sc_kernel<C, UNIFORM, true, false, VG_PROPOSE_FLIP>, grid, tpb, s, a, tab, key, part);
  if (proposal == VG_PROPOSE_FLIP) {
    if (m) return launch_pdl(ising_sc_kernel<C, UNIFORM, true, true, VG_PROPOSE_FLIP>, grid, tpb, s, a, tab, key, part);
    return launch_pdl(ising_sc_kernel<C, UNIFORM, false, true, VG_PROPOSE_FLIP>, grid, tpb, s, a, tab, key, part);
  }
  if (m) return launch_pdl(ising_sc_kernel<C, UNIFORM, true, true, VG_PROPOSE_RANDOM>, grid, tpb, s, a, tab, key, part);
  return launch_pdl(ising_sc_kernel<C, UNIFORM, false, true, VG_PROPOSE_RANDOM>, grid, tpb, s, a, tab, key, part);
}

template <int C, bool ALLPER>
static cudaError_t sc2_dispatch(const IsingScArgs& a, const IsingTable& tab, RngKey key, int proposal, bool update,
                                long long* part, int grid, int tpb, cudaStream_t s) {
  const bool m = part != nullptr;
  const FastDiv f2 = make_fastdiv((uint32_t)(a.G >> 1));
  if (!update)
    return launch_pdl(ising_sc2_kernel<C, true, false, VG_PROPOSE_FLIP, ALLPER>, grid, tpb, s, a, f2, tab, key, part);
  if (proposal == VG_PROPOSE_FLIP) {
    if (m) return launch_pdl(ising_sc2_kernel<C, true, true, VG_PROPOSE_FLIP, ALLPER>, grid, tpb, s, a, f2, tab, key, part);
    return launch_pdl(ising_sc2_kernel<C, false, true, VG_PROPOSE_FLIP, ALLPER>, grid, tpb, s, a, f2, tab, key, part);
  }
  if (m) return launch_pdl(ising_sc2_kernel<C, true, true, VG_PROPOSE_RANDOM, ALLPER>, grid, tpb, s, a, f2, tab, key, part);
  return launch_pdl(ising_sc2_kernel<C, false, true, VG_PROPOSE_RANDOM, ALLPER>, grid, tpb, s, a, f2, tab, key, part);
}

// Pairs of groups per thread when every site has the same coordination and
// rows hold an even number of groups.
static bool use_pairs(const IsingScArgs& a, const IsingTable& tab) { return tab.zeff >= 0 && a.G % 2 == 0; }

// Resident blocks per SM of the sc kernel that launch_ising_sc runs for
// these arguments (for grid sizing).
int ising_sc_blocks_per_sm(const IsingScArgs& a, const IsingTable& tab, int tpb) {
  int n = 0;
  if (use_pairs(a, tab))
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, ising_sc2_kernel<1, true, true, VG_PROPOSE_FLIP, true>, tpb, 0);
  else if (tab.zeff >= 0)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, ising_sc_kernel<1, true, true, true, VG_PROPOSE_FLIP>, tpb, 0);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, ising_sc_kernel<1, false, true, true, VG_PROPOSE_FLIP>, tpb, 0);
  return n > 0 ? n : 1;
}

cudaError_t launch_ising_sc(const IsingScArgs& a, const IsingTable& tab, RngKey key, int colour, int proposal,
                            bool update, long long* part, int grid, int tpb, cudaStream_t s) {
  if (use_pairs(a, tab)) {
    const bool allper = a.pbx && a.pby && a.pbz;
    if (colour == 0) {
      return allper ? sc2_dispatch<0, true>(a, tab, key, proposal, update, part, grid, tpb, s)
                    : sc2_dispatch<0, false>(a, tab, key, proposal, update, part, grid, tpb, s);
    }
    return allper ? sc2_dispatch<1, true>(a, tab, key, proposal, update, part, grid, tpb, s)
                  : sc2_dispatch<1, false>(a, tab, key, proposal, update, part, grid, tpb, s);
  }
  const bool uniform = tab.zeff >= 0;
  if (colour == 0) {
    return uniform ? sc_dispatch<0, true>(a, tab, key, proposal, update, part, grid, tpb, s)
                   : sc_dispatch<0, false>(a, tab, key, proposal, update, part, grid, tpb, s);
  }
  return uniform ? sc_dispatch<1, true>(a, tab, key, proposal, update, part, grid, tpb, s)
                 : sc_dispatch<1, false>(a, tab, key, proposal, update, part, grid, tpb, s);
}

template <int ZT, int NI>
static cudaError_t gen_dispatch_ni(const IsingGenArgs& a, const IsingTable& tab, RngKey key, int colour,
                                   int proposal, bool update, long long* part, int grid, int tpb, cudaStream_t s) {
  const bool m = part != nullptr;
  if (!update) {
    launch_pdl(ising_gen_kernel<ZT, NI, true, false, VG_PROPOSE_FLIP>, grid, tpb, s, a, tab, key, colour, part);
  } else if (proposal == VG_PROPOSE_FLIP) {
    if (m) launch_pdl(ising_gen_kernel<ZT, NI, true, true, VG_PROPOSE_FLIP>, grid, tpb, s, a, tab, key, colour, part);
    else launch_pdl(ising_gen_kernel<ZT, NI, false, true, VG_PROPOSE_FLIP>, grid, tpb, s, a, tab, key, colour, part);
  } else {
    if (m) launch_pdl(ising_gen_kernel<ZT, NI, true, true, VG_PROPOSE_RANDOM>, grid, tpb, s, a, tab, key, colour, part);
    else launch_pdl(ising_gen_kernel<ZT, NI, false, true, VG_PROPOSE_RANDOM>, grid, tpb, s, a, tab, key, colour, part);
  }
  return cudaGetLastError();
}

// more class entries than threads: NI entries at a time (4 up to eight
// neighbours, 2 for twelve: registers)
template <int ZT>
static cudaError_t gen_dispatch(const IsingGenArgs& a, const IsingTable& tab, RngKey key, int colour, int proposal,
                                bool update, long long* part, int grid, int tpb, cudaStream_t s) {
  if (a.n_c > (long long)grid * tpb)
    return gen_dispatch_ni<ZT, ZT <= 8 ? 4 : 2>(a, tab, key, colour, proposal, update, part, grid, tpb, s);
  return gen_dispatch_ni<ZT, 1>(a, tab, key, colour, proposal, update, part, grid, tpb, s);
}

template <int ZT, int NI>
static cudaError_t bond_dispatch_ni(const IsingGenArgs& a, RngKey key, int colour, int proposal, bool update,
                                    double* part, int grid, int tpb, cudaStream_t s) {
  const bool m = part != nullptr;
  if (!update) {
    launch_pdl(ising_bond_kernel<ZT, NI, true, false, VG_PROPOSE_FLIP>, grid, tpb, s, a, key, colour, part);
  } else if (proposal == VG_PROPOSE_FLIP) {
    if (m) launch_pdl(ising_bond_kernel<ZT, NI, true, true, VG_PROPOSE_FLIP>, grid, tpb, s, a, key, colour, part);
    else launch_pdl(ising_bond_kernel<ZT, NI, false, true, VG_PROPOSE_FLIP>, grid, tpb, s, a, key, colour, part);
  } else {
    if (m) launch_pdl(ising_bond_kernel<ZT, NI, true, true, VG_PROPOSE_RANDOM>, grid, tpb, s, a, key, colour, part);
    else launch_pdl(ising_bond_kernel<ZT, NI, false, true, VG_PROPOSE_RANDOM>, grid, tpb, s, a, key, colour, part);
  }
  return cudaGetLastError();
}

template <int ZT>
static cudaError_t bond_dispatch(const IsingGenArgs& a, RngKey key, int colour, int proposal, bool update,
                                 double* part, int grid, int tpb, cudaStream_t s) {
  if (a.n_c > (long long)grid * tpb) return bond_dispatch_ni<ZT, 2>(a, key, colour, proposal, update, part, grid, tpb, s);
  return bond_dispatch_ni<ZT, 1>(a, key, colour, proposal, update, part, grid, tpb, s);
}

cudaError_t launch_ising_gen(const IsingGenArgs& a, const IsingTable& tab, RngKey key, int colour, int proposal,
                             bool update, long long* part, int grid, int tpb, cudaStream_t s) {
  if (a.jb) {  // per-bond constants: FP64 partial rows in the same 8-byte slots
    double* dpart = reinterpret_cast<double*>(part);
    if (a.z <= 6) return bond_dispatch<6>(a, key, colour, proposal, update, dpart, grid, tpb, s);
    if (a.z <= 8) return bond_dispatch<8>(a, key, colour, proposal, update, dpart, grid, tpb, s);
    return bond_dispatch<12>(a, key, colour, proposal, update, dpart, grid, tpb, s);
  }
  if (a.z <= 6) return gen_dispatch<6>(a, tab, key, colour, proposal, update, part, grid, tpb, s);
  if (a.z <= 8) return gen_dispatch<8>(a, tab, key, colour, proposal, update, part, grid, tpb, s);
  return gen_dispatch<12>(a, tab, key, colour, proposal, update, part, grid, tpb, s);
}

template <int NB, int CLS>
static cudaError_t sub_dispatch(const IsingSubArgs& a, const IsingTable& tab, RngKey key, int proposal, bool update,
                                long long* part, int grid, int tpb, cudaStream_t s) {
  const bool m = part != nullptr;
  if (!update) return launch_pdl(ising_sub_kernel<NB, CLS, true, false, VG_PROPOSE_FLIP>, grid, tpb, s, a, tab, key, part);
  if (proposal == VG_PROPOSE_FLIP) {
    if (m) return launch_pdl(ising_sub_kernel<NB, CLS, true, true, VG_PROPOSE_FLIP>, grid, tpb, s, a, tab, key, part);
    return launch_pdl(ising_sub_kernel<NB, CLS, false, true, VG_PROPOSE_FLIP>, grid, tpb, s, a, tab, key, part);
  }
  if (m) return launch_pdl(ising_sub_kernel<NB, CLS, true, true, VG_PROPOSE_RANDOM>, grid, tpb, s, a, tab, key, part);
  return launch_pdl(ising_sub_kernel<NB, CLS, false, true, VG_PROPOSE_RANDOM>, grid, tpb, s, a, tab, key, part);
}

cudaError_t launch_ising_sub(const IsingSubArgs& a, int nb, const IsingTable& tab, RngKey key, int colour,
                             int proposal, bool update, long long* part, int grid, int tpb, cudaStream_t s) {
  if (nb == 2)
    return colour == 0 ? sub_dispatch<2, 0>(a, tab, key, proposal, update, part, grid, tpb, s)
                       : sub_dispatch<2, 1>(a, tab, key, proposal, update, part, grid, tpb, s);
  switch (colour) {
    case 0: return sub_dispatch<4, 0>(a, tab, key, proposal, update, part, grid, tpb, s);
    case 1: return sub_dispatch<4, 1>(a, tab, key, proposal, update, part, grid, tpb, s);
    case 2: return sub_dispatch<4, 2>(a, tab, key, proposal, update, part, grid, tpb, s);
    default: return sub_dispatch<4, 3>(a, tab, key, proposal, update, part, grid, tpb, s);
  }
}

}  // namespace vg
