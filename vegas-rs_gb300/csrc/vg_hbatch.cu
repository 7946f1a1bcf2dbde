// vg_hbatch.cu -- batched Heisenberg replicas of one bcc or fcc lattice under
// a shared field schedule (the vg_hbatch_* ABI).
//
// Replaces, for many replicas at once, MetropolisIntegrator::step for
// HeisenbergSpin (src/integrator.rs:66-92) driven by HysteresisLoop::run
// (src/program.rs:281-335): every field point relaxes, then measures, each
// replica at its own temperature and energy constants.
//
// Layout in HBM: one SoA plane per (replica, sublattice, component),
// [replica][class][xyz][cell] with cell = (z ny + y) nx + x.  The colour
// classes are the basis sublattices: in bcc and fcc every nearest neighbour
// of a site lies on another sublattice, so a sublattice is an independent
// set, and it is exactly the class the greedy colouring assigns (the site
// of basis b of a cell always finds colours 0..b-1 taken by the earlier
// basis sites of its own cell and colour b free).  The neighbours of basis b
// on basis q sit in the cells c + sum_{a in D(b,q)} {0, d_b[a]} e_a, where
// D(b,q) are the axes on which the two basis positions differ by half a
// cell (bcc: all three, 8 neighbours; fcc: two, 4 neighbours per other
// sublattice) and d_b[a] = +1 if basis b sits at the half-cell position on
// axis a, -1 otherwise.  A run of four cells along x is one float4 per
// plane; the x-shifted run reuses it plus one scalar at the run's edge.
//
// One launch per colour covers every replica (grid.y = replica).  The
// lattice sums a measured sweep reports are tracked, not recomputed: before
// the measured sweeps of a field point one kernel sums the state exactly
// (each bond from its higher-class end); during them every accepted move
// adds its change of each sum, which the pass already has in registers (the
// field h of the site is current, so the bond-sum change (s' - s).h is
// exact).  Partials are FP32 per thread and warp and FP64 per block row; a
// reduction kernel adds the rows, in a fixed order, to FP64 running totals
// and those to the per-point accumulators.  A field point (relax sweeps,
// exact sums, measured sweeps, counter advance) is captured once into a
// CUDA graph and replayed for every point; the kernels read the sweep
// counter and the field value from device memory.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "vg_heis_common.cuh"
#include "vg_sublattice.cuh"

using namespace vg;

namespace {

constexpr int kHbSums = VG_HB_NSUMS;
constexpr int kTpb = 256;            // reduction and set-up kernels
constexpr int kPassTpb = 256;        // colour passes and measurement
// 64 registers: 32 resident warps per SM (latency-bound loads).  One run
// already has its 36 neighbour loads in flight: two runs per thread at a
// time, loads before stores, ran the c5 sample at 62 flips/ns against 74.7
// (spilling at 64 registers, or at 80 with three blocks per SM).
constexpr int kPassMinBlocks = 4;
constexpr int kTrackMinBlocks = 4;   // tracked passes too (partials in shared memory)

template <typename R>
struct HbArgs {
  R* spin;             // [rep][class][xyz][cell]
  uint32_t ncell;
  int nx, ny, nz;
  int pbx, pby, pbz;
  uint32_t runs;       // ncell / W
  FastDiv frow;        // run index -> row (runs per row = nx / W)
  FastDiv fny;
  int rpr;             // runs per row
};

struct HbRep {         // per replica
  KeySchedule ks;
  uint32_t replica, k0, k1, pad;
  double beta, J, K, Kc;
  float fbeta, fJ, fK, fKc;  // the same constants in FP32 for the FP32 kernels
};

// The per-point field value in both precisions.
struct HbField {
  double h;
  float hf, pad;
};

struct HbShared {      // per batch
  double ax, ay, az, bx, by, bz, zsign;
  float fax, fay, faz, fbx, fby, fbz, fzsign, pad;
};

struct HbDev {         // device counters read by every kernel of a point
  uint32_t sweep_base;
  int32_t point;
};

template <typename R>
__device__ __forceinline__ HeisParams<R> rep_params(const HbRep& rp, const HbShared& sh, const HbField& f) {
  HeisParams<R> P;
  if constexpr (sizeof(R) == 4) {
    P.J = rp.fJ;
    P.K = rp.fK;
    P.Kc = rp.fKc;
    P.beta = rp.fbeta;
    P.hz = sh.fzsign * f.hf;
    P.ax = sh.fax;
    P.ay = sh.fay;
    P.az = sh.faz;
    P.bx = sh.fbx;
    P.by = sh.fby;
    P.bz = sh.fbz;
  } else {
    P.J = rp.J;
    P.K = rp.K;
    P.Kc = rp.Kc;
    P.beta = rp.beta;
    P.hz = sh.zsign * f.h;
    P.ax = sh.ax;
    P.ay = sh.ay;
    P.az = sh.az;
    P.bx = sh.bx;
    P.by = sh.by;
    P.bz = sh.bz;
  }
  P.T = (R)0;  // unused by the update
  return P;
}

// One colour pass of every replica: grid (blocks per replica, replicas).
// TRACK (measured sweeps): every accepted move adds its change of the
// lattice sums to the thread's partials -- bond sum (s' - s).h, which is
// exact because no two sites of a class are neighbours and h is the current
// field; (s'.e)^2 - (s.e)^2; the quartic sum; s' - s; one accepted move --
// and the block writes one row [class][replica][block].  (The Zeeman sum is
// M.b and follows from the magnetisation.)  The partials live in the
// thread's own shared-memory slots, which keeps the registers of the
// update free.
template <typename R, int NB, int CLS, int W, bool TRACK, int PROP>
__global__ void __launch_bounds__(kPassTpb, TRACK ? kTrackMinBlocks : kPassMinBlocks) hb_pass(const HbArgs<R> a, const HbRep* __restrict__ reps,
                                                                  const HbShared sh, const HbField* __restrict__ fields,
                                                                  const HbDev* __restrict__ dev, const uint32_t t,
                                                                  double* __restrict__ part) {
  const int r = blockIdx.y;
  const HbRep rp = reps[r];
  const HbDev d = *dev;
  const HeisParams<R> P = rep_params<R>(rp, sh, fields[d.point]);
  const uint32_t sweep = d.sweep_base + t;
  R* rep_base = a.spin + (size_t)r * NB * 3 * a.ncell;
  R* own[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) own[c] = rep_base + (size_t)(CLS * 3 + c) * a.ncell;
  constexpr int kTracked = 7;  // bond, aniso, cubic, mx, my, mz, accepted
  __shared__ R s_dl[TRACK ? kTracked : 1][kPassTpb];
  if (TRACK) {
#pragma unroll
    for (int i = 0; i < kTracked; ++i) s_dl[i][threadIdx.x] = (R)0;
  }
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < a.runs; u += stride) {
    const int row = (int)fdiv(u, a.frow);
    const int x0 = (int)(u - (uint32_t)row * (uint32_t)a.rpr) * W;
    const int z = (int)fdiv((uint32_t)row, a.fny);
    const int y = row - z * a.ny;
    Run<R, W> hf[3];
    run_field<R, NB, CLS, W>(a, rep_base, x0, y, z, hf);
    const uint32_t j0 = (uint32_t)row * (uint32_t)a.nx + (uint32_t)x0;
    Run<R, W> S[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) S[c] = load_run<R, W>(own[c] + j0);
    bool changed = false;
#pragma unroll
    for (int k = 0; k < W; ++k) {
      const V3<R> s = {S[0].v[k], S[1].v[k], S[2].v[k]};
      const V3<R> h = {hf[0].v[k], hf[1].v[k], hf[2].v[k]};
      const uint4 w =
          philox_ks<kHeisRounds>(make_uint4(j0 + (uint32_t)k, sweep, (kTagHeis << 24) | ((uint32_t)CLS << 8), rp.replica),
                                 rp.ks);
      V3<R> sn;
      if (heis_update<R, PROP>(s, h, P, w, sn)) {
        S[0].v[k] = sn.x;
        S[1].v[k] = sn.y;
        S[2].v[k] = sn.z;
        changed = true;
        if (TRACK) {
          const V3<R> ds = {sn.x - s.x, sn.y - s.y, sn.z - s.z};
          const R pe = sn.x * P.ax + sn.y * P.ay + sn.z * P.az;
          const R se = s.x * P.ax + s.y * P.ay + s.z * P.az;
          const int q = threadIdx.x;
          s_dl[0][q] += ds.x * h.x + ds.y * h.y + ds.z * h.z;
          s_dl[1][q] += pe * pe - se * se;
          s_dl[2][q] += quart(sn) - quart(s);
          s_dl[3][q] += ds.x;
          s_dl[4][q] += ds.y;
          s_dl[5][q] += ds.z;
          s_dl[6][q] += (R)1;
        }
      }
    }
    if (changed) {
#pragma unroll
      for (int c = 0; c < 3; ++c) store_run<R, W>(own[c] + j0, S[c]);
    }
  }
  if (TRACK) {
    const int q = threadIdx.x;
    R dl[kNumSums] = {s_dl[0][q], s_dl[1][q], (R)0, s_dl[2][q], s_dl[3][q], s_dl[4][q], s_dl[5][q], s_dl[6][q]};
    flush_sums(dl, part + ((size_t)CLS * gridDim.y + r) * gridDim.x * kNumSums);
  }
}

// Lattice sums of every replica after a sweep (all classes final): per run
// of W cells, each class's site terms and its bonds to the lower classes.
// FP32 per thread and warp, FP64 per block row [replica][block].
template <typename R, int NB, int CLS, int W>
__device__ __forceinline__ void measure_class(const HbArgs<R>& a, const R* rep_base, int x0, int y, int z,
                                              uint32_t j0, const HeisParams<R>& P, R (&acc)[kNumSums]) {
  Run<R, W> S[3], lo[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) S[c] = load_run<R, W>(rep_base + (size_t)(CLS * 3 + c) * a.ncell + j0);
  low_field<R, NB, CLS, W>(a, rep_base, x0, y, z, lo);
#pragma unroll
  for (int k = 0; k < W; ++k) {
    const V3<R> s = {S[0].v[k], S[1].v[k], S[2].v[k]};
    const V3<R> low = {lo[0].v[k], lo[1].v[k], lo[2].v[k]};
    add_site_sums(acc, s, low, P);
  }
}

template <typename R, int NB, int W>
__global__ void __launch_bounds__(kPassTpb) hb_measure(const HbArgs<R> a, const HbShared sh,
                                                       double* __restrict__ part) {
  const int r = blockIdx.y;
  HeisParams<R> P{};
  P.ax = (R)sh.ax;
  P.ay = (R)sh.ay;
  P.az = (R)sh.az;
  P.bx = (R)sh.bx;
  P.by = (R)sh.by;
  P.bz = (R)sh.bz;
  const R* rep_base = a.spin + (size_t)r * NB * 3 * a.ncell;
  R acc[kNumSums];
#pragma unroll
  for (int i = 0; i < kNumSums; ++i) acc[i] = (R)0;
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < a.runs; u += stride) {
    const int row = (int)fdiv(u, a.frow);
    const int x0 = (int)(u - (uint32_t)row * (uint32_t)a.rpr) * W;
    const int z = (int)fdiv((uint32_t)row, a.fny);
    const int y = row - z * a.ny;
    const uint32_t j0 = (uint32_t)row * (uint32_t)a.nx + (uint32_t)x0;
    measure_class<R, NB, 0, W>(a, rep_base, x0, y, z, j0, P, acc);
    measure_class<R, NB, 1, W>(a, rep_base, x0, y, z, j0, P, acc);
    if constexpr (NB == 4) {
      measure_class<R, NB, 2, W>(a, rep_base, x0, y, z, j0, P, acc);
      measure_class<R, NB, 3, W>(a, rep_base, x0, y, z, j0, P, acc);
    }
  }
  flush_sums(acc, part + (size_t)r * gridDim.x * kNumSums);
}

// Block rows [rows][replica r][nbx] of replica r summed in a fixed order
// with Kahan compensation (block r = replica; 256 threads: value v = tid % 8,
// lane tid / 8), then the 32 lanes of each value combined by a fixed
// shuffle tree; thread 0 returns the totals.  (FP64 latency is long on this
// part, so no thread walks a long serial chain.)
__device__ __forceinline__ void sum_rows(const double* __restrict__ part, int rows, int nbx, int n_rep, int r,
                                         double (&s)[kNumSums]) {
  __shared__ double s_sum[kNumSums][32];
  __shared__ double s_tot[kNumSums];
  const int v = threadIdx.x % kNumSums, lane = threadIdx.x / kNumSums;
  double sum = 0.0, comp = 0.0;
  for (int c = 0; c < rows; ++c) {
    const double* p = part + (((size_t)c * n_rep + r) * nbx) * kNumSums + v;
    for (int bx = lane; bx < nbx; bx += 32) {
      const double y = p[(size_t)bx * kNumSums] - comp;
      const double t = sum + y;
      comp = (t - sum) - y;
      sum = t;
    }
  }
  s_sum[v][lane] = sum - comp;
  __syncthreads();
  if (threadIdx.x < 32 * kNumSums) {  // warp w combines value w (blockDim = 256)
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    double x = s_sum[w][l];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (l == 0) s_tot[w] = x;
  }
  __syncthreads();
  if (threadIdx.x == 0)
    for (int k = 0; k < kNumSums; ++k) s[k] = s_tot[k];
}

// Exact lattice sums of every replica (hb_measure rows) become the running
// totals that the tracked sweeps update.
__global__ void __launch_bounds__(kTpb) hb_sync(const double* __restrict__ part, int nbx, int n_rep,
                                                double* __restrict__ tot) {
  double s[kNumSums];
  sum_rows(part, 1, nbx, n_rep, blockIdx.x, s);
  if (threadIdx.x == 0)
    for (int k = 0; k < 7; ++k) tot[(size_t)blockIdx.x * kNumSums + k] = s[k];
}

// After a measured sweep: adds the sweep's changes (rows of the nb passes)
// to the running totals and the totals to the point accumulators.
__global__ void __launch_bounds__(kTpb) hb_reduce(const double* __restrict__ part, int nb, int nbx, int n_rep,
                                                  double* __restrict__ tot, const HbRep* __restrict__ reps,
                                                  const HbShared sh, const HbField* __restrict__ fields,
                                                  const HbDev* __restrict__ dev, double* __restrict__ acc) {
  const int r = blockIdx.x;
  double s[kNumSums];
  sum_rows(part, nb, nbx, n_rep, r, s);
  if (threadIdx.x == 0) {
    double* T = tot + (size_t)r * kNumSums;
    for (int k = 0; k < 7; ++k) T[k] += s[k];
    T[2] = sh.bx * T[4] + sh.by * T[5] + sh.bz * T[6];  // sum s.b = M.b
    for (int k = 0; k < 7; ++k) s[k] = T[k];
    const HbDev d = *dev;
    const HbRep rp = reps[r];
    const double h = fields[d.point].h;
    const double m2 = s[4] * s[4] + s[5] * s[5] + s[6] * s[6];
    const double m = sqrt(m2);
    const double e = -2.0 * rp.J * s[0] + rp.K * s[1] + sh.zsign * h * s[2] - rp.Kc * s[3];
    double* o = acc + ((size_t)d.point * n_rep + r) * kHbSums;
    for (int k = 0; k < kNumSums; ++k) o[k] += s[k];
    o[8] += m;
    o[9] += m2;
    o[10] += e;
    o[11] += e * e;
  }
}

__global__ void hb_advance(HbDev* dev, uint32_t sweeps) {
  dev->sweep_base += sweeps;
  dev->point += 1;
}

template <typename R, int NB>
__global__ void hb_init(HbArgs<R> a, const HbRep* __restrict__ reps) {
  const int r = blockIdx.y;
  const HbRep rp = reps[r];
  RngKey key;
  key.k0 = rp.k0;
  key.k1 = rp.k1;
  key.replica = rp.replica;
  key.sweep = 0;
  R* base = a.spin + (size_t)r * NB * 3 * a.ncell;
  const uint32_t n = a.ncell * (uint32_t)NB;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t cell = i / NB, b = i % NB;
    const V3<R> s = heis_init_spin<R>(i, key);
    base[(size_t)(b * 3 + 0) * a.ncell + cell] = s.x;
    base[(size_t)(b * 3 + 1) * a.ncell + cell] = s.y;
    base[(size_t)(b * 3 + 2) * a.ncell + cell] = s.z;
  }
}

template <typename R>
__global__ void hb_import(R* base, uint32_t ncell, int nb, const double* __restrict__ src, int* flag) {
  const uint32_t n = ncell * (uint32_t)nb;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t cell = i / nb, b = i % nb;
    const double x = src[3 * (size_t)i], y = src[3 * (size_t)i + 1], z = src[3 * (size_t)i + 2];
    if (!(fabs(x * x + y * y + z * z - 1.0) < 1e-3)) atomicOr(flag, 1);
    base[(size_t)(b * 3 + 0) * ncell + cell] = (R)x;
    base[(size_t)(b * 3 + 1) * ncell + cell] = (R)y;
    base[(size_t)(b * 3 + 2) * ncell + cell] = (R)z;
  }
}

template <typename R>
__global__ void hb_export(const R* base, uint32_t ncell, int nb, double* __restrict__ dst) {
  const uint32_t n = ncell * (uint32_t)nb;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t cell = i / nb, b = i % nb;
    dst[3 * (size_t)i] = (double)base[(size_t)(b * 3 + 0) * ncell + cell];
    dst[3 * (size_t)i + 1] = (double)base[(size_t)(b * 3 + 1) * ncell + cell];
    dst[3 * (size_t)i + 2] = (double)base[(size_t)(b * 3 + 2) * ncell + cell];
  }
}

// ------------------------------------------------------------ dispatch
using PassFn = void (*)(const void* args, const HbRep* reps, const HbShared& sh, const HbField* fields,
                        const HbDev* dev, uint32_t t, double* part, dim3 grid, cudaStream_t s);

template <typename R, int NB, int CLS, int W, bool COUNT, int PROP>
void pass_launch(const void* args, const HbRep* reps, const HbShared& sh, const HbField* fields, const HbDev* dev,
                 uint32_t t, double* part, dim3 grid, cudaStream_t s) {
  hb_pass<R, NB, CLS, W, COUNT, PROP>
      <<<grid, kPassTpb, 0, s>>>(*static_cast<const HbArgs<R>*>(args), reps, sh, fields, dev, t, part);
}

template <typename R, int NB, int W, bool COUNT, int PROP>
PassFn pick_cls(int cls) {
  switch (cls) {
    case 0: return pass_launch<R, NB, 0, W, COUNT, PROP>;
    case 1: return pass_launch<R, NB, 1, W, COUNT, PROP>;
    case 2: return NB == 4 ? pass_launch<R, NB, (NB == 4 ? 2 : 0), W, COUNT, PROP> : nullptr;
    default: return NB == 4 ? pass_launch<R, NB, (NB == 4 ? 3 : 0), W, COUNT, PROP> : nullptr;
  }
}

template <typename R, int NB, int W>
PassFn pick_mp(int cls, bool count, int proposal) {
  if (proposal == VG_PROPOSE_RANDOM)
    return count ? pick_cls<R, NB, W, true, VG_PROPOSE_RANDOM>(cls) : pick_cls<R, NB, W, false, VG_PROPOSE_RANDOM>(cls);
  return count ? pick_cls<R, NB, W, true, VG_PROPOSE_FLIP>(cls) : pick_cls<R, NB, W, false, VG_PROPOSE_FLIP>(cls);
}

PassFn pick_pass(bool fp64, int nb, int w, int cls, bool count, int proposal) {
  if (fp64) return nb == 2 ? pick_mp<double, 2, 1>(cls, count, proposal) : pick_mp<double, 4, 1>(cls, count, proposal);
  if (w == 4) return nb == 2 ? pick_mp<float, 2, 4>(cls, count, proposal) : pick_mp<float, 4, 4>(cls, count, proposal);
  return nb == 2 ? pick_mp<float, 2, 1>(cls, count, proposal) : pick_mp<float, 4, 1>(cls, count, proposal);
}

template <typename R, int NB, int W>
void measure_launch(const HbArgs<R>& a, const HbShared& sh, double* part, dim3 grid, cudaStream_t s) {
  hb_measure<R, NB, W><<<grid, kPassTpb, 0, s>>>(a, sh, part);
}

}  // namespace

struct vg_hbatch {
  int device = 0;
  cudaStream_t own_stream = nullptr, stream = nullptr;
  vg_hbatch_desc desc{};
  int nb = 2, n_rep = 0, w = 1;
  bool fp64 = false;
  uint32_t ncell = 0;
  int nbx = 1;
  HbArgs<float> a32{};
  HbArgs<double> a64{};
  HbShared sh{};
  void* d_spin = nullptr;
  HbRep* d_reps = nullptr;
  double* d_part = nullptr;
  double* d_mpart = nullptr;     // hb_measure rows [replica][block]
  double* d_tot = nullptr;       // running totals [replica][kNumSums]
  HbField* d_fields = nullptr;
  int fields_cap = 0;
  double* d_acc = nullptr;
  size_t acc_points = 0;
  HbDev* d_dev = nullptr;
  int* d_flag = nullptr;
  double* d_stage = nullptr;
  uint64_t sweep = 0;
  int last_points = 0;
  cudaGraphExec_t graph = nullptr;
  uint32_t g_relax = 0, g_measure = 0;
  int64_t device_bytes = 0;
  std::string err;
};

extern "C" void vg_internal_set_last_error(const char* msg);

namespace {

int hfail(vg_hbatch* b, int code, const std::string& m) {
  if (b) b->err = m;
  vg_internal_set_last_error(m.c_str());
  return code;
}

#define VG_HCUDA(b, expr)                                                                          \
  do {                                                                                             \
    cudaError_t _e = (expr);                                                                       \
    if (_e != cudaSuccess)                                                                         \
      return hfail((b), _e == cudaErrorMemoryAllocation ? VG_ERR_OOM : VG_ERR_CUDA,                \
                   std::string(#expr) + ": " + cudaGetErrorString(_e));                            \
  } while (0)

template <typename T>
int halloc(vg_hbatch* b, T** p, size_t count) {
  const size_t bytes = std::max<size_t>(count, 1) * sizeof(T);
  VG_HCUDA(b, cudaMalloc((void**)p, bytes));
  b->device_bytes += (int64_t)bytes;
  return VG_OK;
}

void hdestroy(vg_hbatch* b) {
  if (!b) return;
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->graph) cudaGraphExecDestroy(b->graph);
  cudaFree(b->d_spin);
  cudaFree(b->d_reps);
  cudaFree(b->d_part);
  cudaFree(b->d_mpart);
  cudaFree(b->d_tot);
  cudaFree(b->d_fields);
  cudaFree(b->d_acc);
  cudaFree(b->d_dev);
  cudaFree(b->d_flag);
  cudaFree(b->d_stage);
  if (b->own_stream) cudaStreamDestroy(b->own_stream);
  delete b;
}

const void* args_of(const vg_hbatch* b) {
  return b->fp64 ? static_cast<const void*>(&b->a64) : static_cast<const void*>(&b->a32);
}

int enqueue_sweep(vg_hbatch* b, uint32_t t, bool measure) {
  const dim3 grid((unsigned)b->nbx, (unsigned)b->n_rep);
  for (int c = 0; c < b->nb; ++c) {
    PassFn f = pick_pass(b->fp64, b->nb, b->w, c, measure, b->desc.proposal);
    f(args_of(b), b->d_reps, b->sh, b->d_fields, b->d_dev, t, b->d_part, grid, b->stream);
    VG_HCUDA(b, cudaGetLastError());
  }
  if (measure) {
    hb_reduce<<<b->n_rep, kTpb, 0, b->stream>>>(b->d_part, b->nb, b->nbx, b->n_rep, b->d_tot, b->d_reps, b->sh,
                                                b->d_fields, b->d_dev, b->d_acc);
    VG_HCUDA(b, cudaGetLastError());
  }
  return VG_OK;
}

// Exact sums of the current state into the running totals.
int enqueue_sync(vg_hbatch* b) {
  const dim3 grid((unsigned)b->nbx, (unsigned)b->n_rep);
  if (b->fp64) {
    if (b->nb == 2) measure_launch<double, 2, 1>(b->a64, b->sh, b->d_mpart, grid, b->stream);
    else measure_launch<double, 4, 1>(b->a64, b->sh, b->d_mpart, grid, b->stream);
  } else if (b->w == 4) {
    if (b->nb == 2) measure_launch<float, 2, 4>(b->a32, b->sh, b->d_mpart, grid, b->stream);
    else measure_launch<float, 4, 4>(b->a32, b->sh, b->d_mpart, grid, b->stream);
  } else {
    if (b->nb == 2) measure_launch<float, 2, 1>(b->a32, b->sh, b->d_mpart, grid, b->stream);
    else measure_launch<float, 4, 1>(b->a32, b->sh, b->d_mpart, grid, b->stream);
  }
  VG_HCUDA(b, cudaGetLastError());
  hb_sync<<<b->n_rep, kTpb, 0, b->stream>>>(b->d_mpart, b->nbx, b->n_rep, b->d_tot);
  VG_HCUDA(b, cudaGetLastError());
  return VG_OK;
}

// One field point: relax sweeps, exact sums, measured (tracked) sweeps,
// counter advance.
int enqueue_point(vg_hbatch* b, uint32_t relax, uint32_t measure) {
  int rc;
  for (uint32_t t = 0; t < relax; ++t)
    if ((rc = enqueue_sweep(b, t, false))) return rc;
  if (measure && (rc = enqueue_sync(b))) return rc;
  for (uint32_t t = relax; t < relax + measure; ++t)
    if ((rc = enqueue_sweep(b, t, true))) return rc;
  hb_advance<<<1, 1, 0, b->stream>>>(b->d_dev, relax + measure);
  VG_HCUDA(b, cudaGetLastError());
  return VG_OK;
}

int check_replica(vg_hbatch* b, int32_t r, int64_t n_sites, const void* p) {
  if (r < 0 || r >= b->n_rep) return hfail(b, VG_ERR_INVALID_ARG, "replica index out of range");
  if (!p) return hfail(b, VG_ERR_INVALID_ARG, "NULL state buffer");
  if (n_sites != (int64_t)b->ncell * b->nb) return hfail(b, VG_ERR_INVALID_ARG, "state size does not match the lattice");
  return VG_OK;
}

}  // namespace

extern "C" {

int vg_hbatch_create(const vg_hbatch_desc* d, const vg_heis_replica* reps, int32_t n_rep, vg_hbatch** out) {
  if (!out || !d || !reps) return hfail(nullptr, VG_ERR_INVALID_ARG, "NULL argument");
  *out = nullptr;
  const vg_lattice_desc& L = d->lattice;
  if (L.cell != VG_CELL_BCC && L.cell != VG_CELL_FCC)
    return hfail(nullptr, VG_ERR_UNSUPPORTED, "batched Heisenberg replicas need a bcc or fcc lattice");
  if (L.nx < 1 || L.ny < 1 || L.nz < 1) return hfail(nullptr, VG_ERR_INVALID_ARG, "lattice extents must be >= 1");
  if (n_rep < 1 || n_rep > 65535) return hfail(nullptr, VG_ERR_INVALID_ARG, "n_replicas must be in [1, 65535]");
  if (d->precision != VG_FP32 && d->precision != VG_FP64) return hfail(nullptr, VG_ERR_INVALID_ARG, "unknown precision");
  if (d->proposal != VG_PROPOSE_RANDOM && d->proposal != VG_PROPOSE_FLIP)
    return hfail(nullptr, VG_ERR_INVALID_ARG, "unknown proposal");
  const int nb = L.cell == VG_CELL_BCC ? 2 : 4;
  const double ncell = (double)L.nx * L.ny * L.nz;
  if (ncell * nb > 2147483647.0) return hfail(nullptr, VG_ERR_UNSUPPORTED, "lattice has more than 2^31-1 sites");
  if (3.0 * ncell * nb >= 4294967296.0)  // 32-bit offsets within a replica
    return hfail(nullptr, VG_ERR_UNSUPPORTED, "a replica holds more than 2^32 spin components");
  for (int k = 0; k < 3; ++k)
    if (!std::isfinite(d->anisotropy_axis[k]) || !std::isfinite(d->field_axis[k]))
      return hfail(nullptr, VG_ERR_INVALID_ARG, "axes must be finite");
  if (!std::isfinite(d->zeeman_sign)) return hfail(nullptr, VG_ERR_INVALID_ARG, "zeeman_sign must be finite");
  for (int r = 0; r < n_rep; ++r) {
    const vg_heis_replica& q = reps[r];
    if (!std::isfinite(q.temperature) || !std::isfinite(q.exchange) || !std::isfinite(q.anisotropy) ||
        !std::isfinite(q.cubic))
      return hfail(nullptr, VG_ERR_INVALID_ARG, "replica constants must be finite");
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    return hfail(nullptr, VG_ERR_NO_DEVICE, "no CUDA device is visible");

  vg_hbatch* b = new (std::nothrow) vg_hbatch();
  if (!b) return hfail(nullptr, VG_ERR_OOM, "host allocation failed");
  cudaGetDevice(&b->device);
  if (cudaStreamCreateWithFlags(&b->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
    hdestroy(b);
    return hfail(nullptr, VG_ERR_CUDA, "stream creation failed");
  }
  b->stream = b->own_stream;
  b->desc = *d;
  b->nb = nb;
  b->n_rep = n_rep;
  b->fp64 = d->precision == VG_FP64;
  b->ncell = (uint32_t)ncell;
  b->w = (!b->fp64 && L.nx % 4 == 0) ? 4 : 1;
  const uint32_t runs = b->ncell / (uint32_t)b->w;
  // two waves of resident blocks over all replicas (four per SM at the pass
  // kernels' 64 registers), each block walking several runs of 256: fewer
  // block rows to reduce in the measured sweeps than one block per 256 runs
  // (fcc 64^3 cells x 64 replicas: 60.3 -> 63.9 flips/ns; one wave 60.6,
  // four 63.6, sixteen 62.2)
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device) != cudaSuccess || sms < 1) sms = 1;
  const uint32_t wave = (uint32_t)std::max(1, 2 * sms * kPassMinBlocks / n_rep);
  b->nbx = (int)std::min<uint32_t>(std::min<uint32_t>((runs + kPassTpb - 1) / kPassTpb, wave), 4096u);
  auto fill = [&](auto& a) {
    a.ncell = b->ncell;
    a.nx = L.nx;
    a.ny = L.ny;
    a.nz = L.nz;
    a.pbx = L.pbc_x != 0;
    a.pby = L.pbc_y != 0;
    a.pbz = L.pbc_z != 0;
    a.runs = runs;
    a.rpr = L.nx / b->w;
    a.frow = make_fastdiv((uint32_t)a.rpr);
    a.fny = make_fastdiv((uint32_t)L.ny);
  };
  fill(b->a32);
  fill(b->a64);
  // Unit axes; a zero axis leaves the term at zero.
  auto unit = [](const double* v, double* o) {
    const double n = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    for (int k = 0; k < 3; ++k) o[k] = n > 0.0 ? v[k] / n : 0.0;
  };
  double ax[3], bx[3];
  unit(d->anisotropy_axis, ax);
  unit(d->field_axis, bx);
  b->sh = HbShared{ax[0], ax[1], ax[2], bx[0], bx[1], bx[2], d->zeeman_sign,
                   (float)ax[0], (float)ax[1], (float)ax[2], (float)bx[0], (float)bx[1], (float)bx[2],
                   (float)d->zeeman_sign, 0.f};

  std::vector<HbRep> h(n_rep);
  for (int r = 0; r < n_rep; ++r) {
    const vg_heis_replica& q = reps[r];
    const uint32_t k0 = (uint32_t)q.seed, k1 = (uint32_t)(q.seed >> 32);
    h[r].ks = make_key_schedule(k0, k1);
    h[r].replica = q.replica;
    h[r].k0 = k0;
    h[r].k1 = k1;
    h[r].pad = 0;
    // Thermostat::new clamps T to f64::EPSILON (src/thermostat.rs:29-39)
    const double eps = 2.220446049250313e-16;
    const double T = q.temperature < eps ? eps : q.temperature;
    h[r].beta = 1.0 / T;
    h[r].J = q.exchange;
    h[r].K = q.anisotropy;
    h[r].Kc = q.cubic;
    h[r].fbeta = (float)h[r].beta;
    h[r].fJ = (float)q.exchange;
    h[r].fK = (float)q.anisotropy;
    h[r].fKc = (float)q.cubic;
  }
  const size_t planes = (size_t)n_rep * nb * 3 * b->ncell;
  int rc = 0;
  if (b->fp64) {
    double* p = nullptr;
    rc = halloc(b, &p, planes);
    b->d_spin = p;
    b->a64.spin = p;
  } else {
    float* p = nullptr;
    rc = halloc(b, &p, planes);
    b->d_spin = p;
    b->a32.spin = p;
  }
  if (!rc) rc = halloc(b, &b->d_reps, (size_t)n_rep);
  if (!rc) rc = halloc(b, &b->d_part, (size_t)nb * n_rep * b->nbx * kNumSums);
  if (!rc) rc = halloc(b, &b->d_mpart, (size_t)n_rep * b->nbx * kNumSums);
  if (!rc) rc = halloc(b, &b->d_tot, (size_t)n_rep * kNumSums);
  if (!rc) rc = halloc(b, &b->d_dev, 1);
  if (!rc) rc = halloc(b, &b->d_flag, 1);
  if (!rc) rc = halloc(b, &b->d_fields, 1);
  if (rc) {
    std::string e = b->err;
    hdestroy(b);
    return hfail(nullptr, rc, e);
  }
  b->fields_cap = 1;
  const HbField zero{0.0, 0.f, 0.f};
  const HbDev d0{0u, 0};
  cudaError_t e = cudaMemcpyAsync(b->d_reps, h.data(), sizeof(HbRep) * n_rep, cudaMemcpyHostToDevice, b->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(b->d_fields, &zero, sizeof(HbField), cudaMemcpyHostToDevice, b->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(b->d_dev, &d0, sizeof(HbDev), cudaMemcpyHostToDevice, b->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(b->d_spin, 0, planes * (b->fp64 ? 8 : 4), b->stream);

  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  if (e != cudaSuccess) {
    hdestroy(b);
    return hfail(nullptr, VG_ERR_CUDA, std::string("batch set-up: ") + cudaGetErrorString(e));
  }
  *out = b;
  return VG_OK;
}

int vg_hbatch_destroy(vg_hbatch* b) {
  if (!b) return VG_ERR_INVALID_ARG;
  hdestroy(b);
  return VG_OK;
}

const char* vg_hbatch_last_error(const vg_hbatch* b) { return b ? b->err.c_str() : ""; }

int vg_hbatch_get_info(const vg_hbatch* b, vg_hbatch_info* o) {
  if (!b || !o) return VG_ERR_INVALID_ARG;
  o->n_replicas = b->n_rep;
  o->n_classes = b->nb;
  o->sites_per_replica = (int64_t)b->ncell * b->nb;
  o->sweep_index = b->sweep;
  o->sites_per_thread = b->w;
  o->graph = b->graph != nullptr;
  o->device_bytes = b->device_bytes;
  return VG_OK;
}

int vg_hbatch_get_stream(const vg_hbatch* b, void** s) {
  if (!b || !s) return VG_ERR_INVALID_ARG;
  *s = (void*)b->stream;
  return VG_OK;
}

int vg_hbatch_init_random(vg_hbatch* b) {
  if (!b) return VG_ERR_INVALID_ARG;
  VG_HCUDA(b, cudaSetDevice(b->device));
  const dim3 grid(std::max(1u, std::min<uint32_t>((b->ncell * b->nb + kTpb - 1) / kTpb, 1024u)), (unsigned)b->n_rep);
  if (b->fp64) {
    if (b->nb == 2) hb_init<double, 2><<<grid, kTpb, 0, b->stream>>>(b->a64, b->d_reps);
    else hb_init<double, 4><<<grid, kTpb, 0, b->stream>>>(b->a64, b->d_reps);
  } else {
    if (b->nb == 2) hb_init<float, 2><<<grid, kTpb, 0, b->stream>>>(b->a32, b->d_reps);
    else hb_init<float, 4><<<grid, kTpb, 0, b->stream>>>(b->a32, b->d_reps);
  }
  VG_HCUDA(b, cudaGetLastError());
  VG_HCUDA(b, cudaStreamSynchronize(b->stream));
  return VG_OK;
}

int vg_hbatch_set_replica(vg_hbatch* b, int32_t r, const double* xyz, int64_t n_sites) {
  if (!b) return VG_ERR_INVALID_ARG;
  int rc = check_replica(b, r, n_sites, xyz);
  if (rc) return rc;
  VG_HCUDA(b, cudaSetDevice(b->device));
  if (!b->d_stage && (rc = halloc(b, &b->d_stage, (size_t)n_sites * 3))) return rc;
  VG_HCUDA(b, cudaMemcpyAsync(b->d_stage, xyz, (size_t)n_sites * 3 * 8, cudaMemcpyHostToDevice, b->stream));
  VG_HCUDA(b, cudaMemsetAsync(b->d_flag, 0, sizeof(int), b->stream));
  const size_t off = (size_t)r * b->nb * 3 * b->ncell;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((n_sites + kTpb - 1) / kTpb, 1024));
  if (b->fp64) hb_import<double><<<grid, kTpb, 0, b->stream>>>(b->a64.spin + off, b->ncell, b->nb, b->d_stage, b->d_flag);
  else hb_import<float><<<grid, kTpb, 0, b->stream>>>(b->a32.spin + off, b->ncell, b->nb, b->d_stage, b->d_flag);
  VG_HCUDA(b, cudaGetLastError());
  int flag = 0;
  VG_HCUDA(b, cudaMemcpyAsync(&flag, b->d_flag, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
  VG_HCUDA(b, cudaStreamSynchronize(b->stream));
  if (flag) return hfail(b, VG_ERR_INVALID_ARG, "Heisenberg spins must be unit vectors");
  return VG_OK;
}

int vg_hbatch_get_replica(vg_hbatch* b, int32_t r, double* xyz, int64_t n_sites) {
  if (!b) return VG_ERR_INVALID_ARG;
  int rc = check_replica(b, r, n_sites, xyz);
  if (rc) return rc;
  VG_HCUDA(b, cudaSetDevice(b->device));
  if (!b->d_stage && (rc = halloc(b, &b->d_stage, (size_t)n_sites * 3))) return rc;
  const size_t off = (size_t)r * b->nb * 3 * b->ncell;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((n_sites + kTpb - 1) / kTpb, 1024));
  if (b->fp64) hb_export<double><<<grid, kTpb, 0, b->stream>>>(b->a64.spin + off, b->ncell, b->nb, b->d_stage);
  else hb_export<float><<<grid, kTpb, 0, b->stream>>>(b->a32.spin + off, b->ncell, b->nb, b->d_stage);
  VG_HCUDA(b, cudaGetLastError());
  VG_HCUDA(b, cudaMemcpyAsync(xyz, b->d_stage, (size_t)n_sites * 3 * 8, cudaMemcpyDeviceToHost, b->stream));
  VG_HCUDA(b, cudaStreamSynchronize(b->stream));
  return VG_OK;
}

int vg_hbatch_run_async(vg_hbatch* b, const double* fields, int32_t n_points, uint32_t relax, uint32_t measure) {
  if (!b) return VG_ERR_INVALID_ARG;
  if (!fields || n_points < 1) return hfail(b, VG_ERR_INVALID_ARG, "the field schedule is empty");
  if (relax + measure == 0 || relax + measure < relax) return hfail(b, VG_ERR_INVALID_ARG, "a field point needs sweeps");
  for (int i = 0; i < n_points; ++i)
    if (!std::isfinite(fields[i])) return hfail(b, VG_ERR_INVALID_ARG, "field values must be finite");
  if (!sweep_range_ok(b->sweep, (uint64_t)n_points * ((uint64_t)relax + measure)))
    return hfail(b, VG_ERR_INVALID_ARG, "the run passes sweep index 2^32 (the 32-bit sweep word of the Philox counter)");
  VG_HCUDA(b, cudaSetDevice(b->device));
  int rc;
  // Buffers baked into the captured graph: growing one drops the graph.
  if (n_points > b->fields_cap || (size_t)n_points > b->acc_points) {
    VG_HCUDA(b, cudaStreamSynchronize(b->stream));
    if (b->graph) {
      cudaGraphExecDestroy(b->graph);
      b->graph = nullptr;
    }
    if (n_points > b->fields_cap) {
      cudaFree(b->d_fields);
      b->d_fields = nullptr;
      const int cap = std::max(n_points, 2 * b->fields_cap);
      if ((rc = halloc(b, &b->d_fields, (size_t)cap))) return rc;
      b->fields_cap = cap;
    }
    if ((size_t)n_points > b->acc_points) {
      cudaFree(b->d_acc);
      b->d_acc = nullptr;
      const size_t cap = std::max<size_t>((size_t)n_points, 2 * b->acc_points);
      if ((rc = halloc(b, &b->d_acc, cap * b->n_rep * kHbSums))) return rc;
      b->acc_points = cap;
    }
  }
  if (b->graph && (b->g_relax != relax || b->g_measure != measure)) {
    VG_HCUDA(b, cudaStreamSynchronize(b->stream));
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  std::vector<HbField> fv((size_t)n_points);
  for (int i = 0; i < n_points; ++i) fv[i] = HbField{fields[i], (float)fields[i], 0.f};
  VG_HCUDA(b, cudaMemcpyAsync(b->d_fields, fv.data(), sizeof(HbField) * n_points, cudaMemcpyHostToDevice, b->stream));
  VG_HCUDA(b, cudaMemsetAsync(b->d_acc, 0, sizeof(double) * n_points * b->n_rep * kHbSums, b->stream));
  const HbDev d0{(uint32_t)b->sweep, 0};
  VG_HCUDA(b, cudaMemcpyAsync(b->d_dev, &d0, sizeof(d0), cudaMemcpyHostToDevice, b->stream));
  VG_HCUDA(b, cudaStreamSynchronize(b->stream));  // the host copies above come from caller memory
  if (!b->graph) {
    cudaGraph_t g = nullptr;
    bool ok = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
    if (ok) {
      const int erc = enqueue_point(b, relax, measure);
      ok = cudaStreamEndCapture(b->stream, &g) == cudaSuccess && erc == VG_OK;
    }
    if (ok && cudaGraphInstantiate(&b->graph, g, 0) != cudaSuccess) b->graph = nullptr;
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();  // a failed capture falls back to direct launches
    b->g_relax = relax;
    b->g_measure = measure;
  }
  for (int p = 0; p < n_points; ++p) {
    if (b->graph) {
      VG_HCUDA(b, cudaGraphLaunch(b->graph, b->stream));
    } else if ((rc = enqueue_point(b, relax, measure))) {
      return rc;
    }
  }
  b->sweep += (uint64_t)n_points * (relax + measure);
  b->last_points = n_points;
  return VG_OK;
}

int vg_hbatch_synchronize(vg_hbatch* b) {
  if (!b) return VG_ERR_INVALID_ARG;
  VG_HCUDA(b, cudaStreamSynchronize(b->stream));
  return VG_OK;
}

int vg_hbatch_run(vg_hbatch* b, const double* fields, int32_t n_points, uint32_t relax, uint32_t measure) {
  int rc = vg_hbatch_run_async(b, fields, n_points, relax, measure);
  if (rc) return rc;
  return vg_hbatch_synchronize(b);
}

int vg_hbatch_point_sums(vg_hbatch* b, double* out, int64_t cap) {
  if (!b || !out) return VG_ERR_INVALID_ARG;
  const int64_t need = (int64_t)b->last_points * b->n_rep * kHbSums;
  if (b->last_points == 0) return hfail(b, VG_ERR_INVALID_ARG, "no run yet");
  if (cap < need) return hfail(b, VG_ERR_INVALID_ARG, "output buffer too small");
  VG_HCUDA(b, cudaSetDevice(b->device));
  VG_HCUDA(b, cudaMemcpyAsync(out, b->d_acc, sizeof(double) * need, cudaMemcpyDeviceToHost, b->stream));
  VG_HCUDA(b, cudaStreamSynchronize(b->stream));
  return VG_OK;
}

int vg_hbatch_time_passes(vg_hbatch* b, uint32_t n, double* ms) {
  if (!b || !ms || n == 0) return VG_ERR_INVALID_ARG;
  if (!sweep_range_ok(b->sweep, n))
    return hfail(b, VG_ERR_INVALID_ARG, "the run passes sweep index 2^32 (the 32-bit sweep word of the Philox counter)");
  VG_HCUDA(b, cudaSetDevice(b->device));
  const HbField zero{0.0, 0.f, 0.f};
  const HbDev d0{(uint32_t)b->sweep, 0};
  VG_HCUDA(b, cudaMemcpyAsync(b->d_fields, &zero, sizeof(HbField), cudaMemcpyHostToDevice, b->stream));
  VG_HCUDA(b, cudaStreamSynchronize(b->stream));
  VG_HCUDA(b, cudaMemcpyAsync(b->d_dev, &d0, sizeof(d0), cudaMemcpyHostToDevice, b->stream));
  cudaEvent_t e0, e1;
  VG_HCUDA(b, cudaEventCreate(&e0));
  VG_HCUDA(b, cudaEventCreate(&e1));
  VG_HCUDA(b, cudaEventRecord(e0, b->stream));
  int rc = VG_OK;
  for (uint32_t t = 0; t < n && !rc; ++t) rc = enqueue_sweep(b, t, false);
  cudaEventRecord(e1, b->stream);
  const cudaError_t se = cudaStreamSynchronize(b->stream);
  float el = 0.f;
  if (!rc && se == cudaSuccess) cudaEventElapsedTime(&el, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  VG_HCUDA(b, se);
  b->sweep += n;
  b->last_points = 0;
  *ms = (double)el / n;
  return VG_OK;
}

}  // extern "C"
