// vg_noalloc.cu -- an Ising sweep entry point that allocates no memory.
//
// Some callers cannot call cudaMalloc: a plugin hosted by a framework that
// owns all device memory through its own pool allocator, code that enqueues
// work while someone else is capturing the stream into a CUDA graph, or a
// real-time loop in which an allocation (which may synchronise the device)
// is not allowed.  vg_ising_sc_sweeps_noalloc runs the same checkerboard
// colour passes as vg_sweeps on spin arrays and an output buffer the caller
// already owns.  The only other memory the passes need -- one row of partial
// sums per thread block and colour pass, reduced per sweep -- lives in the
// fixed-size array below, which every GPU that loads this library holds until
// the process exits.
//
// Set-up: the first call on a device looks up the array's device address
// (cudaGetSymbolAddress) with that device current and caches it; make that
// first call before any stream capture.  The cached address belongs to the
// device's primary context: after a device reset it is stale and there is no
// way to look it up again, so the entry point must not be used on a device
// the process has reset.  All calls share the one array and
// each colour pass overwrites every row it later reads, so nothing has to be
// cleared between calls -- but calls whose work overlaps on the GPU (two
// streams, or two host threads) race on the array and must be serialised by
// the caller.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>

#include "vg_internal.cuh"

extern "C" void vg_internal_set_last_error(const char* msg);

namespace {

using namespace vg;

constexpr int kNoAllocChunk = 8;                      // sweeps per reduction
constexpr int kNoAllocMaxRowsPerPass = 2048;          // thread blocks per colour pass
constexpr size_t kNoAllocRows = (size_t)kNoAllocChunk * 2 * kNoAllocMaxRowsPerPass;

// 8 sweeps x 2 colour passes x 2048 blocks x 8 int64 = 2 MiB
__device__ __align__(256) long long g_noalloc_scratch[kNoAllocRows * kNumSums];

constexpr int kMaxDevices = 64;
void* g_scratch_addr[kMaxDevices] = {};
std::mutex g_scratch_mutex;

int fail(int code, const char* msg) {
  vg_internal_set_last_error(msg);
  return code;
}

// Per-sweep rows -> finished sums (bond, N, mz, N, 0, 0, mz, accepted), the
// layout of vg_sums; the zeeman member is mz whatever the field's
// orientation (the caller folded it into the coefficient).
__global__ void noalloc_finish(const long long* __restrict__ rows, int rows_per_sweep, long long n_sites,
                               double* __restrict__ out) {
  __shared__ long long s[3][256];
  const long long* r = rows + (size_t)blockIdx.x * rows_per_sweep * kNumSums;
  long long b = 0, u = 0, a = 0;
  for (int i = threadIdx.x; i < rows_per_sweep; i += blockDim.x) {
    b += r[(size_t)i * kNumSums + 0];
    u += r[(size_t)i * kNumSums + 6];
    a += r[(size_t)i * kNumSums + 7];
  }
  s[0][threadIdx.x] = b;
  s[1][threadIdx.x] = u;
  s[2][threadIdx.x] = a;
  __syncthreads();
  if (threadIdx.x == 0) {
    long long tb = 0, tu = 0, ta = 0;
    for (int i = 0; i < (int)blockDim.x; ++i) {
      tb += s[0][i];
      tu += s[1][i];
      ta += s[2][i];
    }
    const double mz = 2.0 * (double)tu - (double)n_sites;
    double* o = out + (size_t)blockIdx.x * kNumSums;
    o[0] = (double)tb;
    o[1] = (double)n_sites;
    o[2] = mz;
    o[3] = (double)n_sites;
    o[4] = 0.0;
    o[5] = 0.0;
    o[6] = mz;
    o[7] = (double)ta;
  }
}

}  // namespace

extern "C" int vg_ising_sc_sweeps_noalloc(const vg_lattice_desc* L, double exchange, double zeeman,
                                          double temperature, uint64_t seed, uint32_t replica, uint64_t sweep0,
                                          uint64_t n_sweeps, uint8_t* class0, uint8_t* class1, double* sums_out,
                                          void* cuda_stream) {
  if (!L || !class0 || !class1) return fail(VG_ERR_INVALID_ARG, "NULL lattice or spin array");
  if (L->cell != VG_CELL_SC || L->nx < 32 || L->ny < 1 || L->nz < 1 || L->nx % 2 || (L->nx / 2) % kIsingGroup ||
      (L->pbc_y && L->ny % 2) || (L->pbc_z && L->nz % 2) || (L->pbc_y && L->ny == 1) || (L->pbc_z && L->nz == 1))
    return fail(VG_ERR_UNSUPPORTED,
                "no-alloc sweeps need an sc lattice with x a multiple of 32 and even extents (>= 2) on periodic axes");
  if ((double)L->nx * L->ny * L->nz > 2147483647.0) return fail(VG_ERR_UNSUPPORTED, "lattice has more than 2^31-1 sites");
  if (std::isnan(temperature) || !std::isfinite(exchange) || !std::isfinite(zeeman))
    return fail(VG_ERR_INVALID_ARG, "temperature, exchange and field must be numbers");
  if (!sweep_range_ok(sweep0, n_sweeps))
    return fail(VG_ERR_INVALID_ARG, "sweep0 + n_sweeps passes 2^32 (the 32-bit sweep word of the Philox counter)");
  const double eps = 2.220446049250313e-16;
  const double T = temperature < eps ? eps : temperature;

  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return fail(VG_ERR_NO_DEVICE, "no current CUDA device");
  long long* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_addr[dev]) {
      void* p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess) return fail(VG_ERR_CUDA, cudaGetErrorString(e));
      g_scratch_addr[dev] = p;
    }
    scratch = (long long*)g_scratch_addr[dev];
  }
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return fail(VG_ERR_CUDA, "cannot query the multiprocessor count");

  IsingScArgs a;
  a.cls[0] = class0;
  a.cls[1] = class1;
  a.Hx = L->nx / 2;
  a.Ly = L->ny;
  a.Lz = L->nz;
  a.G = a.Hx / kIsingGroup;
  a.groups = (uint32_t)a.G * (uint32_t)a.Ly * (uint32_t)a.Lz;
  a.pbx = L->pbc_x != 0;
  a.pby = L->pbc_y != 0;
  a.pbz = L->pbc_z != 0;
  a.fG = make_fastdiv((uint32_t)a.G);
  a.fLy = make_fastdiv((uint32_t)a.Ly);
  set_sc_offsets(a);
  const int tpb = 256;
  const long long want = ((long long)a.groups + tpb - 1) / tpb;
  const int grid = (int)std::max(1LL, std::min(want, (long long)sms * 8));
  if (grid > kNoAllocMaxRowsPerPass)
    return fail(VG_ERR_UNSUPPORTED, "no-alloc sweeps: the launch needs more partial-sum rows than the 2 MiB "
                                    "scratch array holds (at most 2048 thread blocks per colour pass)");

  const int ext[3] = {L->nx, L->ny, L->nz};
  const int per[3] = {L->pbc_x, L->pbc_y, L->pbc_z};
  const IsingTable tab = make_ising_table(exchange, zeeman, T, 6, true, ext, per);
  cudaStream_t s = (cudaStream_t)cuda_stream;
  const long long n_sites = (long long)L->nx * L->ny * L->nz;
  for (uint64_t t0 = 0; t0 < n_sweeps; t0 += kNoAllocChunk) {
    const int m = (int)std::min<uint64_t>(kNoAllocChunk, n_sweeps - t0);
    for (int t = 0; t < m; ++t)
      for (int col = 0; col < 2; ++col) {
        RngKey key;
        key.k0 = (uint32_t)seed;
        key.k1 = (uint32_t)(seed >> 32);
        key.replica = replica;
        key.sweep = (uint32_t)(sweep0 + t0 + t);
        key.ks = make_key_schedule(key.k0, key.k1);
        long long* part = sums_out ? scratch + ((size_t)t * 2 + col) * grid * kNumSums : nullptr;
        const cudaError_t e = launch_ising_sc(a, tab, key, col, VG_PROPOSE_FLIP, true, part, grid, tpb, s);
        if (e != cudaSuccess) return fail(VG_ERR_CUDA, cudaGetErrorString(e));
      }
    if (sums_out) {
      noalloc_finish<<<m, 256, 0, s>>>(scratch, 2 * grid, n_sites, sums_out + t0 * kNumSums);
      const cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) return fail(VG_ERR_CUDA, cudaGetErrorString(e));
    }
  }
  return VG_OK;
}
