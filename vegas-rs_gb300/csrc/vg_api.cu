// vg_api.cu -- the C ABI (include/vegas_gpu.h): contexts, lattice geometry,
// device layouts, the sweep loop and the per-sweep reductions.
//
// Data layout in HBM
//  * sc lattices whose checkerboard is a proper colouring use the STRUCTURED
//    path: two class arrays (sites with (x+y+z)&1 == c), row-major
//    [z][y][x/2]; Ising as uint8 0/1, Heisenberg as three planes (SoA) of
//    FP32 or FP64.  A colour pass reads all of the other class and
//    reads+writes its own: (C+1) x payload bytes per site per sweep.
//  * bcc / fcc Ising lattices with x a multiple of 16, and every bcc / fcc
//    Heisenberg lattice, also use STRUCTURED: one array per basis
//    sublattice (the colour classes), [class][cell] uint8 0/1 for Ising and
//    [class][xyz][cell] planes for Heisenberg, cell = (z ny + y) nx + x.
//  * every other lattice uses the GENERIC path: natural-order spins plus,
//    per colour class of a greedy colouring, the class's site list, an ELL
//    neighbour table [z][n_c] and a lower-colour bit mask.
//  * per-sweep partial sums: one row of 8 values per block per pass, reduced
//    per sweep in a fixed order (deterministic), 8 doubles per sweep.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "vg_heis_common.cuh"

using namespace vg;

struct vg_ctx {
  int device = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  vg_lattice_desc lat{};
  vg_hamiltonian_desc ham{};
  vg_options opt{};
  uint64_t seed = 0;
  uint64_t sweep = 0;
  int64_t n = 0;
  int nb = 1, z = 6, ncol = 2;
  int path = VG_PATH_GENERIC;
  int sm_count = 0, grid = 0, tpb = 256;
  bool all_periodic = false;
  // thermostat
  double T = 2.8;
  double bhat[3] = {0, 0, 1};
  double bmag = 0.0;
  // spins
  void* spin[2][3] = {{nullptr, nullptr, nullptr}, {nullptr, nullptr, nullptr}};
  // tiled path: the second buffer of the class-array pair a sweep writes
  // into, and the tiling of the y-z plane of rows
  uint8_t* tile_buf[2] = {nullptr, nullptr};
  IsingTileArgs tile{};
  int* d_tile_err = nullptr;  // raised by a tiled sweep whose staging wait ran out
  // generic path tables
  std::vector<int64_t> class_size;
  int32_t* d_sites[kMaxColours] = {};
  int32_t* d_nbr[kMaxColours] = {};
  uint32_t* d_low[kMaxColours] = {};
  // staging and reductions
  void* d_stage = nullptr;
  size_t stage_bytes = 0;
  void* d_part = nullptr;
  size_t part_rows = 0;   // rows of kNumSums elements
  double* d_sums = nullptr;
  size_t sums_cap = 0;    // sweeps
  uint64_t last_batch = 0;
  int* d_flag = nullptr;
  double* h_pin = nullptr;  // pinned readback
  size_t h_pin_cap = 0;
  int64_t device_bytes = 0;
  int32_t* d_wnbr = nullptr;             // natural-order neighbour table [n][z] (Wolff, site energies)
  uint8_t* d_wocc = nullptr;             // Wolff: occurrence of each bond among repeated ones
  uint32_t* d_wmark = nullptr;           // Wolff, multi-block: per-site step stamps [n]
  int32_t* d_wq = nullptr;               // Wolff, multi-block: the cluster queue [n]
  WolffGrid* d_wgrid = nullptr;          // Wolff, multi-block: counters and grid barrier
  bool bonds = false;                    // per-bond exchange constants set (generic path)
  std::vector<double> bonds_nat;         // those constants in neighbour-table layout [n][z]
  double* d_jnat = nullptr;              // device copy of bonds_nat (uploaded on first use)
  double* d_eaux = nullptr;              // site-energy buffers: proposals [n][3] + results [n]
  size_t eaux_cap = 0;                   // doubles
  double* d_jb[kMaxColours] = {};        // [z][n_c] per class, FP64
  float* d_jbf[kMaxColours] = {};        // the same in FP32 (FP32 Heisenberg kernels)
  std::string err;
};

namespace {

thread_local std::string g_err;

int fail(vg_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  g_err = msg;
  return code;
}

int cuda_fail(vg_ctx* c, cudaError_t e, const char* what) {
  const int code = e == cudaErrorMemoryAllocation ? VG_ERR_OOM : VG_ERR_CUDA;
  return fail(c, code, std::string(what) + ": " + cudaGetErrorString(e));
}

// Sweeps [c->sweep, c->sweep + n) must have 32-bit indices.
int check_sweeps(vg_ctx* c, uint64_t n) {
  if (sweep_range_ok(c->sweep, n)) return VG_OK;
  return fail(c, VG_ERR_INVALID_ARG, "sweep index " + std::to_string(c->sweep) + " + " + std::to_string(n) +
                                         " sweeps passes 2^32 (the 32-bit sweep word of the Philox counter)");
}

#define VG_CUDA(c, expr)                                    \
  do {                                                      \
    cudaError_t _e = (expr);                                \
    if (_e != cudaSuccess) return cuda_fail((c), _e, #expr); \
  } while (0)

// ------------------------------------------------------------ geometry
// Unit cells of Lattice::sc/bcc/fcc(1.0) in half-cell units and their
// nearest-neighbour vectors; vegas-lattice's expand + drop_x/y/z semantics:
// a bond leaving the box wraps on a periodic axis and is dropped on an open
// one (src/input.rs:296-322).
const int kBasisPos[3][4][3] = {{{0, 0, 0}}, {{0, 0, 0}, {1, 1, 1}}, {{0, 0, 0}, {1, 1, 0}, {1, 0, 1}, {0, 1, 1}}};
const int kBasisN[3] = {1, 2, 4};
const int kCoord[3] = {6, 8, 12};
const int kNNVec[3][12][3] = {
    {{2, 0, 0}, {-2, 0, 0}, {0, 2, 0}, {0, -2, 0}, {0, 0, 2}, {0, 0, -2}},
    {{1, 1, 1}, {-1, 1, 1}, {1, -1, 1}, {-1, -1, 1}, {1, 1, -1}, {-1, 1, -1}, {1, -1, -1}, {-1, -1, -1}},
    {{1, 1, 0}, {-1, 1, 0}, {1, -1, 0}, {-1, -1, 0}, {1, 0, 1}, {-1, 0, 1}, {1, 0, -1}, {-1, 0, -1}, {0, 1, 1},
     {0, -1, 1}, {0, 1, -1}, {0, -1, -1}}};

struct Geometry {
  int cell = 0, nb = 1, z = 6;
  int ext[3] = {1, 1, 1}, per[3] = {1, 1, 1};
  int64_t n = 0;
  int tgt[4][kMaxZ];        // basis index of neighbour k of basis b
  int dcell[4][kMaxZ][3];   // its cell offset
};

int geometry_init(const vg_lattice_desc* d, Geometry* g, std::string* why) {
  if (!d) return (*why = "lattice descriptor is NULL", VG_ERR_INVALID_ARG);
  if (d->cell < 0 || d->cell > 2) return (*why = "unknown unit cell", VG_ERR_INVALID_ARG);
  if (d->nx < 1 || d->ny < 1 || d->nz < 1) return (*why = "lattice extents must be >= 1", VG_ERR_INVALID_ARG);
  g->cell = d->cell;
  g->nb = kBasisN[d->cell];
  g->z = kCoord[d->cell];
  g->ext[0] = d->nx;
  g->ext[1] = d->ny;
  g->ext[2] = d->nz;
  g->per[0] = d->pbc_x != 0;
  g->per[1] = d->pbc_y != 0;
  g->per[2] = d->pbc_z != 0;
  const double nn = (double)d->nx * d->ny * d->nz * g->nb;
  if (nn > 2147483647.0) return (*why = "lattice has more than 2^31-1 sites", VG_ERR_UNSUPPORTED);
  g->n = (int64_t)d->nx * d->ny * d->nz * g->nb;
  if (g->cell == VG_CELL_SC)
    for (int a = 0; a < 3; ++a)
      if (g->per[a] && g->ext[a] == 1)
        return (*why = "a periodic sc axis of extent 1 bonds each site to itself", VG_ERR_UNSUPPORTED);
  for (int b = 0; b < g->nb; ++b)
    for (int k = 0; k < g->z; ++k) {
      int h[3];
      for (int a = 0; a < 3; ++a) {
        const int v = kBasisPos[g->cell][b][a] + kNNVec[g->cell][k][a];
        const int cdel = v >= 0 ? v / 2 : -((1 - v) / 2);
        g->dcell[b][k][a] = cdel;
        h[a] = v - 2 * cdel;
      }
      g->tgt[b][k] = -1;
      for (int q = 0; q < g->nb; ++q)
        if (kBasisPos[g->cell][q][0] == h[0] && kBasisPos[g->cell][q][1] == h[1] && kBasisPos[g->cell][q][2] == h[2])
          g->tgt[b][k] = q;
      if (g->tgt[b][k] < 0) return (*why = "internal: neighbour vector leaves the basis", VG_ERR_INVALID_ARG);
    }
  return VG_OK;
}

int32_t neighbour_of(const Geometry& g, int64_t i, int k) {
  const int b = (int)(i % g.nb);
  int64_t cidx = i / g.nb;
  int c[3];
  c[0] = (int)(cidx % g.ext[0]);
  cidx /= g.ext[0];
  c[1] = (int)(cidx % g.ext[1]);
  c[2] = (int)(cidx / g.ext[1]);
  for (int a = 0; a < 3; ++a) {
    int v = c[a] + g.dcell[b][k][a];
    if (v < 0 || v >= g.ext[a]) {
      if (!g.per[a]) return -1;
      v = ((v % g.ext[a]) + g.ext[a]) % g.ext[a];
    }
    c[a] = v;
  }
  return (int32_t)((((int64_t)c[2] * g.ext[1] + c[1]) * g.ext[0] + c[0]) * g.nb + g.tgt[b][k]);
}

void build_neighbours(const Geometry& g, std::vector<int32_t>& nbr) {
  nbr.resize((size_t)g.n * g.z);
  for (int64_t i = 0; i < g.n; ++i)
    for (int k = 0; k < g.z; ++k) nbr[(size_t)i * g.z + k] = neighbour_of(g, i, k);
}

// Greedy sequential colouring in site order: each site takes the smallest
// colour unused by its already-coloured neighbours.
int greedy_colouring(const Geometry& g, const std::vector<int32_t>& nbr, std::vector<int32_t>& col) {
  col.assign((size_t)g.n, -1);
  int ncol = 0;
  for (int64_t i = 0; i < g.n; ++i) {
    uint64_t used = 0;
    for (int k = 0; k < g.z; ++k) {
      const int32_t j = nbr[(size_t)i * g.z + k];
      if (j >= 0 && j != i && col[j] >= 0) used |= 1ull << col[j];
    }
    int c = 0;
    while ((used >> c) & 1ull) ++c;
    col[i] = c;
    ncol = std::max(ncol, c + 1);
  }
  return ncol;
}

// ------------------------------------------------------------ device helpers
struct ScMap {
  uint32_t Lx, Ly, Hx;
  FastDiv fLx, fLy;
  int nbshift;       // sublattice layout: log2 of the basis size
  long long ncell;   // sublattice layout: entries per class
};

// Layouts of the state (ising_layout): 0 natural order, 1 sc checkerboard
// (two class arrays), 2 bcc / fcc sublattices (one array, class q at
// q ncell for Ising, q 3 ncell for Heisenberg's xyz planes).

__device__ __forceinline__ void sc_locate(long long i, const ScMap& m, int& c, long long& j) {
  const uint32_t ii = (uint32_t)i;
  const uint32_t r = fdiv(ii, m.fLx), x = ii - r * m.Lx;
  const uint32_t zz = fdiv(r, m.fLy), y = r - zz * m.Ly;
  c = (int)((x + y + zz) & 1);
  j = (long long)r * m.Hx + (x >> 1);
}

__device__ __forceinline__ long long ising_offset(long long i, int layout, const ScMap& m, int& c) {
  if (layout == 2) {
    c = 0;
    return (i & ((1ll << m.nbshift) - 1)) * m.ncell + (i >> m.nbshift);
  }
  c = 0;
  if (layout == 0) return i;
  long long j;
  sc_locate(i, m, c, j);
  return j;
}

__global__ void ising_import(const int8_t* __restrict__ src, long long n, int layout, ScMap m, uint8_t* d0,
                             uint8_t* d1, int* flag) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int8_t v = src[i];
    if (v != 1 && v != -1) atomicOr(flag, 1);
    int c;
    const long long j = ising_offset(i, layout, m, c);
    (c ? d1 : d0)[j] = v > 0 ? 1 : 0;
  }
}

__global__ void ising_export(int8_t* __restrict__ dst, long long n, int layout, ScMap m, const uint8_t* d0,
                             const uint8_t* d1) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    int c;
    const long long j = ising_offset(i, layout, m, c);
    dst[i] = (c ? d1 : d0)[j] ? 1 : -1;
  }
}

// State::rand_with_size for Ising (src/state.rs:260-262, :76-84): site i is
// Up iff byte (i & 15) of the block (i >> 4, 0, tag) is < 128 (u < 0.5).
__global__ void ising_init(long long n, int layout, ScMap m, uint8_t* d0, uint8_t* d1, RngKey key) {
  const long long ng = (n + 15) >> 4;
  for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x; g < ng; g += (long long)gridDim.x * blockDim.x) {
    const uint4 b = philox(make_uint4((uint32_t)g, 0u, kTagInitIsing << 24, key.replica), key.k0, key.k1);
    for (int k = 0; k < 16; ++k) {
      const long long i = (g << 4) + k;
      if (i >= n) break;
      int c;
      const long long j = ising_offset(i, layout, m, c);
      (c ? d1 : d0)[j] = blk_byte(b, k) < 128 ? 1 : 0;
    }
  }
}

template <typename R>
struct Planes {
  R* x[2];
  R* y[2];
  R* z[2];
};

// Heisenberg layouts: 0 natural order (three planes), 1 sc checkerboard
// (three planes per class), 2 bcc / fcc sublattices (one array at P.x[0],
// [class][xyz][cell]).
template <typename R>
__device__ __forceinline__ R* heis_at(long long i, int layout, const ScMap& m, const Planes<R>& P, int comp) {
  if (layout == 2) {
    const long long b = i & ((1ll << m.nbshift) - 1), cell = i >> m.nbshift;
    return P.x[0] + (b * 3 + comp) * m.ncell + cell;
  }
  int c = 0;
  long long j = i;
  if (layout == 1) sc_locate(i, m, c, j);
  return (comp == 0 ? P.x[c] : comp == 1 ? P.y[c] : P.z[c]) + j;
}

template <typename R>
__device__ __forceinline__ void heis_put(long long i, int layout, const ScMap& m, const Planes<R>& P, R x, R y,
                                         R z) {
  *heis_at(i, layout, m, P, 0) = x;
  *heis_at(i, layout, m, P, 1) = y;
  *heis_at(i, layout, m, P, 2) = z;
}

template <typename R>
__global__ void heis_import(const double* __restrict__ src, long long n, int layout, ScMap m, Planes<R> P,
                            int* flag) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double x = src[3 * i], y = src[3 * i + 1], z = src[3 * i + 2];
    if (!(fabs(x * x + y * y + z * z - 1.0) < 1e-3)) atomicOr(flag, 1);
    heis_put<R>(i, layout, m, P, (R)x, (R)y, (R)z);
  }
}

template <typename R>
__global__ void heis_export(double* __restrict__ dst, long long n, int layout, ScMap m, Planes<R> P) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
#pragma unroll
    for (int c = 0; c < 3; ++c) dst[3 * i + c] = (double)*heis_at(i, layout, m, P, c);
  }
}

// State::rand_with_size for Heisenberg (heis_init_spin).
template <typename R>
__global__ void heis_init(long long n, int layout, ScMap m, Planes<R> P, RngKey key) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const V3<R> s = heis_init_spin<R>((uint32_t)i, key);
    heis_put<R>(i, layout, m, P, s.x, s.y, s.z);
  }
}

// One block per sweep: rows [sweep][row][kNumSums] -> out[sweep][kNumSums],
// summed in a fixed order with Kahan compensation (deterministic).
template <typename T>
__global__ void reduce_rows(const T* __restrict__ part, long long rows, double* __restrict__ out) {
  constexpr int kLanes = 32;
  __shared__ double s_sum[kNumSums][kLanes];
  const int v = threadIdx.x % kNumSums, lane = threadIdx.x / kNumSums;  // blockDim = 256
  const T* p = part + (long long)blockIdx.x * rows * kNumSums;
  double sum = 0.0, comp = 0.0;
  for (long long r = lane; r < rows; r += kLanes) {
    const double y = (double)p[r * kNumSums + v] - comp;
    const double t = sum + y;
    comp = (t - sum) - y;
    sum = t;
  }
  s_sum[v][lane] = sum;
  __syncthreads();
  if (threadIdx.x < kNumSums) {
    double s = 0.0, cc = 0.0;
    for (int l = 0; l < kLanes; ++l) {
      const double y = s_sum[threadIdx.x][l] - cc;
      const double t = s + y;
      cc = (t - s) - y;
      s = t;
    }
    out[(long long)blockIdx.x * kNumSums + threadIdx.x] = s;
  }
}

// exact int64 lane sums before the conversion to double
template <>
__global__ void reduce_rows<long long>(const long long* __restrict__ part, long long rows, double* __restrict__ out) {
  constexpr int kLanes = 32;
  __shared__ long long s_sum[kNumSums][kLanes];
  const int v = threadIdx.x % kNumSums, lane = threadIdx.x / kNumSums;
  const long long* p = part + (long long)blockIdx.x * rows * kNumSums;
  long long s = 0;
  for (long long r = lane; r < rows; r += kLanes) s += p[r * kNumSums + v];
  s_sum[v][lane] = s;
  __syncthreads();
  if (threadIdx.x < kNumSums) {
    long long t = 0;
    for (int l = 0; l < kLanes; ++l) t += s_sum[threadIdx.x][l];
    out[(long long)blockIdx.x * kNumSums + threadIdx.x] = (double)t;
  }
}

// ------------------------------------------------------------ host helpers
constexpr int kChunk = 64;  // sweeps per reduction launch

bool is_ising(const vg_ctx* c) { return c->opt.spin_kind == VG_SPIN_ISING; }
// the checkerboard class layout (structured grid kernels or the resident kernel)
bool sc_layout(const vg_ctx* c) {
  return (c->path == VG_PATH_STRUCTURED || c->path == VG_PATH_RESIDENT || c->path == VG_PATH_TILED) &&
         c->lat.cell == VG_CELL_SC;
}
// bcc / fcc Ising with one array per sublattice (the structured path of those cells)
bool sub_layout(const vg_ctx* c) { return c->path == VG_PATH_STRUCTURED && c->lat.cell != VG_CELL_SC; }
int ising_layout(const vg_ctx* c) { return sc_layout(c) ? 1 : sub_layout(c) ? 2 : 0; }
// Cells per thread of the sublattice Heisenberg kernel: runs of 4 (vector
// loads, shared index arithmetic) whenever x allows it.  Even a class of
// fewer runs than the grid has resident threads does better so: fcc 64^3
// cells, 65,536 runs per class, 28.6 flips/ns against 19.2 with one cell per
// thread.
int heis_run(const vg_ctx* c) { return c->lat.nx % 4 == 0 ? 4 : 1; }
bool fp64(const vg_ctx* c) { return c->opt.precision == VG_FP64; }
size_t real_size(const vg_ctx* c) { return fp64(c) ? 8 : 4; }

constexpr int64_t kWolffMaxSites = 16384;    // up to here one block holds the Wolff state as bytes and stamps
constexpr int64_t kWolffMidSites = 786432;   // up to here one block holds spins and marks as bits

int dalloc(vg_ctx* c, void** p, size_t bytes) {
  if (bytes == 0) bytes = 16;
  if (c->opt.max_device_bytes > 0 && c->device_bytes + (int64_t)bytes > c->opt.max_device_bytes)
    return fail(c, VG_ERR_OOM, "device memory cap of " + std::to_string(c->opt.max_device_bytes) + " bytes reached");
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) return cuda_fail(c, e, "cudaMalloc");
  c->device_bytes += (int64_t)bytes;
  return VG_OK;
}

ScMap sc_map(const vg_ctx* c) {
  ScMap m;
  m.Lx = (uint32_t)c->lat.nx;
  m.Ly = (uint32_t)c->lat.ny;
  m.Hx = (uint32_t)(c->lat.nx / 2);
  m.fLx = make_fastdiv(m.Lx);
  m.fLy = make_fastdiv(m.Ly);
  m.nbshift = c->lat.cell == VG_CELL_FCC ? 2 : c->lat.cell == VG_CELL_BCC ? 1 : 0;
  m.ncell = (long long)c->lat.nx * c->lat.ny * c->lat.nz;
  return m;
}

IsingSubArgs ising_sub_args(const vg_ctx* c) {
  IsingSubArgs a;
  a.base = (uint8_t*)c->spin[0][0];
  a.nx = c->lat.nx;
  a.ny = c->lat.ny;
  a.nz = c->lat.nz;
  a.ncell = (uint32_t)a.nx * (uint32_t)a.ny * (uint32_t)a.nz;
  a.groups = a.ncell / 16u;
  a.z = c->z;
  a.pbx = c->lat.pbc_x != 0;
  a.pby = c->lat.pbc_y != 0;
  a.pbz = c->lat.pbc_z != 0;
  a.fnx = make_fastdiv((uint32_t)a.nx);
  a.fny = make_fastdiv((uint32_t)a.ny);
  return a;
}

RngKey rng_key(const vg_ctx* c, uint64_t sweep) {
  RngKey k;
  k.k0 = (uint32_t)c->seed;
  k.k1 = (uint32_t)(c->seed >> 32);
  k.replica = c->opt.replica;
  k.sweep = (uint32_t)sweep;
  k.ks = make_key_schedule(k.k0, k.k1);
  return k;
}

int launch_grid(const vg_ctx* c, long long items) {
  const long long want = (items + c->tpb - 1) / c->tpb;
  const long long cap = (long long)c->sm_count * (c->opt.blocks_per_sm > 0 ? c->opt.blocks_per_sm : 8);
  return (int)std::max(1LL, std::min(want, cap));
}

double clamp_temperature(double T) {
  const double eps = 2.220446049250313e-16;  // f64::EPSILON (src/thermostat.rs:29-39)
  return T < eps ? eps : T;
}

double zeeman_coef(const vg_ctx* c) {
  return c->ham.has_zeeman ? c->ham.zeeman_sign * std::fabs(c->bmag) : 0.0;
}

// Ising thresholds: accept iff U < thr (see vg_ising.cu)
IsingTable ising_table(const vg_ctx* c) {
  const double J = c->ham.has_exchange ? c->ham.exchange : 0.0;
  const double o = c->bhat[2] >= 0.0 ? 1.0 : -1.0;  // Field<IsingSpin> orientation Up / Down
  const int ext[3] = {c->lat.nx, c->lat.ny, c->lat.nz};
  const int per[3] = {c->lat.pbc_x, c->lat.pbc_y, c->lat.pbc_z};
  return make_ising_table(J, zeeman_coef(c) * o, clamp_temperature(c->T), c->z, sc_layout(c), ext, per);
}

template <typename R>
HeisParams<R> heis_params(const vg_ctx* c) {
  HeisParams<R> p;
  const double T = clamp_temperature(c->T);
  // per-bond constants carry the exchange in the neighbour field
  p.J = (R)(c->ham.has_exchange ? (c->bonds ? 1.0 : c->ham.exchange) : 0.0);
  p.K = (R)(c->ham.has_anisotropy ? c->ham.anisotropy : 0.0);
  p.ax = (R)c->ham.anisotropy_axis[0];
  p.ay = (R)c->ham.anisotropy_axis[1];
  p.az = (R)c->ham.anisotropy_axis[2];
  p.hz = (R)zeeman_coef(c);
  p.bx = (R)c->bhat[0];
  p.by = (R)c->bhat[1];
  p.bz = (R)c->bhat[2];
  p.Kc = (R)(c->ham.has_cubic ? c->ham.cubic : 0.0);
  p.beta = (R)(1.0 / T);
  p.T = (R)T;
  return p;
}

int ensure_part(vg_ctx* c, size_t rows) {
  if (rows <= c->part_rows) return VG_OK;
  if (c->d_part) {
    cudaFree(c->d_part);
    c->device_bytes -= (int64_t)(c->part_rows * kNumSums * 8);
    c->d_part = nullptr;
  }
  int rc = dalloc(c, &c->d_part, rows * kNumSums * 8);
  if (rc) return rc;
  c->part_rows = rows;
  return VG_OK;
}

int ensure_sums(vg_ctx* c, size_t sweeps) {
  if (sweeps <= c->sums_cap) return VG_OK;
  if (c->d_sums) {
    cudaFree(c->d_sums);
    c->device_bytes -= (int64_t)(c->sums_cap * kNumSums * 8);
    c->d_sums = nullptr;
  }
  int rc = dalloc(c, (void**)&c->d_sums, sweeps * kNumSums * 8);
  if (rc) return rc;
  c->sums_cap = sweeps;
  return VG_OK;
}

int ensure_pinned(vg_ctx* c, size_t doubles) {
  if (doubles <= c->h_pin_cap) return VG_OK;
  if (c->h_pin) cudaFreeHost(c->h_pin);
  c->h_pin = nullptr;
  VG_CUDA(c, cudaMallocHost((void**)&c->h_pin, doubles * 8));
  c->h_pin_cap = doubles;
  return VG_OK;
}

IsingScArgs ising_sc_args(const vg_ctx* c) {
  IsingScArgs a;
  a.cls[0] = (uint8_t*)c->spin[0][0];
  a.cls[1] = (uint8_t*)c->spin[1][0];
  a.Hx = c->lat.nx / 2;
  a.Ly = c->lat.ny;
  a.Lz = c->lat.nz;
  a.G = a.Hx / kIsingGroup;
  a.groups = (uint32_t)a.G * (uint32_t)a.Ly * (uint32_t)a.Lz;
  a.pbx = c->lat.pbc_x != 0;
  a.pby = c->lat.pbc_y != 0;
  a.pbz = c->lat.pbc_z != 0;
  a.fG = make_fastdiv((uint32_t)a.G);
  a.fLy = make_fastdiv((uint32_t)a.Ly);
  set_sc_offsets(a);
  return a;
}

// One colour pass.  part_row: first partial row of this pass (or null).
int launch_pass(vg_ctx* c, int colour, bool update, uint64_t sweep, void* part_row) {
  const RngKey key = rng_key(c, sweep);
  cudaError_t e = cudaSuccess;
  if (is_ising(c)) {
    const IsingTable tab = ising_table(c);
    long long* part = (long long*)part_row;
    if (sc_layout(c)) {
      e = launch_ising_sc(ising_sc_args(c), tab, key, colour, c->opt.proposal, update, part, c->grid, c->tpb,
                          c->stream);
    } else if (sub_layout(c)) {
      e = launch_ising_sub(ising_sub_args(c), c->ncol, tab, key, colour, c->opt.proposal, update, part, c->grid,
                           c->tpb, c->stream);
    } else {
      IsingGenArgs a;
      a.spin = (uint8_t*)c->spin[0][0];
      a.sites = c->d_sites[colour];
      a.nbr = c->d_nbr[colour];
      a.lowmask = c->d_low[colour];
      a.n_c = c->class_size[colour];
      a.z = c->z;
      a.jb = c->bonds ? c->d_jb[colour] : nullptr;
      a.hz = zeeman_coef(c) * (c->bhat[2] >= 0.0 ? 1.0 : -1.0);
      a.T = clamp_temperature(c->T);
      e = launch_ising_gen(a, tab, key, colour, c->opt.proposal, update, part, c->grid, c->tpb, c->stream);
    }
  } else {
    double* part = (double*)part_row;
    auto run = [&](auto zero) -> cudaError_t {
      using R = decltype(zero);
      const HeisParams<R> P = heis_params<R>(c);
      if (sc_layout(c)) {
        HeisScArgs<R> a;
        for (int k = 0; k < 2; ++k) {
          a.x[k] = (R*)c->spin[k][0];
          a.y[k] = (R*)c->spin[k][1];
          a.z[k] = (R*)c->spin[k][2];
        }
        a.Hx = c->lat.nx / 2;
        a.Ly = c->lat.ny;
        a.Lz = c->lat.nz;
        a.n_c = (uint32_t)a.Hx * (uint32_t)a.Ly * (uint32_t)a.Lz;
        a.pbx = c->lat.pbc_x != 0;
        a.pby = c->lat.pbc_y != 0;
        a.pbz = c->lat.pbc_z != 0;
        a.fHx = make_fastdiv((uint32_t)a.Hx);
        a.fLy = make_fastdiv((uint32_t)a.Ly);
        return launch_heis_sc<R>(a, P, key, colour, c->opt.proposal, update, part, c->grid, c->tpb, c->stream);
      }
      if (sub_layout(c)) {
        HeisSubArgs<R> a;
        const int W = heis_run(c);
        a.spin = (R*)c->spin[0][0];
        a.nx = c->lat.nx;
        a.ny = c->lat.ny;
        a.nz = c->lat.nz;
        a.ncell = (uint32_t)a.nx * (uint32_t)a.ny * (uint32_t)a.nz;
        a.pbx = c->lat.pbc_x != 0;
        a.pby = c->lat.pbc_y != 0;
        a.pbz = c->lat.pbc_z != 0;
        a.rpr = a.nx / W;
        a.runs = a.ncell / (uint32_t)W;
        a.frow = make_fastdiv((uint32_t)a.rpr);
        a.fny = make_fastdiv((uint32_t)a.ny);
        return launch_heis_sub<R>(a, c->ncol, W, P, key, colour, c->opt.proposal, update, part, c->grid, c->tpb,
                                  c->stream);
      }
      HeisGenArgs<R> a;
      a.x = (R*)c->spin[0][0];
      a.y = (R*)c->spin[0][1];
      a.z = (R*)c->spin[0][2];
      a.sites = c->d_sites[colour];
      a.nbr = c->d_nbr[colour];
      a.lowmask = c->d_low[colour];
      a.n_c = c->class_size[colour];
      a.zc = c->z;
      a.jb = nullptr;
      if (c->bonds) a.jb = sizeof(R) == 8 ? (const R*)c->d_jb[colour] : (const R*)c->d_jbf[colour];
      return launch_heis_gen<R>(a, P, key, colour, c->opt.proposal, update, part, c->grid, c->tpb, c->stream);
    };
    e = fp64(c) ? run(0.0) : run(0.0f);
  }
  if (e != cudaSuccess) return cuda_fail(c, e, "kernel launch");
  return VG_OK;
}

size_t rows_per_sweep(const vg_ctx* c) { return (size_t)c->ncol * (size_t)c->grid; }
// blocks (one partial row each) of a tiled sweep; 0 off the tiled path
int tile_count(const vg_ctx* c) { return c->path == VG_PATH_TILED ? c->tile.nyt * c->tile.nzt : 0; }

int launch_reduce(vg_ctx* c, int sweeps, double* out, long long rows) {
  if (is_ising(c) && !c->bonds)
    reduce_rows<long long><<<sweeps, 256, 0, c->stream>>>((const long long*)c->d_part, rows, out);
  else
    reduce_rows<double><<<sweeps, 256, 0, c->stream>>>((const double*)c->d_part, rows, out);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(c, e, "reduce launch");
  return VG_OK;
}

// Enqueue n sweeps; with measure, per-sweep raw sums land in d_sums[0..n).
int enqueue(vg_ctx* c, uint64_t n, bool measure) {
  int rc;
  if ((rc = check_sweeps(c, n))) return rc;
  if (c->path == VG_PATH_RESIDENT) {  // all n sweeps in one launch
    if (measure && (rc = ensure_sums(c, (size_t)std::max<uint64_t>(n, 1)))) return rc;
    const IsingScArgs a = ising_sc_args(c);
    const int tpb = (int)std::min<long long>(1024, ((long long)a.groups * 16 + 31) / 32 * 32);
    for (uint64_t t0 = 0; t0 < n; t0 += (1u << 30)) {
      const uint32_t m = (uint32_t)std::min<uint64_t>(n - t0, 1u << 30);
      const cudaError_t e = launch_ising_resident(a, ising_table(c), rng_key(c, c->sweep + t0), c->opt.proposal, m,
                                                  measure ? c->d_sums + t0 * kNumSums : nullptr, tpb, c->stream);
      if (e != cudaSuccess) return cuda_fail(c, e, "resident kernel launch");
    }
    c->sweep += n;
    if (measure) c->last_batch = n;
    return VG_OK;
  }
  if (measure) {
    if ((rc = ensure_sums(c, (size_t)std::max<uint64_t>(n, 1)))) return rc;
    if ((rc = ensure_part(c, std::max<size_t>(rows_per_sweep(c), (size_t)tile_count(c)) * kChunk))) return rc;
  }
  uint64_t done = 0;
  if (c->path == VG_PATH_TILED) {
    // whole sweeps, one launch each, alternating between the class arrays
    // and the second buffer: an even count ends in the class arrays; an odd
    // last sweep runs as two colour passes in place (identical draws)
    const uint64_t even = n & ~1ull;
    const IsingTable tab = ising_table(c);
    const size_t rows = (size_t)tile_count(c);
    for (uint64_t t0 = 0; t0 < even; t0 += kChunk) {
      const int m = (int)std::min<uint64_t>(kChunk, even - t0);
      for (int t = 0; t < m; ++t) {
        IsingTileArgs a = c->tile;
        uint8_t* base[2] = {(uint8_t*)c->spin[0][0], (uint8_t*)c->spin[1][0]};
        const bool odd = ((t0 + (uint64_t)t) & 1ull) != 0;
        for (int k = 0; k < 2; ++k) {
          a.in[k] = odd ? c->tile_buf[k] : base[k];
          a.out[k] = odd ? base[k] : c->tile_buf[k];
        }
        long long* part = measure ? (long long*)c->d_part + (size_t)t * rows * kNumSums : nullptr;
        const cudaError_t e = launch_ising_tile_sweep(a, tab, rng_key(c, c->sweep + t0 + t), c->opt.proposal, part,
                                                      c->stream);
        if (e != cudaSuccess) return cuda_fail(c, e, "tiled sweep launch");
      }
      if (measure && (rc = launch_reduce(c, m, c->d_sums + t0 * kNumSums, (long long)rows))) return rc;
    }
    done = even;
  }
  const size_t rps = rows_per_sweep(c);
  for (uint64_t t0 = done; t0 < n; t0 += kChunk) {
    const int m = (int)std::min<uint64_t>(kChunk, n - t0);
    for (int t = 0; t < m; ++t) {
      for (int col = 0; col < c->ncol; ++col) {
        char* row = nullptr;
        if (measure) row = (char*)c->d_part + ((size_t)t * rps + (size_t)col * c->grid) * kNumSums * 8;
        if ((rc = launch_pass(c, col, true, c->sweep + t0 + t, row))) return rc;
      }
    }
    if (measure && (rc = launch_reduce(c, m, c->d_sums + t0 * kNumSums, (long long)rps))) return rc;
  }
  c->sweep += n;
  if (measure) c->last_batch = n;
  return VG_OK;
}

// raw device row -> vg_sums with the spin kind's meaning
void finish_sums(const vg_ctx* c, const double* raw, vg_sums* s) {
  if (is_ising(c)) {
    const double N = (double)c->n;
    const double mz = 2.0 * raw[6] - N;
    const double o = c->bhat[2] >= 0.0 ? 1.0 : -1.0;
    const double ao = c->ham.anisotropy_axis[2] >= 0.0 ? 1.0 : -1.0;
    (void)ao;
    s->bond = raw[0];
    s->anisotropy = N;  // (s.e)^2 = 1 for Ising spins
    s->zeeman = mz * o;
    s->cubic = N;
    s->mx = 0.0;
    s->my = 0.0;
    s->mz = mz;
    s->accepted = raw[7];
  } else {
    s->bond = raw[0];
    s->anisotropy = raw[1];
    s->zeeman = raw[2];
    s->cubic = raw[3];
    s->mx = raw[4];
    s->my = raw[5];
    s->mz = raw[6];
    s->accepted = raw[7];
  }
}

// Totals with the reference's semantics (see vegas_gpu.h).
void energy_of(const vg_ctx* c, const vg_sums* s, double* E, double* M) {
  const vg_hamiltonian_desc& h = c->ham;
  const double N = (double)c->n;
  const double B = std::fabs(c->bmag);
  double e = 0.0;
  const double J = c->bonds ? 1.0 : h.exchange;  // per-bond constants are inside the bond sum
  if (h.compound) {
    if (h.has_exchange) e += -2.0 * J * s->bond;
    if (h.has_anisotropy) e += h.anisotropy * s->anisotropy;
    if (h.has_zeeman) e += h.zeeman_sign * B * s->zeeman;
    if (h.has_gauge) e += N * h.gauge;
    if (h.has_cubic) e += -h.cubic * s->cubic;
  } else if (h.has_exchange) {
    e = -J * s->bond;
  } else if (h.has_anisotropy) {
    e = s->anisotropy;
  } else if (h.has_zeeman) {
    e = -B * s->zeeman;
  } else if (h.has_gauge) {
    e = N * h.gauge;
  } else if (h.has_cubic) {
    e = -h.cubic * s->cubic;
  }
  if (E) *E = e;
  if (M) {
    if (is_ising(c)) {
      *M = std::fabs(s->mz);
    } else {
      const double m = std::sqrt(s->mx * s->mx + s->my * s->my + s->mz * s->mz);
      *M = std::fabs(m) < 2.220446049250313e-16 ? 0.0 : m;
    }
  }
}

int sync_stream(vg_ctx* c) {
  VG_CUDA(c, cudaStreamSynchronize(c->stream));
  if (c->d_tile_err) {  // a tiled sweep that gave up writes nothing: the state is not to be trusted
    int flag = 0;
    VG_CUDA(c, cudaMemcpy(&flag, c->d_tile_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (flag) {
      VG_CUDA(c, cudaMemset(c->d_tile_err, 0, sizeof(int)));
      return fail(c, VG_ERR_TIMEOUT, "a tiled sweep's wait for its staged rows ran out; the state is undefined");
    }
  }
  return VG_OK;
}

int read_raw(vg_ctx* c, uint64_t count, double** host) {
  int rc;
  if ((rc = ensure_pinned(c, (size_t)count * kNumSums))) return rc;
  if (count) VG_CUDA(c, cudaMemcpyAsync(c->h_pin, c->d_sums, count * kNumSums * 8, cudaMemcpyDeviceToHost, c->stream));
  if ((rc = sync_stream(c))) return rc;
  *host = c->h_pin;
  return VG_OK;
}

int validate_ham(const vg_hamiltonian_desc* h, std::string* why) {
  if (!h) return (*why = "hamiltonian descriptor is NULL", VG_ERR_INVALID_ARG);
  const int terms = (h->has_exchange != 0) + (h->has_anisotropy != 0) + (h->has_zeeman != 0) + (h->has_gauge != 0) +
                    (h->has_cubic != 0);
  if (terms == 0) return (*why = "hamiltonian has no terms", VG_ERR_INVALID_ARG);
  if (!h->compound && terms != 1)
    return (*why = "a non-compound hamiltonian must have exactly one term", VG_ERR_INVALID_ARG);
  const double vals[] = {h->exchange, h->anisotropy, h->anisotropy_axis[0], h->anisotropy_axis[1],
                         h->anisotropy_axis[2], h->zeeman_sign, h->gauge, h->cubic};
  for (double v : vals)
    if (!std::isfinite(v)) return (*why = "hamiltonian coefficients must be finite", VG_ERR_INVALID_ARG);
  return VG_OK;
}

int setup_generic(vg_ctx* c, const Geometry& g) {
  // the kernels index a class's neighbour table [z][n_c] with 32-bit offsets
  if ((int64_t)g.z * g.n >= (int64_t)UINT32_MAX)
    return fail(c, VG_ERR_UNSUPPORTED, "the generic path needs n_sites x coordination < 2^32");
  std::vector<int32_t> nbr, col;
  build_neighbours(g, nbr);
  c->ncol = greedy_colouring(g, nbr, col);
  if (c->ncol > kMaxColours) return fail(c, VG_ERR_UNSUPPORTED, "greedy colouring needs too many colours");
  c->class_size.assign(c->ncol, 0);
  std::vector<std::vector<int32_t>> sites(c->ncol);
  for (int64_t i = 0; i < g.n; ++i) sites[col[i]].push_back((int32_t)i);
  for (int k = 0; k < c->ncol; ++k) {
    const int64_t nc = (int64_t)sites[k].size();
    c->class_size[k] = nc;
    std::vector<int32_t> ell((size_t)g.z * nc);
    std::vector<uint32_t> low((size_t)nc, 0u);
    for (int64_t j = 0; j < nc; ++j) {
      const int32_t i = sites[k][j];
      for (int q = 0; q < g.z; ++q) {
        const int32_t t = nbr[(size_t)i * g.z + q];
        ell[(size_t)q * nc + j] = t;
        if (t >= 0 && col[t] < k) low[j] |= 1u << q;
        if (t >= 0 && col[t] == k && t != i) return fail(c, VG_ERR_INVALID_ARG, "internal: improper colouring");
      }
    }
    int rc;
    if ((rc = dalloc(c, (void**)&c->d_sites[k], sizeof(int32_t) * nc))) return rc;
    if ((rc = dalloc(c, (void**)&c->d_nbr[k], sizeof(int32_t) * ell.size()))) return rc;
    if ((rc = dalloc(c, (void**)&c->d_low[k], sizeof(uint32_t) * nc))) return rc;
    VG_CUDA(c, cudaMemcpy(c->d_sites[k], sites[k].data(), sizeof(int32_t) * nc, cudaMemcpyHostToDevice));
    VG_CUDA(c, cudaMemcpy(c->d_nbr[k], ell.data(), sizeof(int32_t) * ell.size(), cudaMemcpyHostToDevice));
    VG_CUDA(c, cudaMemcpy(c->d_low[k], low.data(), sizeof(uint32_t) * nc, cudaMemcpyHostToDevice));
  }
  return VG_OK;
}

void destroy(vg_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  for (int k = 0; k < 2; ++k)
    for (int a = 0; a < 3; ++a)
      if (c->spin[k][a]) cudaFree(c->spin[k][a]);
  for (int k = 0; k < 2; ++k)
    if (c->tile_buf[k]) cudaFree(c->tile_buf[k]);
  if (c->d_tile_err) cudaFree(c->d_tile_err);
  for (int k = 0; k < kMaxColours; ++k) {
    if (c->d_sites[k]) cudaFree(c->d_sites[k]);
    if (c->d_nbr[k]) cudaFree(c->d_nbr[k]);
    if (c->d_low[k]) cudaFree(c->d_low[k]);
    if (c->d_jb[k]) cudaFree(c->d_jb[k]);
    if (c->d_jbf[k]) cudaFree(c->d_jbf[k]);
  }
  if (c->d_stage) cudaFree(c->d_stage);
  if (c->d_wnbr) cudaFree(c->d_wnbr);
  if (c->d_wocc) cudaFree(c->d_wocc);
  if (c->d_wmark) cudaFree(c->d_wmark);
  if (c->d_wq) cudaFree(c->d_wq);
  if (c->d_wgrid) cudaFree(c->d_wgrid);
  if (c->d_jnat) cudaFree(c->d_jnat);
  if (c->d_eaux) cudaFree(c->d_eaux);
  if (c->d_part) cudaFree(c->d_part);
  if (c->d_sums) cudaFree(c->d_sums);
  if (c->d_flag) cudaFree(c->d_flag);
  if (c->h_pin) cudaFreeHost(c->h_pin);
  if (c->own_stream) cudaStreamDestroy(c->own_stream);
  delete c;
}

int ensure_stage(vg_ctx* c, size_t bytes) {
  if (bytes <= c->stage_bytes) return VG_OK;
  if (c->d_stage) {
    cudaFree(c->d_stage);
    c->device_bytes -= (int64_t)c->stage_bytes;
    c->d_stage = nullptr;
  }
  int rc = dalloc(c, &c->d_stage, bytes);
  if (rc) return rc;
  c->stage_bytes = bytes;
  return VG_OK;
}

int copy_grid(const vg_ctx* c, long long n) {
  return (int)std::max(1LL, std::min((n + 255) / 256, (long long)c->sm_count * 8));
}

}  // namespace

// ===================================================================== ABI
extern "C" {

const char* vg_status_string(int s) {
  switch (s) {
    case VG_OK: return "ok";
    case VG_ERR_INVALID_ARG: return "invalid argument";
    case VG_ERR_CUDA: return "CUDA error";
    case VG_ERR_TIMEOUT: return "timeout";
    case VG_ERR_OOM: return "out of device memory";
    case VG_ERR_UNSUPPORTED: return "unsupported configuration";
    case VG_ERR_NO_DEVICE: return "no CUDA device";
    default: return "unknown status";
  }
}

int vg_abi_version(void) { return VG_ABI_VERSION; }

int vg_device_count(int32_t* count) {
  if (!count) return VG_ERR_INVALID_ARG;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  *count = e == cudaSuccess ? n : 0;
  return e == cudaSuccess ? VG_OK : fail(nullptr, VG_ERR_NO_DEVICE, cudaGetErrorString(e));
}

int vg_device_name(int32_t device, char* name, int32_t capacity) {
  if (!name || capacity < 1) return VG_ERR_INVALID_ARG;
  name[0] = '\0';
  cudaDeviceProp prop;
  const cudaError_t e = cudaGetDeviceProperties(&prop, device);
  if (e != cudaSuccess) return fail(nullptr, VG_ERR_NO_DEVICE, cudaGetErrorString(e));
  std::strncpy(name, prop.name, (size_t)capacity - 1);
  name[capacity - 1] = '\0';
  return VG_OK;
}

int vg_options_default(int32_t spin_kind, vg_options* o) {
  if (!o || (spin_kind != VG_SPIN_ISING && spin_kind != VG_SPIN_HEISENBERG)) return VG_ERR_INVALID_ARG;
  std::memset(o, 0, sizeof(*o));
  o->spin_kind = spin_kind;
  o->proposal = spin_kind == VG_SPIN_ISING ? VG_PROPOSE_FLIP : VG_PROPOSE_RANDOM;
  o->path = VG_PATH_AUTO;
  o->precision = VG_FP32;
  o->device = -1;
  return VG_OK;
}

int vg_ctx_create(const vg_lattice_desc* lat, const vg_hamiltonian_desc* ham, int32_t spin_kind, uint64_t seed,
                  vg_ctx** out) {
  vg_options o;
  if (vg_options_default(spin_kind, &o)) return fail(nullptr, VG_ERR_INVALID_ARG, "unknown spin kind");
  return vg_ctx_create_ex(lat, ham, &o, seed, out);
}

int vg_ctx_create_ex(const vg_lattice_desc* lat, const vg_hamiltonian_desc* ham, const vg_options* opt,
                     uint64_t seed, vg_ctx** out) {
  if (!out || !opt) return fail(nullptr, VG_ERR_INVALID_ARG, "NULL argument");
  *out = nullptr;
  std::string why;
  Geometry g;
  int rc = geometry_init(lat, &g, &why);
  if (rc) return fail(nullptr, rc, why);
  if ((rc = validate_ham(ham, &why))) return fail(nullptr, rc, why);
  if (opt->spin_kind != VG_SPIN_ISING && opt->spin_kind != VG_SPIN_HEISENBERG)
    return fail(nullptr, VG_ERR_INVALID_ARG, "unknown spin kind");
  if (opt->proposal != VG_PROPOSE_FLIP && opt->proposal != VG_PROPOSE_RANDOM)
    return fail(nullptr, VG_ERR_INVALID_ARG, "unknown proposal");
  if (opt->precision != VG_FP32 && opt->precision != VG_FP64)
    return fail(nullptr, VG_ERR_INVALID_ARG, "unknown precision");
  if (opt->path < VG_PATH_AUTO || opt->path > VG_PATH_TILED) return fail(nullptr, VG_ERR_INVALID_ARG, "unknown path");
  if (opt->threads_per_block && (opt->threads_per_block % 32 || opt->threads_per_block > 256 ||
                                 opt->threads_per_block < 32))
    return fail(nullptr, VG_ERR_INVALID_ARG, "threads_per_block must be a multiple of 32 in [32, 256]");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    return fail(nullptr, VG_ERR_NO_DEVICE, "no CUDA device is visible");

  vg_ctx* c = new (std::nothrow) vg_ctx();
  if (!c) return fail(nullptr, VG_ERR_OOM, "host allocation failed");
  c->lat = *lat;
  c->ham = *ham;
  c->opt = *opt;
  c->seed = seed;
  c->n = g.n;
  c->nb = g.nb;
  c->z = g.z;
  c->all_periodic = lat->pbc_x && lat->pbc_y && lat->pbc_z;
  if (opt->device >= 0) {
    if (opt->device >= ndev) {
      delete c;
      return fail(nullptr, VG_ERR_INVALID_ARG, "device index out of range");
    }
    c->device = opt->device;
  } else {
    cudaGetDevice(&c->device);
  }
  cudaError_t e = cudaSetDevice(c->device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, c->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    int r = cuda_fail(nullptr, e, "device setup");
    destroy(c);
    return r;
  }
  c->stream = c->own_stream;
  c->tpb = opt->threads_per_block ? opt->threads_per_block : 256;

  // Kernel family: the checkerboard layout needs an sc lattice with even
  // x extent and even extents on every periodic axis (so that the
  // checkerboard is the greedy colouring); Ising also needs x/2 to be a
  // multiple of 16 (one uint4 per 16-site group).
  const bool sc_ok = g.cell == VG_CELL_SC && g.n / 2 <= (int64_t)INT32_MAX && lat->nx % 2 == 0 &&
                     (!lat->pbc_y || lat->ny % 2 == 0) &&
                     (!lat->pbc_z || lat->nz % 2 == 0) &&
                     (opt->spin_kind != VG_SPIN_ISING || (lat->nx / 2) % kIsingGroup == 0);
  // bcc / fcc: one array per sublattice; Ising in runs of 16 cells along x
  // (x a multiple of 16), Heisenberg in runs of 4 (x a multiple of 4) or 1,
  // with 32-bit offsets over the [class][xyz][cell] planes
  const bool bf = g.cell == VG_CELL_BCC || g.cell == VG_CELL_FCC;
  const bool sub_ok = bf && (opt->spin_kind == VG_SPIN_ISING ? lat->nx % kIsingGroup == 0 && g.n <= (int64_t)INT32_MAX
                                                             : 3 * g.n <= (int64_t)UINT32_MAX);
  if (opt->path == VG_PATH_STRUCTURED && !sc_ok && !sub_ok) {
    destroy(c);
    return fail(nullptr, VG_ERR_UNSUPPORTED,
                "lattice does not admit a structured path (sc checkerboard, bcc / fcc Ising with x a multiple of "
                "16, or bcc / fcc Heisenberg)");
  }
  const bool res_ok = sc_ok && opt->spin_kind == VG_SPIN_ISING && g.n <= 65536;
  if (opt->path == VG_PATH_RESIDENT && !res_ok) {
    destroy(c);
    return fail(nullptr, VG_ERR_UNSUPPORTED, "the resident path needs an Ising lattice of at most 65536 sites "
                                             "that admits the checkerboard layout");
  }
  // the tiled sweep kernel: Ising on a fully periodic checkerboard lattice
  // whose rows fit a tiling of shared memory
  IsingTileArgs plan{};
  const bool tile_ok = sc_ok && opt->spin_kind == VG_SPIN_ISING && lat->pbc_x && lat->pbc_y && lat->pbc_z &&
                       lat->ny >= 4 && lat->nz >= 4 &&
                       ising_tile_plan(lat->nx / 2, lat->ny, lat->nz, c->sm_count, &plan);
  if (opt->path == VG_PATH_TILED && !tile_ok) {
    destroy(c);
    return fail(nullptr, VG_ERR_UNSUPPORTED, "the tiled path needs an Ising sc lattice, periodic on every axis, with "
                                             "x a multiple of 64, even y and z of at least 4");
  }
  // AUTO does not take it: on the GB300 it ran slower than the two-pass
  // kernels at every size measured (sc 128^3 - 512^3; 256^3: 727-739
  // against 792 flips/ns)
  if (opt->path == VG_PATH_GENERIC || !(sc_ok || sub_ok)) c->path = VG_PATH_GENERIC;
  else if (opt->path == VG_PATH_RESIDENT || (opt->path == VG_PATH_AUTO && res_ok && g.n <= 8192)) c->path = VG_PATH_RESIDENT;
  else if (opt->path == VG_PATH_TILED) c->path = VG_PATH_TILED;
  else c->path = VG_PATH_STRUCTURED;
  if (c->path == VG_PATH_TILED) {
    plan.Hx = lat->nx / 2;
    plan.Ly = lat->ny;
    plan.Lz = lat->nz;
    plan.G = plan.Hx / kIsingGroup;
    if ((rc = dalloc(c, (void**)&c->d_tile_err, sizeof(int))) ||
        (e = cudaMemsetAsync(c->d_tile_err, 0, sizeof(int), c->stream)) != cudaSuccess) {
      if (!rc) rc = cuda_fail(nullptr, e, "tiled path set-up");
      g_err = c->err.empty() ? g_err : c->err;
      destroy(c);
      return rc;
    }
    plan.err = c->d_tile_err;
    c->tile = plan;
    e = ising_tile_prepare();
    if (e != cudaSuccess) {
      int r = cuda_fail(nullptr, e, "tiled sweep kernel set-up");
      destroy(c);
      return r;
    }
    for (int k = 0; k < 2 && !rc; ++k) rc = dalloc(c, (void**)&c->tile_buf[k], (size_t)(g.n / 2));
    if (rc) {
      g_err = c->err;
      destroy(c);
      return rc;
    }
  }

  if (sc_layout(c)) {
    c->ncol = 2;
    c->class_size.assign(2, g.n / 2);
    const size_t per = (size_t)(g.n / 2);
    for (int k = 0; k < 2; ++k) {
      if (is_ising(c)) {
        rc = dalloc(c, &c->spin[k][0], per);
      } else {
        for (int a = 0; a < 3 && !rc; ++a) rc = dalloc(c, &c->spin[k][a], per * real_size(c));
      }
      if (rc) {
        destroy(c);
        return rc;
      }
    }
  } else if (sub_layout(c)) {
    c->ncol = g.nb;
    c->class_size.assign(g.nb, g.n / g.nb);
    if ((rc = dalloc(c, &c->spin[0][0], (size_t)g.n * (is_ising(c) ? 1 : 3 * real_size(c))))) {
      destroy(c);
      return rc;
    }
  } else {
    rc = setup_generic(c, g);
    if (!rc) {
      if (is_ising(c)) {
        rc = dalloc(c, &c->spin[0][0], (size_t)g.n);
      } else {
        for (int a = 0; a < 3 && !rc; ++a) rc = dalloc(c, &c->spin[0][a], (size_t)g.n * real_size(c));
      }
    }
    if (rc) {
      g_err = c->err;
      destroy(c);
      return rc;
    }
  }
  long long items = 0;
  for (int k = 0; k < c->ncol; ++k) {
    const long long nc = c->class_size[k];
    // the structured Ising kernels take 16-site groups, the sublattice
    // Heisenberg kernel runs of heis_run(c) cells, every other kernel one entry per thread
    items = std::max(items, is_ising(c) && (sc_layout(c) || sub_layout(c)) ? (nc + 15) / 16
                            : sub_layout(c)                                 ? nc / heis_run(c)
                                                                            : nc);
  }
  // sublattice Ising classes too small for one 256-thread block per SM run
  // 128-thread blocks, twice as many (fcc 64^3 cells: 68.4 -> 73.9 flips/ns,
  // bcc 64^3 unchanged; larger classes ran slower so)
  if (is_ising(c) && sub_layout(c) && opt->threads_per_block == 0 && (items + 255) / 256 < c->sm_count) c->tpb = 128;
  c->grid = launch_grid(c, items);
  if (!sc_layout(c) && !sub_layout(c) && opt->blocks_per_sm <= 0) {
    // neighbour-table kernels: one wave of four blocks per SM, each thread
    // taking several entries (fcc 64^3 Ising 24.4 -> 36.8 flips/ns, bcc
    // 128^3 Heisenberg 28.1 -> 30.0 against two waves of eight per SM)
    c->grid = (int)std::min<long long>(c->grid, (long long)c->sm_count * 4);
  }
  if (is_ising(c) && sc_layout(c) && opt->blocks_per_sm <= 0) {
    // one wave of resident blocks, each thread walking several 16-site groups
    const long long cap = (long long)c->sm_count * ising_sc_blocks_per_sm(ising_sc_args(c), ising_table(c), c->tpb);
    c->grid = (int)std::max(1LL, std::min((items + c->tpb - 1) / c->tpb, cap));
  }
  if ((rc = dalloc(c, (void**)&c->d_flag, sizeof(int)))) {
    destroy(c);
    return rc;
  }
  // State::up_with_size until the caller sets or randomises the state
  if (is_ising(c)) {
    for (int k = 0; k < 2; ++k)
      if (c->spin[k][0])
        cudaMemsetAsync(c->spin[k][0], 1, sc_layout(c) ? (size_t)(g.n / 2) : (size_t)g.n, c->stream);
  } else {
    for (int k = 0; k < 2; ++k)
      for (int a = 0; a < 3; ++a)
        if (c->spin[k][a])
          cudaMemsetAsync(c->spin[k][a], 0,
                          (sc_layout(c) ? (size_t)(g.n / 2) : sub_layout(c) ? 3 * (size_t)g.n : (size_t)g.n) *
                              real_size(c),
                          c->stream);
  }
  e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) {
    int r = cuda_fail(nullptr, e, "initial state");
    destroy(c);
    return r;
  }
  if (!is_ising(c)) {
    // Heisenberg up state: set via the import path
    std::vector<double> up((size_t)g.n * 3, 0.0);
    for (int64_t i = 0; i < g.n; ++i) up[3 * i + 2] = 1.0;
    rc = vg_set_state(c, up.data(), g.n);
    if (rc) {
      g_err = c->err;
      destroy(c);
      return rc;
    }
  }
  *out = c;
  return VG_OK;
}

int vg_ctx_destroy(vg_ctx* c) {
  if (!c) return VG_ERR_INVALID_ARG;
  destroy(c);
  return VG_OK;
}

int vg_ctx_info(const vg_ctx* c, vg_info* o) {
  if (!c || !o) return VG_ERR_INVALID_ARG;
  o->n_sites = c->n;
  o->n_colours = c->ncol;
  o->coordination = c->z;
  o->path = c->path;
  o->precision = c->opt.precision;
  o->grid_blocks = c->grid;
  o->threads_per_block = c->tpb;
  o->sm_count = c->sm_count;
  o->device_bytes = c->device_bytes;
  o->sweep_index = c->sweep;
  return VG_OK;
}

const char* vg_last_error(const vg_ctx* c) { return c ? c->err.c_str() : g_err.c_str(); }

int vg_set_stream(vg_ctx* c, void* s) {
  if (!c) return VG_ERR_INVALID_ARG;
  VG_CUDA(c, cudaStreamSynchronize(c->stream));
  c->stream = s ? (cudaStream_t)s : c->own_stream;
  return VG_OK;
}

int vg_get_stream(const vg_ctx* c, void** s) {
  if (!c || !s) return VG_ERR_INVALID_ARG;
  *s = (void*)c->stream;
  return VG_OK;
}

int vg_init_random(vg_ctx* c) {
  if (!c) return VG_ERR_INVALID_ARG;
  VG_CUDA(c, cudaSetDevice(c->device));
  const RngKey key = rng_key(c, 0);
  const int layout = ising_layout(c);
  const ScMap m = sc_map(c);
  if (is_ising(c)) {
    ising_init<<<copy_grid(c, (c->n + 15) / 16), 256, 0, c->stream>>>(c->n, layout, m, (uint8_t*)c->spin[0][0],
                                                                       (uint8_t*)c->spin[1][0], key);
  } else if (fp64(c)) {
    Planes<double> P;
    for (int k = 0; k < 2; ++k) {
      P.x[k] = (double*)c->spin[k][0];
      P.y[k] = (double*)c->spin[k][1];
      P.z[k] = (double*)c->spin[k][2];
    }
    heis_init<double><<<copy_grid(c, c->n), 256, 0, c->stream>>>(c->n, layout, m, P, key);
  } else {
    Planes<float> P;
    for (int k = 0; k < 2; ++k) {
      P.x[k] = (float*)c->spin[k][0];
      P.y[k] = (float*)c->spin[k][1];
      P.z[k] = (float*)c->spin[k][2];
    }
    heis_init<float><<<copy_grid(c, c->n), 256, 0, c->stream>>>(c->n, layout, m, P, key);
  }
  VG_CUDA(c, cudaGetLastError());
  VG_CUDA(c, cudaStreamSynchronize(c->stream));
  return VG_OK;
}

int vg_set_state(vg_ctx* c, const void* host, int64_t n) {
  if (!c || !host) return fail(c, VG_ERR_INVALID_ARG, "NULL argument");
  if (n != c->n) return fail(c, VG_ERR_INVALID_ARG, "state length does not match the lattice");
  VG_CUDA(c, cudaSetDevice(c->device));
  const size_t bytes = is_ising(c) ? (size_t)n : (size_t)n * 3 * sizeof(double);
  int rc = ensure_stage(c, bytes);
  if (rc) return rc;
  VG_CUDA(c, cudaMemcpyAsync(c->d_stage, host, bytes, cudaMemcpyHostToDevice, c->stream));
  VG_CUDA(c, cudaMemsetAsync(c->d_flag, 0, sizeof(int), c->stream));
  const int layout = ising_layout(c);
  const ScMap m = sc_map(c);
  if (is_ising(c)) {
    ising_import<<<copy_grid(c, n), 256, 0, c->stream>>>((const int8_t*)c->d_stage, n, layout, m,
                                                         (uint8_t*)c->spin[0][0], (uint8_t*)c->spin[1][0], c->d_flag);
  } else if (fp64(c)) {
    Planes<double> P;
    for (int k = 0; k < 2; ++k) {
      P.x[k] = (double*)c->spin[k][0];
      P.y[k] = (double*)c->spin[k][1];
      P.z[k] = (double*)c->spin[k][2];
    }
    heis_import<double><<<copy_grid(c, n), 256, 0, c->stream>>>((const double*)c->d_stage, n, layout, m, P,
                                                                  c->d_flag);
  } else {
    Planes<float> P;
    for (int k = 0; k < 2; ++k) {
      P.x[k] = (float*)c->spin[k][0];
      P.y[k] = (float*)c->spin[k][1];
      P.z[k] = (float*)c->spin[k][2];
    }
    heis_import<float><<<copy_grid(c, n), 256, 0, c->stream>>>((const double*)c->d_stage, n, layout, m, P,
                                                                 c->d_flag);
  }
  VG_CUDA(c, cudaGetLastError());
  int flag = 0;
  VG_CUDA(c, cudaMemcpyAsync(&flag, c->d_flag, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  VG_CUDA(c, cudaStreamSynchronize(c->stream));
  if (flag)
    return fail(c, VG_ERR_INVALID_ARG,
                is_ising(c) ? "Ising spins must be +1 or -1" : "Heisenberg spins must be unit vectors (|s| = 1 +- 1e-3)");
  return VG_OK;
}

namespace {

// The state in natural site order into d_stage (int8 +-1, or [n][3]
// doubles), enqueued on the context's stream.
int export_natural(vg_ctx* c) {
  const int64_t n = c->n;
  const size_t bytes = is_ising(c) ? (size_t)n : (size_t)n * 3 * sizeof(double);
  int rc = ensure_stage(c, bytes);
  if (rc) return rc;
  const int layout = ising_layout(c);
  const ScMap m = sc_map(c);
  if (is_ising(c)) {
    ising_export<<<copy_grid(c, n), 256, 0, c->stream>>>((int8_t*)c->d_stage, n, layout, m,
                                                         (const uint8_t*)c->spin[0][0], (const uint8_t*)c->spin[1][0]);
  } else if (fp64(c)) {
    Planes<double> P;
    for (int k = 0; k < 2; ++k) {
      P.x[k] = (double*)c->spin[k][0];
      P.y[k] = (double*)c->spin[k][1];
      P.z[k] = (double*)c->spin[k][2];
    }
    heis_export<double><<<copy_grid(c, n), 256, 0, c->stream>>>((double*)c->d_stage, n, layout, m, P);
  } else {
    Planes<float> P;
    for (int k = 0; k < 2; ++k) {
      P.x[k] = (float*)c->spin[k][0];
      P.y[k] = (float*)c->spin[k][1];
      P.z[k] = (float*)c->spin[k][2];
    }
    heis_export<float><<<copy_grid(c, n), 256, 0, c->stream>>>((double*)c->d_stage, n, layout, m, P);
  }
  VG_CUDA(c, cudaGetLastError());
  return VG_OK;
}

}  // namespace

int vg_get_state(vg_ctx* c, void* host, int64_t n) {
  if (!c || !host) return fail(c, VG_ERR_INVALID_ARG, "NULL argument");
  if (n != c->n) return fail(c, VG_ERR_INVALID_ARG, "state length does not match the lattice");
  VG_CUDA(c, cudaSetDevice(c->device));
  const size_t bytes = is_ising(c) ? (size_t)n : (size_t)n * 3 * sizeof(double);
  int rc = export_natural(c);
  if (rc) return rc;
  VG_CUDA(c, cudaMemcpyAsync(host, c->d_stage, bytes, cudaMemcpyDeviceToHost, c->stream));
  VG_CUDA(c, cudaStreamSynchronize(c->stream));
  return VG_OK;
}

int vg_set_thermostat(vg_ctx* c, double T, const double b[3], double mag) {
  if (!c) return VG_ERR_INVALID_ARG;
  if (std::isnan(T) || !std::isfinite(mag)) return fail(c, VG_ERR_INVALID_ARG, "temperature and field must be numbers");
  if (b && !(std::isfinite(b[0]) && std::isfinite(b[1]) && std::isfinite(b[2])))
    return fail(c, VG_ERR_INVALID_ARG, "field orientation must be finite");
  c->T = clamp_temperature(T);
  if (b) {
    c->bhat[0] = b[0];
    c->bhat[1] = b[1];
    c->bhat[2] = b[2];
  }
  c->bmag = mag;
  return VG_OK;
}

int vg_set_sweep_index(vg_ctx* c, uint64_t s) {
  if (!c) return VG_ERR_INVALID_ARG;
  if (s >= kSweepLimit)
    return fail(c, VG_ERR_INVALID_ARG, "sweep index " + std::to_string(s) + " does not fit the 32-bit sweep word");
  c->sweep = s;
  return VG_OK;
}

int vg_get_sweep_index(const vg_ctx* c, uint64_t* s) {
  if (!c || !s) return VG_ERR_INVALID_ARG;
  *s = c->sweep;
  return VG_OK;
}

int vg_sweeps_async(vg_ctx* c, uint64_t n, int32_t measure) {
  if (!c) return VG_ERR_INVALID_ARG;
  VG_CUDA(c, cudaSetDevice(c->device));
  return enqueue(c, n, measure != 0);
}

int vg_read_sums(vg_ctx* c, uint64_t count, vg_sums* out) {
  if (!c) return VG_ERR_INVALID_ARG;
  if (count > c->last_batch) return fail(c, VG_ERR_INVALID_ARG, "more sums requested than the last batch measured");
  double* raw = nullptr;
  int rc = read_raw(c, count, &raw);
  if (rc) return rc;
  if (out)
    for (uint64_t t = 0; t < count; ++t) finish_sums(c, raw + t * kNumSums, out + t);
  return VG_OK;
}

int vg_synchronize(vg_ctx* c) {
  if (!c) return VG_ERR_INVALID_ARG;
  return sync_stream(c);
}

int vg_sweeps_sums(vg_ctx* c, uint64_t n, vg_sums* out) {
  if (!c) return VG_ERR_INVALID_ARG;
  VG_CUDA(c, cudaSetDevice(c->device));
  int rc = enqueue(c, n, out != nullptr);
  if (rc) return rc;
  if (!out) return sync_stream(c);
  return vg_read_sums(c, n, out);
}

int vg_sweeps(vg_ctx* c, uint64_t n, int32_t measure, double* E, double* M) {
  if (!c) return VG_ERR_INVALID_ARG;
  VG_CUDA(c, cudaSetDevice(c->device));
  int rc = enqueue(c, n, measure != 0);
  if (rc) return rc;
  if (!measure) return sync_stream(c);
  double* raw = nullptr;
  if ((rc = read_raw(c, n, &raw))) return rc;
  for (uint64_t t = 0; t < n; ++t) {
    vg_sums s;
    finish_sums(c, raw + t * kNumSums, &s);
    energy_of(c, &s, E ? E + t : nullptr, M ? M + t : nullptr);
  }
  return VG_OK;
}

int vg_time_passes(vg_ctx* c, uint64_t n, int32_t measure, double* pass_ms, double* sweep_ms) {
  if (!c || n == 0) return VG_ERR_INVALID_ARG;
  VG_CUDA(c, cudaSetDevice(c->device));
  int rc;
  if (measure) {
    if ((rc = ensure_sums(c, (size_t)n + 1))) return rc;
    if ((rc = ensure_part(c, rows_per_sweep(c) * kChunk))) return rc;
  }
  // a launch is one colour pass, or on the tiled path one whole sweep (an
  // even number of them, so that the state ends in the class arrays)
  const bool tiled = c->path == VG_PATH_TILED;
  if (tiled) n = (n + 1) & ~1ull;
  if ((rc = check_sweeps(c, n))) return rc;
  const int per_sweep = tiled ? 1 : c->ncol;
  if (tiled && measure && (rc = ensure_part(c, (size_t)tile_count(c) * kChunk))) return rc;
  std::vector<cudaEvent_t> ev((size_t)n * per_sweep * 2);
  for (auto& e : ev) VG_CUDA(c, cudaEventCreate(&e));
  const size_t rps = rows_per_sweep(c);
  const IsingTable tab = is_ising(c) ? ising_table(c) : IsingTable{};
  for (uint64_t t = 0; t < n; ++t) {
    for (int col = 0; col < per_sweep; ++col) {
      const size_t k = ((size_t)t * per_sweep + col) * 2;
      VG_CUDA(c, cudaEventRecord(ev[k], c->stream));
      if (tiled) {
        IsingTileArgs a = c->tile;
        uint8_t* base[2] = {(uint8_t*)c->spin[0][0], (uint8_t*)c->spin[1][0]};
        for (int q = 0; q < 2; ++q) {
          a.in[q] = (t & 1) ? c->tile_buf[q] : base[q];
          a.out[q] = (t & 1) ? base[q] : c->tile_buf[q];
        }
        long long* part = measure ? (long long*)c->d_part + (size_t)(t % kChunk) * tile_count(c) * kNumSums : nullptr;
        const cudaError_t e = launch_ising_tile_sweep(a, tab, rng_key(c, c->sweep + t), c->opt.proposal, part,
                                                      c->stream);
        if (e != cudaSuccess) return cuda_fail(c, e, "tiled sweep launch");
      } else {
        char* row = nullptr;
        if (measure) row = (char*)c->d_part + ((size_t)(t % kChunk) * rps + (size_t)col * c->grid) * kNumSums * 8;
        if ((rc = launch_pass(c, col, true, c->sweep + t, row))) return rc;
      }
      VG_CUDA(c, cudaEventRecord(ev[k + 1], c->stream));
    }
  }
  VG_CUDA(c, cudaStreamSynchronize(c->stream));
  double tot = 0.0, span = 0.0;
  for (size_t k = 0; k < ev.size(); k += 2) {
    float ms = 0.f;
    VG_CUDA(c, cudaEventElapsedTime(&ms, ev[k], ev[k + 1]));
    tot += ms;
  }
  float whole = 0.f;
  VG_CUDA(c, cudaEventElapsedTime(&whole, ev.front(), ev.back()));
  span = whole;
  for (auto& e : ev) cudaEventDestroy(e);
  c->sweep += n;
  if (pass_ms) *pass_ms = tot / (double)(n * per_sweep);
  if (sweep_ms) *sweep_ms = span / (double)n;
  return VG_OK;
}

int vg_current_sums(vg_ctx* c, vg_sums* out) {
  if (!c || !out) return VG_ERR_INVALID_ARG;
  VG_CUDA(c, cudaSetDevice(c->device));
  int rc;
  if ((rc = ensure_part(c, rows_per_sweep(c)))) return rc;
  if ((rc = ensure_sums(c, 1))) return rc;
  for (int col = 0; col < c->ncol; ++col) {
    char* row = (char*)c->d_part + (size_t)col * c->grid * kNumSums * 8;
    if ((rc = launch_pass(c, col, false, c->sweep, row))) return rc;
  }
  if ((rc = launch_reduce(c, 1, c->d_sums, (long long)rows_per_sweep(c)))) return rc;
  double* raw = nullptr;
  if ((rc = read_raw(c, 1, &raw))) return rc;
  finish_sums(c, raw, out);
  c->last_batch = 0;
  return VG_OK;
}

int vg_total_energy(vg_ctx* c, double* e) {
  if (!c || !e) return VG_ERR_INVALID_ARG;
  vg_sums s{};
  int rc = vg_current_sums(c, &s);
  if (rc) return rc;
  energy_of(c, &s, e, nullptr);
  return VG_OK;
}

int vg_magnetization(vg_ctx* c, double m[3], double* mag) {
  if (!c) return VG_ERR_INVALID_ARG;
  vg_sums s{};
  int rc = vg_current_sums(c, &s);
  if (rc) return rc;
  if (m) {
    m[0] = s.mx;
    m[1] = s.my;
    m[2] = s.mz;
  }
  energy_of(c, &s, nullptr, mag);
  return VG_OK;
}

int vg_energy_from_sums(const vg_ctx* c, const vg_sums* s, double* e, double* mag) {
  if (!c || !s) return VG_ERR_INVALID_ARG;
  energy_of(c, s, e, mag);
  return VG_OK;
}

namespace {

// The neighbour table in natural site order and each bond's occurrence among
// repeated bonds of one pair, built on first use.
int ensure_natural_nbr(vg_ctx* c) {
  if (c->d_wnbr) return VG_OK;
  Geometry g;
  std::string why;
  int rc;
  if ((rc = geometry_init(&c->lat, &g, &why))) return fail(c, rc, why);
  std::vector<int32_t> nbr;
  build_neighbours(g, nbr);
  std::vector<uint8_t> occ(nbr.size(), 0);
  for (int64_t i = 0; i < c->n; ++i)
    for (int k = 0; k < c->z; ++k) {
      const int32_t t = nbr[(size_t)i * c->z + k];
      uint8_t o = 0;
      for (int q = 0; q < k; ++q) o += nbr[(size_t)i * c->z + q] == t;
      occ[(size_t)i * c->z + k] = o;
    }
  if ((rc = dalloc(c, (void**)&c->d_wnbr, sizeof(int32_t) * nbr.size()))) return rc;
  if ((rc = dalloc(c, (void**)&c->d_wocc, occ.size()))) return rc;
  VG_CUDA(c, cudaMemcpy(c->d_wnbr, nbr.data(), sizeof(int32_t) * nbr.size(), cudaMemcpyHostToDevice));
  VG_CUDA(c, cudaMemcpy(c->d_wocc, occ.data(), occ.size(), cudaMemcpyHostToDevice));
  return VG_OK;
}

}  // namespace

int vg_wolff_steps(vg_ctx* c, uint64_t n, int32_t measure, double* E, double* M) {
  if (!c) return VG_ERR_INVALID_ARG;
  if (!is_ising(c)) return fail(c, VG_ERR_UNSUPPORTED, "Wolff steps need an Ising context");
  if (c->n * (int64_t)c->z >= (int64_t)INT32_MAX)
    return fail(c, VG_ERR_UNSUPPORTED, "Wolff steps index bonds with 32-bit integers: n_sites x z < 2^31");
  if (c->bonds) return fail(c, VG_ERR_UNSUPPORTED, "Wolff steps use the uniform exchange constant");
  VG_CUDA(c, cudaSetDevice(c->device));
  int rc;
  if ((rc = check_sweeps(c, n))) return rc;
  if ((rc = ensure_natural_nbr(c))) return rc;
  const bool mid = c->n > kWolffMaxSites && c->n <= kWolffMidSites;
  const bool grid = c->n > kWolffMidSites;
  if ((mid || grid) && !c->d_wq && (rc = dalloc(c, (void**)&c->d_wq, sizeof(int32_t) * (size_t)c->n))) return rc;
  if (grid && !c->d_wmark && (rc = dalloc(c, (void**)&c->d_wmark, sizeof(uint32_t) * (size_t)c->n))) return rc;
  if (grid && !c->d_wgrid && (rc = dalloc(c, (void**)&c->d_wgrid, sizeof(WolffGrid)))) return rc;
  // bond probability 1 - exp(-2 J / T) as a threshold on a 32-bit word (src/integrator.rs:199-203)
  const double J = c->ham.has_exchange ? c->ham.exchange : 0.0;
  const double T = clamp_temperature(c->T);
  const double p = 1.0 - std::exp(-2.0 * J / T);
  unsigned long long thr;
  if (!(p > 0.0)) thr = 0;
  else {
    const double x = std::ceil(p * 4294967296.0);
    thr = x >= 4294967296.0 ? (1ull << 32) : (unsigned long long)x;
  }
  if ((rc = ensure_stage(c, (size_t)c->n))) return rc;
  if (measure && (rc = ensure_sums(c, (size_t)std::max<uint64_t>(n, 1)))) return rc;
  const int layout = ising_layout(c);
  const ScMap m = sc_map(c);
  ising_export<<<copy_grid(c, c->n), 256, 0, c->stream>>>((int8_t*)c->d_stage, c->n, layout, m,
                                                          (const uint8_t*)c->spin[0][0],
                                                          (const uint8_t*)c->spin[1][0]);
  VG_CUDA(c, cudaGetLastError());
  for (uint64_t t0 = 0; t0 < n; t0 += (1u << 30)) {
    const uint32_t k = (uint32_t)std::min<uint64_t>(n - t0, 1u << 30);
    double* sums = measure ? c->d_sums + t0 * kNumSums : nullptr;
    const RngKey key = rng_key(c, c->sweep + t0);
    const cudaError_t e =
        grid ? launch_ising_wolff_grid((int8_t*)c->d_stage, (int)c->n, c->z, c->d_wnbr, c->d_wocc, thr, key, k, sums,
                                       c->d_wmark, c->d_wq, c->d_wgrid, c->sm_count, c->stream)
        : mid ? launch_ising_wolff_mid((int8_t*)c->d_stage, (int)c->n, c->z, c->d_wnbr, c->d_wocc, thr, key, k, sums,
                                       c->d_wq, c->stream)
              : launch_ising_wolff((int8_t*)c->d_stage, (int)c->n, c->z, c->d_wnbr, c->d_wocc, thr, key, k, sums,
                                   c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "Wolff kernel launch");
    if (grid) {  // a grid barrier that gave up leaves the flag set
      unsigned int aborted = 0;
      VG_CUDA(c, cudaMemcpyAsync(&aborted, &c->d_wgrid->abort_flag, sizeof(aborted), cudaMemcpyDeviceToHost,
                                 c->stream));
      VG_CUDA(c, cudaStreamSynchronize(c->stream));
      if (aborted) return fail(c, VG_ERR_TIMEOUT, "Wolff steps: a grid barrier wait ran out (2 s)");
    }
  }
  VG_CUDA(c, cudaMemsetAsync(c->d_flag, 0, sizeof(int), c->stream));
  ising_import<<<copy_grid(c, c->n), 256, 0, c->stream>>>((const int8_t*)c->d_stage, c->n, layout, m,
                                                          (uint8_t*)c->spin[0][0], (uint8_t*)c->spin[1][0],
                                                          c->d_flag);
  VG_CUDA(c, cudaGetLastError());
  c->sweep += n;
  if (!measure) return sync_stream(c);
  c->last_batch = n;
  double* raw = nullptr;
  if ((rc = read_raw(c, n, &raw))) return rc;
  for (uint64_t t = 0; t < n; ++t) {
    vg_sums s;
    finish_sums(c, raw + t * kNumSums, &s);
    energy_of(c, &s, E ? E + t : nullptr, M ? M + t : nullptr);
  }
  return VG_OK;
}

int vg_selftest_grid_barrier(vg_ctx* c, int32_t skip_block) {
  if (!c) return VG_ERR_INVALID_ARG;
  VG_CUDA(c, cudaSetDevice(c->device));
  int rc;
  if (!c->d_wgrid && (rc = dalloc(c, (void**)&c->d_wgrid, sizeof(WolffGrid)))) return rc;
  const int skip = skip_block >= 0 && skip_block < 4 ? skip_block : -1;
  const cudaError_t e = launch_wolff_barrier_probe(c->d_wgrid, 4, skip, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "barrier self-test launch");
  unsigned int aborted = 0;
  VG_CUDA(c, cudaMemcpyAsync(&aborted, &c->d_wgrid->abort_flag, sizeof(aborted), cudaMemcpyDeviceToHost, c->stream));
  VG_CUDA(c, cudaStreamSynchronize(c->stream));
  if (aborted) return fail(c, VG_ERR_TIMEOUT, "grid barrier self-test: a wait ran out (2 s)");
  return VG_OK;
}

int vg_set_exchange_bonds(vg_ctx* c, const double* J, int64_t n_entries) {
  if (!c) return VG_ERR_INVALID_ARG;
  VG_CUDA(c, cudaSetDevice(c->device));
  VG_CUDA(c, cudaStreamSynchronize(c->stream));
  if (c->d_jnat) {  // stale natural-order copy
    cudaFree(c->d_jnat);
    c->device_bytes -= (int64_t)(sizeof(double) * c->bonds_nat.size());
    c->d_jnat = nullptr;
  }
  c->bonds_nat.clear();
  if (!J) {  // back to the uniform constant
    for (int k = 0; k < kMaxColours; ++k) {
      if (c->d_jb[k]) cudaFree(c->d_jb[k]);
      if (c->d_jbf[k]) cudaFree(c->d_jbf[k]);
      c->d_jb[k] = nullptr;
      c->d_jbf[k] = nullptr;
    }
    c->bonds = false;
    return VG_OK;
  }
  if (c->path != VG_PATH_GENERIC)
    return fail(c, VG_ERR_UNSUPPORTED, "per-bond exchange constants need the generic path (vg_options.path)");
  if (!c->ham.has_exchange) return fail(c, VG_ERR_INVALID_ARG, "the Hamiltonian has no exchange term");
  if (n_entries != c->n * (int64_t)c->z) return fail(c, VG_ERR_INVALID_ARG, "expected n_sites x coordination entries");
  Geometry g;
  std::string why;
  int rc = geometry_init(&c->lat, &g, &why);
  if (rc) return fail(c, rc, why);
  std::vector<int32_t> nbr;
  build_neighbours(g, nbr);
  // symmetric (J_ij = J_ji, summed over repeated bonds of one pair) and finite
  for (int64_t i = 0; i < c->n; ++i)
    for (int k = 0; k < c->z; ++k) {
      const int32_t t = nbr[(size_t)i * c->z + k];
      const double v = J[(size_t)i * c->z + k];
      if (t < 0) continue;
      if (!std::isfinite(v)) return fail(c, VG_ERR_INVALID_ARG, "exchange constants must be finite");
      double a = 0.0, b = 0.0;
      for (int q = 0; q < c->z; ++q) {
        if (nbr[(size_t)i * c->z + q] == t) a += J[(size_t)i * c->z + q];
        if (nbr[(size_t)t * c->z + q] == i) b += J[(size_t)t * c->z + q];
      }
      if (std::fabs(a - b) > 1e-12 * std::max(1.0, std::fabs(a)))
        return fail(c, VG_ERR_INVALID_ARG, "exchange constants must be symmetric (J_ij == J_ji)");
    }
  std::vector<int32_t> col;
  greedy_colouring(g, nbr, col);
  for (int k = 0; k < c->ncol; ++k) {
    const int64_t nc = c->class_size[k];
    std::vector<double> ell((size_t)c->z * nc, 0.0);
    std::vector<float> ellf(ell.size(), 0.f);
    int64_t j = 0;
    for (int64_t i = 0; i < c->n; ++i) {  // class entries in ascending site order
      if (col[i] != k) continue;
      for (int q = 0; q < c->z; ++q) {
        const double v = nbr[(size_t)i * c->z + q] >= 0 ? J[(size_t)i * c->z + q] : 0.0;
        ell[(size_t)q * nc + j] = v;
        ellf[(size_t)q * nc + j] = (float)v;
      }
      ++j;
    }
    if (!c->d_jb[k] && (rc = dalloc(c, (void**)&c->d_jb[k], sizeof(double) * ell.size()))) return rc;
    if (!c->d_jbf[k] && (rc = dalloc(c, (void**)&c->d_jbf[k], sizeof(float) * ellf.size()))) return rc;
    VG_CUDA(c, cudaMemcpy(c->d_jb[k], ell.data(), sizeof(double) * ell.size(), cudaMemcpyHostToDevice));
    VG_CUDA(c, cudaMemcpy(c->d_jbf[k], ellf.data(), sizeof(float) * ellf.size(), cudaMemcpyHostToDevice));
  }
  c->bonds_nat.assign(J, J + (size_t)c->n * c->z);
  for (size_t e = 0; e < nbr.size(); ++e)
    if (nbr[e] < 0) c->bonds_nat[e] = 0.0;
  c->bonds = true;
  return VG_OK;
}

namespace {

// Natural-order state, neighbour table, bond constants and an auxiliary
// buffer of `aux` doubles for the energy entry points.
int energy_setup(vg_ctx* c, size_t aux) {
  int rc;
  VG_CUDA(c, cudaSetDevice(c->device));
  if ((rc = ensure_natural_nbr(c))) return rc;
  if (c->bonds && !c->d_jnat) {
    if ((rc = dalloc(c, (void**)&c->d_jnat, sizeof(double) * c->bonds_nat.size()))) return rc;
    VG_CUDA(c, cudaMemcpy(c->d_jnat, c->bonds_nat.data(), sizeof(double) * c->bonds_nat.size(),
                          cudaMemcpyHostToDevice));
  }
  if (aux > c->eaux_cap) {
    if (c->d_eaux) {
      cudaFree(c->d_eaux);
      c->device_bytes -= (int64_t)(sizeof(double) * c->eaux_cap);
      c->d_eaux = nullptr;
      c->eaux_cap = 0;
    }
    if ((rc = dalloc(c, (void**)&c->d_eaux, sizeof(double) * aux))) return rc;
    c->eaux_cap = aux;
  }
  return export_natural(c);
}

SiteTerms site_terms(const vg_ctx* c) {
  const vg_hamiltonian_desc& h = c->ham;
  SiteTerms t;
  t.has_exchange = h.has_exchange;
  t.has_anisotropy = h.has_anisotropy;
  t.has_zeeman = h.has_zeeman;
  t.has_gauge = h.has_gauge;
  t.has_cubic = h.has_cubic;
  t.J = h.exchange;
  t.K = h.anisotropy;
  for (int a = 0; a < 3; ++a) {
    t.axis[a] = h.anisotropy_axis[a];
    t.b[a] = c->bhat[a];
  }
  t.hz = zeeman_coef(c);
  t.gauge = h.gauge;
  t.Kc = h.cubic;
  t.axis_sign = h.anisotropy_axis[2] >= 0.0 ? 1.0 : -1.0;
  t.field_sign = c->bhat[2] >= 0.0 ? 1.0 : -1.0;
  return t;
}

}  // namespace

int vg_site_energies(vg_ctx* c, double* out, int64_t n) {
  if (!c || !out) return fail(c, VG_ERR_INVALID_ARG, "NULL argument");
  if (n != c->n) return fail(c, VG_ERR_INVALID_ARG, "output length does not match the lattice");
  int rc;
  if ((rc = energy_setup(c, (size_t)n))) return rc;
  const cudaError_t e = launch_site_energies(is_ising(c), c->d_stage, n, c->z, c->d_wnbr, c->bonds ? c->d_jnat : nullptr,
                                             site_terms(c), c->d_eaux, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "site energy launch");
  VG_CUDA(c, cudaMemcpyAsync(out, c->d_eaux, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, c->stream));
  return sync_stream(c);
}

int vg_delta_energies(vg_ctx* c, const double* proposals, double* out, int64_t n) {
  if (!c || !proposals || !out) return fail(c, VG_ERR_INVALID_ARG, "NULL argument");
  if (is_ising(c)) return fail(c, VG_ERR_UNSUPPORTED, "energy changes of proposals are computed for Heisenberg spins");
  if (n != c->n) return fail(c, VG_ERR_INVALID_ARG, "proposal length does not match the lattice");
  int rc;
  if ((rc = energy_setup(c, (size_t)n * 4))) return rc;
  double* d_prop = c->d_eaux;
  double* d_out = c->d_eaux + (size_t)n * 3;
  VG_CUDA(c, cudaMemcpyAsync(d_prop, proposals, sizeof(double) * 3 * (size_t)n, cudaMemcpyHostToDevice, c->stream));
  const double* jn = c->bonds ? c->d_jnat : nullptr;
  const cudaError_t e =
      fp64(c) ? launch_heis_delta<double>((const double*)c->d_stage, d_prop, n, c->z, c->d_wnbr, jn,
                                          heis_params<double>(c), d_out, c->stream)
              : launch_heis_delta<float>((const double*)c->d_stage, d_prop, n, c->z, c->d_wnbr, jn,
                                         heis_params<float>(c), d_out, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "energy change launch");
  VG_CUDA(c, cudaMemcpyAsync(out, d_out, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, c->stream));
  return sync_stream(c);
}

int vg_lattice_neighbours(const vg_lattice_desc* lat, int32_t* nbr, int64_t cap, int64_t* n_sites, int32_t* zmax) {
  Geometry g;
  std::string why;
  int rc = geometry_init(lat, &g, &why);
  if (rc) return fail(nullptr, rc, why);
  if (n_sites) *n_sites = g.n;
  if (zmax) *zmax = g.z;
  if (!nbr) return VG_OK;
  if (cap < g.n * g.z) return fail(nullptr, VG_ERR_INVALID_ARG, "neighbour buffer too small");
  for (int64_t i = 0; i < g.n; ++i)
    for (int k = 0; k < g.z; ++k) nbr[i * g.z + k] = neighbour_of(g, i, k);
  return VG_OK;
}

int vg_lattice_colouring(const vg_lattice_desc* lat, int32_t* colour, int64_t cap, int32_t* n_colours) {
  Geometry g;
  std::string why;
  int rc = geometry_init(lat, &g, &why);
  if (rc) return fail(nullptr, rc, why);
  std::vector<int32_t> nbr, col;
  build_neighbours(g, nbr);
  const int nc = greedy_colouring(g, nbr, col);
  if (n_colours) *n_colours = nc;
  if (!colour) return VG_OK;
  if (cap < g.n) return fail(nullptr, VG_ERR_INVALID_ARG, "colour buffer too small");
  std::memcpy(colour, col.data(), sizeof(int32_t) * (size_t)g.n);
  return VG_OK;
}

int vg_host_alloc(void** p, uint64_t bytes) {
  if (!p) return VG_ERR_INVALID_ARG;
  cudaError_t e = cudaMallocHost(p, bytes ? bytes : 1);
  if (e != cudaSuccess) {
    *p = nullptr;
    return fail(nullptr, e == cudaErrorMemoryAllocation ? VG_ERR_OOM : VG_ERR_CUDA, cudaGetErrorString(e));
  }
  return VG_OK;
}

// Lets other translation units record the thread's last error message.
void vg_internal_set_last_error(const char* msg) { g_err = msg ? msg : ""; }

int vg_host_free(void* p) {
  if (!p) return VG_OK;
  cudaError_t e = cudaFreeHost(p);
  return e == cudaSuccess ? VG_OK : fail(nullptr, VG_ERR_CUDA, cudaGetErrorString(e));
}

}  // extern "C"
