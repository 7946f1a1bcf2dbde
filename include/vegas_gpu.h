/*
 * vegas_gpu.h -- C ABI of the GB300 (sm_103a) Metropolis engine for vegas.
 *
 * The engine replaces the hot path of the vegas crate:
 *   Integrator<S>::step            src/integrator.rs:40-49  (trait)
 *   MetropolisFlipIntegrator::step src/integrator.rs:113-137
 *   MetropolisIntegrator::step     src/integrator.rs:66-92
 *   Hamiltonian::energy/total      src/energy.rs:45-60, terms :62-257
 *   State / Spin / Field           src/state.rs:28-318
 *   Thermostat                     src/thermostat.rs:17-79
 * and the per-sweep measurement done by the instruments
 *   StatSensor::after_step         src/instrument.rs:133-141
 *   ObservableSensor::after_step   src/instrument.rs:254-262.
 *
 * Conventions
 *   - Every function returns an int status (VG_OK = 0).  The library never
 *     aborts and never falls back to the CPU: without a usable GPU it returns
 *     VG_ERR_NO_DEVICE / VG_ERR_CUDA.
 *   - A context owns its device memory and one CUDA stream.  A context is not
 *     thread-safe; distinct contexts are independent.
 *   - Host buffers belong to the caller and are copied.  Spin buffers are in
 *     the lattice's site order: site = ((cz*ny + cy)*nx + cx)*nbasis + b.
 *     Ising spins are int8 +1 (Up) / -1 (Down); Heisenberg spins are three
 *     doubles (x, y, z) per site.
 *   - Sweep t of a context draws its random numbers from Philox4x32 keyed by
 *     (seed, replica) with counters (site, t, stream tag): 10 rounds for
 *     Ising draws and initial states, 7 for the Heisenberg update draws and
 *     the batched threshold planes; (seed, sweep index) is the whole RNG
 *     state, so vg_set_sweep_index resumes a run exactly.
 */
#ifndef VEGAS_GPU_H
#define VEGAS_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VG_ABI_VERSION 1

typedef struct vg_ctx vg_ctx;

enum vg_status {
  VG_OK = 0,
  VG_ERR_INVALID_ARG = 1,
  VG_ERR_CUDA = 2,
  VG_ERR_TIMEOUT = 3,
  VG_ERR_OOM = 4,
  VG_ERR_UNSUPPORTED = 5,
  VG_ERR_NO_DEVICE = 6
};

enum vg_spin_kind { VG_SPIN_ISING = 0, VG_SPIN_HEISENBERG = 1 };
enum vg_unit_cell { VG_CELL_SC = 0, VG_CELL_BCC = 1, VG_CELL_FCC = 2 };
/* FLIP: MetropolisFlipIntegrator (src/integrator.rs:99-138).
 * RANDOM: MetropolisIntegrator, proposal Spin::rand (src/integrator.rs:56-92). */
enum vg_proposal { VG_PROPOSE_FLIP = 0, VG_PROPOSE_RANDOM = 1 };
/* Kernel family.  AUTO picks RESIDENT for Ising lattices of at most 8192
 * sites that admit STRUCTURED, else STRUCTURED when the lattice allows it,
 * else GENERIC.  STRUCTURED: sc lattices with an even x extent (Ising: x/2 a
 * multiple of 16) and even periodic y / z extents, as a checkerboard; bcc /
 * fcc Ising lattices with x a multiple of 16 and every bcc / fcc Heisenberg
 * lattice, one array (Heisenberg: three planes) per basis sublattice.  GENERIC: any lattice, and per-bond exchange constants
 * (vg_set_exchange_bonds).  RESIDENT keeps the checkerboard layout of STRUCTURED in one
 * thread block's shared memory and runs all sweeps of a call in one launch
 * (Ising, at most 65536 sites).  TILED (Ising sc, periodic on every axis,
 * x a multiple of 64, even y and z >= 4) runs each sweep as one launch:
 * both colour passes on shared-memory tiles with halos, reading the class
 * arrays and writing a second pair, so the context holds twice the spins;
 * AUTO does not choose it (the two-pass kernels measured faster).  Results
 * are identical across paths. */
enum vg_path { VG_PATH_AUTO = 0, VG_PATH_GENERIC = 1, VG_PATH_STRUCTURED = 2, VG_PATH_RESIDENT = 3, VG_PATH_TILED = 4 };
enum vg_precision { VG_FP32 = 0, VG_FP64 = 1 };

/* Lattice::sc/bcc/fcc(1.0).expand(nx, ny, nz) with drop_x/y/z on the open
 * axes (src/input.rs:296-322). */
typedef struct {
  int32_t cell;           /* vg_unit_cell */
  int32_t nx, ny, nz;     /* unit cells per axis, >= 1 */
  int32_t pbc_x, pbc_y, pbc_z;
} vg_lattice_desc;

/* A Hamiltonian assembled from the reference's terms (src/energy.rs):
 *   Exchange::from_lattice(J)  per site -J sum_j s_i.s_j          (:176-206)
 *   UniaxialAnisotropy(e, K)   per site +K (s.e)^2                (:108-112)
 *   Zeeman                     per site zeeman_sign |B| (s.b)     (:147-151)
 *   Gauge(g)                   per site g                         (:75-80)
 *   cubic (extension, no reference counterpart)  -Kc (sx^4+sy^4+sz^4)
 * compound = 1 selects Compound's total (sum_i energy(i), :55-59, :248-257);
 * compound = 0 requires exactly one term and uses that term's own
 * total_energy (Exchange halves :208-213, UniaxialAnisotropy drops K
 * :114-120, Zeeman negates :153-160, Gauge N g). */
typedef struct {
  int32_t has_exchange;   double exchange;
  int32_t has_anisotropy; double anisotropy; double anisotropy_axis[3];
  int32_t has_zeeman;     double zeeman_sign; /* +1 reproduces the reference */
  int32_t has_gauge;      double gauge;
  int32_t has_cubic;      double cubic;
  int32_t compound;
} vg_hamiltonian_desc;

typedef struct {
  int32_t spin_kind;          /* vg_spin_kind */
  int32_t proposal;           /* vg_proposal */
  int32_t path;               /* vg_path */
  int32_t precision;          /* vg_precision (Heisenberg only) */
  uint32_t replica;           /* replica id mixed into the RNG counters */
  int32_t threads_per_block;  /* 0 = library default */
  int32_t blocks_per_sm;      /* 0 = library default (grid-stride cap) */
  int32_t device;             /* -1 = current device */
  int64_t max_device_bytes;   /* 0 = no cap; beyond it allocations fail with VG_ERR_OOM */
} vg_options;

/* Raw per-sweep lattice sums (FP64), from which every total the reference
 * reports is formed.  bond counts each bond once (with multiplicity). */
typedef struct {
  double bond;        /* sum over bonds s_i . s_j */
  double anisotropy;  /* sum_i (s_i . e)^2 */
  double zeeman;      /* sum_i s_i . b */
  double cubic;       /* sum_i sx^4 + sy^4 + sz^4 */
  double mx, my, mz;  /* magnetisation vector */
  double accepted;    /* accepted proposals in the sweep */
} vg_sums;

typedef struct {
  int64_t n_sites;
  int32_t n_colours;
  int32_t coordination;
  int32_t path;               /* the path actually used */
  int32_t precision;
  int32_t grid_blocks;
  int32_t threads_per_block;
  int32_t sm_count;
  int64_t device_bytes;       /* device memory held by the context */
  uint64_t sweep_index;
} vg_info;

/* ---------------------------------------------------------------- status */
const char* vg_status_string(int status);
int vg_abi_version(void);
int vg_device_count(int32_t* count);
/* Name of a CUDA device (for tuning caches); NUL-terminated, truncated to capacity. */
int vg_device_name(int32_t device, char* name, int32_t capacity);

/* ------------------------------------------------------------- lifecycle */
/* Defaults: flip proposal for Ising, random proposal for Heisenberg (the
 * integrators src/input.rs:347-364 picks), AUTO path, FP32. */
int vg_options_default(int32_t spin_kind, vg_options* out);
int vg_ctx_create(const vg_lattice_desc* lattice, const vg_hamiltonian_desc* hamiltonian,
                  int32_t spin_kind, uint64_t seed, vg_ctx** out);
int vg_ctx_create_ex(const vg_lattice_desc* lattice, const vg_hamiltonian_desc* hamiltonian,
                     const vg_options* options, uint64_t seed, vg_ctx** out);
int vg_ctx_destroy(vg_ctx* ctx);
int vg_ctx_info(const vg_ctx* ctx, vg_info* out);
const char* vg_last_error(const vg_ctx* ctx);
/* Run the context's work on a caller-owned cudaStream_t (NULL restores the
 * context's own stream). */
int vg_set_stream(vg_ctx* ctx, void* cuda_stream);
int vg_get_stream(const vg_ctx* ctx, void** cuda_stream);

/* ------------------------------------------------------ state and bath */
/* State::rand_with_size (src/state.rs:260-262) on the device. */
int vg_init_random(vg_ctx* ctx);
int vg_set_state(vg_ctx* ctx, const void* host_spins, int64_t n_sites);
int vg_get_state(vg_ctx* ctx, void* host_spins, int64_t n_sites);
/* Thermostat::new(T, Field::new(orientation, magnitude)); T is clamped to
 * f64::EPSILON (src/thermostat.rs:29-39) and |magnitude| is used
 * (Field::magnitude, src/state.rs:219-221). For Ising only the sign of
 * b_hat[2] matters (Up / Down). */
int vg_set_thermostat(vg_ctx* ctx, double temperature, const double b_hat[3], double magnitude);
int vg_set_sweep_index(vg_ctx* ctx, uint64_t sweep);
int vg_get_sweep_index(const vg_ctx* ctx, uint64_t* sweep);

/* ---------------------------------------------------------------- sweeps */
/* n Metropolis sweeps (each attempts one update per site).  If measure, the
 * per-sweep total energy (with the desc's total semantics) and |M| are
 * written to E_out[t] and M_out[t] (either may be NULL).  Synchronous. */
int vg_sweeps(vg_ctx* ctx, uint64_t n, int32_t measure, double* E_out, double* M_out);
/* Same, returning the raw per-sweep sums (out may be NULL). Synchronous. */
int vg_sweeps_sums(vg_ctx* ctx, uint64_t n, vg_sums* out);
/* Enqueue n sweeps on the context stream and return at once.  With measure,
 * the per-sweep sums stay on the device; vg_read_sums fetches the last
 * enqueued batch.  Used for device-resident timing. */
int vg_sweeps_async(vg_ctx* ctx, uint64_t n, int32_t measure);
int vg_read_sums(vg_ctx* ctx, uint64_t count, vg_sums* out);
int vg_synchronize(vg_ctx* ctx);

/* Run n sweeps with a CUDA event pair around every launch on the context
 * stream; returns the mean launch duration and the mean sweep duration (ms).
 * A launch is one colour pass, or on the tiled path one whole sweep (there n
 * is rounded up to an even count).  The sweeps are real work (the sweep
 * index advances). */
int vg_time_passes(vg_ctx* ctx, uint64_t n, int32_t measure, double* mean_pass_ms, double* mean_sweep_ms);

/* Wolff cluster steps (WolffIntegrator::step, src/integrator.rs:140-230) of
 * an Ising context: each step picks a source site, grows the cluster of
 * spins equal to it over bonds active with probability 1 - exp(-2 J / T)
 * (the Hamiltonian's exchange constant J, the thermostat's T; the field is
 * not used, as in the reference) and flips it.  Per step, E and |M| as
 * vg_sweeps; vg_sums.accepted of vg_current_sums-style rows is the cluster
 * size.  A step advances the context's sweep index by one.  Lattices of up
 * to 786432 sites run in one thread block's shared memory (spins and marks
 * as bytes up to 16384 sites, as bits beyond); larger ones in one
 * cooperative launch over the whole grid (a grid barrier per breadth-first
 * level; VG_ERR_TIMEOUT if one ever waits more than 2 s).  The uniform
 * exchange constant only (no per-bond constants). */
int vg_wolff_steps(vg_ctx* ctx, uint64_t n_steps, int32_t measure, double* E, double* M);

/* Self-test of the bounded waits of the grid barrier vg_wolff_steps uses on
 * large lattices (no reference counterpart): one barrier over four blocks of
 * a cooperative launch on the context's device and stream.  With
 * skip_block in [0, 4) that block never arrives and the others' waits run
 * out after 2 s: VG_ERR_TIMEOUT.  Otherwise VG_OK.  The context stays
 * usable either way. */
int vg_selftest_grid_barrier(vg_ctx* ctx, int32_t skip_block);

/* Per-bond exchange constants: Exchange's CSR with arbitrary J_ij
 * (src/energy.rs:169-206) instead of one constant for every bond.
 * J[i * z + k] is the constant of the bond from site i to its k-th
 * neighbour in vg_lattice_neighbours order (n_entries = n_sites x z; entries
 * of absent neighbours are ignored).  The table must be symmetric (per pair
 * of sites, the constants of its repeated bonds summed, J_ij == J_ji).  It
 * replaces the Hamiltonian's uniform exchange constant; the bond sum then
 * carries the constants (vg_sums.bond = sum over bonds of J_ij s_i.s_j) and
 * the totals use J = 1.  Needs a context on the generic path
 * (vg_options.path = VG_PATH_GENERIC) with an exchange term; Ising
 * thresholds are then formed per site in FP64.  J = NULL restores the
 * uniform constant. */
int vg_set_exchange_bonds(vg_ctx* ctx, const double* J, int64_t n_entries);

/* ---------------------------------------------------------- observables */
int vg_current_sums(vg_ctx* ctx, vg_sums* out);
int vg_total_energy(vg_ctx* ctx, double* energy);
int vg_magnetization(vg_ctx* ctx, double m[3], double* magnitude);
/* Total energy / |M| from raw sums with a context's Hamiltonian semantics. */
int vg_energy_from_sums(const vg_ctx* ctx, const vg_sums* sums, double* energy, double* magnitude);

/* Per-site energies of the current state: out[i] = Hamiltonian::energy(i)
 * (src/energy.rs:45-52), the sum of the Hamiltonian's terms at site i as
 * Compound::energy forms it (src/energy.rs:254-256): exchange
 * -sum_j J_ij s_i.s_j over the site's neighbours (src/energy.rs:194-208),
 * anisotropy K (s.e)^2 (:108-112), Zeeman |B| (s.b) with the reference's
 * sign (:147-152), gauge g (:75-80), and -Kc (sx^4 + sy^4 + sz^4) for the
 * cubic term.  Computed in FP64 on the device from the state as the context
 * holds it; n = the number of sites. */
int vg_site_energies(vg_ctx* ctx, double* out, int64_t n);

/* Energy changes of single-site proposals (Heisenberg contexts):
 * out[i] = energy of site i with its spin replaced by proposals[3i..3i+2],
 * every other spin as it is, minus its current energy; the difference the
 * Metropolis step accepts with probability min(1, exp(-dE / T))
 * (src/integrator.rs:77-86).  Runs the
 * sweeps' own energy-change function in the context's precision (FP32 or
 * FP64), so FP32 rounding can be checked against FP64. */
int vg_delta_energies(vg_ctx* ctx, const double* proposals, double* out, int64_t n);

/* ------------------------------------------------------ batched replicas */
/* Many independent Ising replicas (MetropolisFlipIntegrator,
 * src/integrator.rs:99-138, with Exchange only, h = 0) run at once: 32
 * replicas of one lattice share each 32-bit word (multi-spin coding; bit l
 * is replica 32w + l, 1 = Up).  A group is n_replicas (a multiple of 32, at
 * most 1024) replicas of one sc lattice with even extents, periodic on every
 * axis or 2D (nz = 1, open z), and a temperature ladder: replica r starts at
 * ladder entry r.  Work proceeds in rounds of sweeps_per_round sweeps; after
 * each round the engine records, per replica, the number of anti-aligned
 * bonds and of up spins, and (if replica_exchange) swaps the temperatures of
 * adjacent ladder entries i, i+1 (i even in even rounds, odd in odd rounds)
 * with probability min(1, exp((1/T_i - 1/T_j)(E_i - E_j))).  A round is
 * replayed as one CUDA graph.  Every replica's updates are bit-exact against
 * an independent single-replica oracle of the same draws. */
typedef struct {
  vg_lattice_desc lattice;
  int32_t n_replicas;
  const double* temperatures;  /* n_replicas ladder entries (copied) */
} vg_replica_group;

typedef struct vg_batch vg_batch;

typedef struct {
  int32_t n_groups;
  int32_t total_replicas;
  int32_t replica_words;
  int32_t sweeps_per_round;
  int64_t replica_sites;       /* sum over replicas of lattice sites: flips per sweep */
  uint64_t sweep_index;
  uint32_t round_index;
  int32_t graph;               /* 1 if a round is replayed as a CUDA graph */
} vg_batch_info;

int vg_batch_create(const vg_replica_group* groups, int32_t n_groups, double exchange, uint64_t seed,
                    int32_t sweeps_per_round, int32_t replica_exchange, vg_batch** out);
int vg_batch_destroy(vg_batch* batch);
const char* vg_batch_last_error(const vg_batch* batch);
int vg_batch_get_info(const vg_batch* batch, vg_batch_info* out);
int vg_batch_get_stream(const vg_batch* batch, void** cuda_stream);
/* Launch shape of the multi-spin-coded passes.  Every supported shape gives
 * identical results: threads_per_block 128 or 256, words_per_thread 2, 4 or
 * 8 (a block covers threads x words consecutive words), words_in_flight 1 or
 * 2 (words a thread decides together).  Default {256, 4, 1}. */
typedef struct {
  int32_t threads_per_block;
  int32_t words_per_thread;
  int32_t words_in_flight;
} vg_batch_tuning;
int vg_batch_get_tuning(const vg_batch* batch, vg_batch_tuning* out);
int vg_batch_set_tuning(vg_batch* batch, const vg_batch_tuning* tuning);
/* Times every supported shape over `rounds` rounds (after one warm-up
 * round each) on this batch and keeps the fastest.  The spins, ladders,
 * tables, counters and the last run's observables are saved before and
 * restored after, so the batch continues exactly as if it had not been
 * tuned.  best / best_ms_per_round may be NULL. */
int vg_batch_autotune(vg_batch* batch, uint32_t rounds, vg_batch_tuning* best, double* best_ms_per_round);
/* Every replica random (bit l of Philox(site, 0, tag, word)), ladder reset. */
int vg_batch_init_random(vg_batch* batch);
/* rounds x sweeps_per_round sweeps (synchronous / enqueue only). */
int vg_batch_run(vg_batch* batch, uint64_t rounds);
int vg_batch_run_async(vg_batch* batch, uint64_t rounds);
int vg_batch_synchronize(vg_batch* batch);
/* Round `round` (0-based) of the last run: counts[2 r] = anti-aligned bonds,
 * counts[2 r + 1] = up spins of replica r (global index), tau[r] = its
 * ladder entry during that round.  E_r = -J (z N / 2 - 2 anti), M_r = 2 up - N. */
int vg_batch_observables(vg_batch* batch, uint64_t round, int64_t* counts, int32_t* tau);
/* Current ladder entry of every replica of a group. */
int vg_batch_ladder(vg_batch* batch, int32_t group, int32_t* tau);
/* Accepted / attempted swaps of ladder pairs (i, i+1), per i. */
int vg_batch_swap_stats(vg_batch* batch, int32_t group, int64_t* accepted, int64_t* attempted);
/* One replica's spins (int8 +1/-1, site order). */
int vg_batch_get_replica(vg_batch* batch, int32_t group, int32_t replica, int8_t* spins);
int vg_batch_set_replica(vg_batch* batch, int32_t group, int32_t replica, const int8_t* spins);

/* -------------------------------------------- batched Heisenberg replicas
 * Many Heisenberg replicas of one bcc or fcc lattice swept together under a
 * shared field schedule (hysteresis loops; HysteresisLoop::run,
 * src/program.rs:281-335, and MetropolisIntegrator::step for every replica,
 * src/integrator.rs:66-92).  Every replica has its own seed, Philox stream
 * id, temperature and energy constants.  The colour classes are the basis
 * sublattices (bcc 2, fcc 4), which is what the greedy colouring of these
 * lattices gives, and a class entry is the cell index, so a replica draws
 * exactly the numbers of a single-lattice context with the same seed and
 * replica id and follows its trajectory (up to summation order).
 * Per-site energy: -J sum_j s.s_j + K (s.e)^2 + zeeman_sign h (s.b)
 *                  - Kc (sx^4 + sy^4 + sz^4), h the field point's value
 * (signed), e the anisotropy axis and b the field axis. */
typedef struct {
  uint64_t seed;
  uint32_t replica;           /* Philox stream id (counter word 3) */
  uint32_t reserved;
  double temperature;
  double exchange;            /* J */
  double anisotropy;          /* uniaxial K */
  double cubic;               /* Kc */
} vg_heis_replica;

typedef struct {
  vg_lattice_desc lattice;    /* VG_CELL_BCC or VG_CELL_FCC */
  double anisotropy_axis[3];
  double field_axis[3];
  double zeeman_sign;         /* +1: the reference's per-site sign; -1: spins align with the field */
  int32_t precision;          /* VG_FP32 or VG_FP64 */
  int32_t proposal;           /* VG_PROPOSE_RANDOM or VG_PROPOSE_FLIP */
} vg_hbatch_desc;

/* Per (field point, replica), sums over the point's measured sweeps of:
 * 0 bond sum s_i.s_j, 1 sum (s.e)^2, 2 sum s.b, 3 sum (sx^4+sy^4+sz^4),
 * 4-6 Mx, My, Mz, 7 accepted moves, 8 |M|, 9 |M|^2, 10 E, 11 E^2, with
 * E = sum_i energy(i) (the reference's Compound total:
 * -2 J bond + K aniso + zeeman_sign h zeeman - Kc cubic). */
#define VG_HB_NSUMS 12

typedef struct vg_hbatch vg_hbatch;
typedef struct {
  int32_t n_replicas;
  int32_t n_classes;
  int64_t sites_per_replica;
  uint64_t sweep_index;
  int32_t sites_per_thread;    /* 4: float4 runs along x; 1: scalar */
  int32_t graph;               /* 1 if a field point is replayed as a CUDA graph */
  int64_t device_bytes;
} vg_hbatch_info;

int vg_hbatch_create(const vg_hbatch_desc* desc, const vg_heis_replica* replicas, int32_t n_replicas,
                     vg_hbatch** out);
int vg_hbatch_destroy(vg_hbatch* batch);
const char* vg_hbatch_last_error(const vg_hbatch* batch);
int vg_hbatch_get_info(const vg_hbatch* batch, vg_hbatch_info* out);
int vg_hbatch_get_stream(const vg_hbatch* batch, void** cuda_stream);
/* Every replica random, as vg_init_random of a context with its seed and id. */
int vg_hbatch_init_random(vg_hbatch* batch);
/* Replica state as n_sites x 3 doubles in the reference's site order. */
int vg_hbatch_set_replica(vg_hbatch* batch, int32_t replica, const double* xyz, int64_t n_sites);
int vg_hbatch_get_replica(vg_hbatch* batch, int32_t replica, double* xyz, int64_t n_sites);
/* For each of the n_points field values: relax_sweeps sweeps, then
 * measure_sweeps sweeps whose sums are accumulated (VG_HB_NSUMS per point
 * and replica).  A point is one CUDA graph launch. */
int vg_hbatch_run(vg_hbatch* batch, const double* fields, int32_t n_points, uint32_t relax_sweeps,
                  uint32_t measure_sweeps);
int vg_hbatch_run_async(vg_hbatch* batch, const double* fields, int32_t n_points, uint32_t relax_sweeps,
                        uint32_t measure_sweeps);
int vg_hbatch_synchronize(vg_hbatch* batch);
/* out[(point * n_replicas + replica) * VG_HB_NSUMS + k] of the last run. */
int vg_hbatch_point_sums(vg_hbatch* batch, double* out, int64_t capacity);
/* Mean device time of one sweep's colour passes (all replicas, update only,
 * field 0), over n_sweeps sweeps timed with CUDA events on the batch stream. */
int vg_hbatch_time_passes(vg_hbatch* batch, uint32_t n_sweeps, double* ms_per_sweep);

/* ------------------------------------------------------ no-alloc sweeps */
/* No counterpart in the reference.  n Ising flip-proposal sweeps of an sc
 * lattice (x a multiple of 32, even extents on periodic axes) that allocate
 * no memory, for callers that cannot call cudaMalloc: plugins whose host
 * framework owns all device memory through its own pool, code enqueueing
 * work while another party captures the stream into a CUDA graph, real-time
 * loops where an allocation could synchronise the device.  The caller owns
 * every buffer: class0 / class1 are the two checkerboard classes on the
 * device (uint8 0 = Down / 1 = Up, sites with (x+y+z)&1 == c, row-major
 * [z][y][x/2]) and sums_out (may be NULL) receives n_sweeps vg_sums rows.
 * zeeman is the per-site Zeeman coefficient (sign * |B| * orientation, the
 * field's z orientation folded in), so the rows cannot know the orientation:
 * their zeeman member is the sum of s.z (mz), which a context reports for a
 * field along +z; for a field along -z the context's zeeman member is -mz,
 * and callers forming energies multiply by the orientation themselves.  Work
 * is enqueued on cuda_stream (NULL = default stream); results are valid once
 * that stream has been synchronised.  Draws, spins and every other member of
 * the rows equal vg_sweeps on a context with the same seed and replica at
 * sweep index sweep0 (sweep0 + n_sweeps <= 2^32).  The per-block partial
 * sums live in a 2 MiB array inside the library (at most 2048 thread blocks
 * per colour pass; larger launches are rejected with VG_ERR_UNSUPPORTED);
 * every call shares it, so calls that overlap on the GPU race.  The first
 * call on a device looks up the array's address and keeps it for the rest of
 * the process: make it before any stream capture.  A device reset
 * (cudaDeviceReset, or the primary context being destroyed) moves the array
 * and the library cannot look it up again, so a process that resets a device
 * must not call this entry point on it afterwards. */
int vg_ising_sc_sweeps_noalloc(const vg_lattice_desc* lattice, double exchange, double zeeman, double temperature,
                               uint64_t seed, uint32_t replica, uint64_t sweep0, uint64_t n_sweeps,
                               uint8_t* class0, uint8_t* class1, double* sums_out, void* cuda_stream);

/* ------------------------------------------------------- host utilities */
/* Neighbour table of a lattice (nbr[i*zmax + k], -1 = absent) and its greedy
 * colouring; pass NULL buffers to query n and zmax. */
int vg_lattice_neighbours(const vg_lattice_desc* lattice, int32_t* nbr, int64_t capacity,
                          int64_t* n_sites, int32_t* zmax);
int vg_lattice_colouring(const vg_lattice_desc* lattice, int32_t* colour, int64_t capacity,
                         int32_t* n_colours);
/* Page-locked host buffers for fast host<->device copies. */
int vg_host_alloc(void** ptr, uint64_t bytes);
int vg_host_free(void* ptr);

#ifdef __cplusplus
}
#endif
#endif
