/*
 * vegas_oracle.h -- CPU oracle for the vegas Metropolis hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker, never the product:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs load it.
 * The GPU library (libvegas_gpu.so) never links or calls it.
 *
 * Two oracles live here:
 *
 *  (a) colour_cpu -- the GPU's own update order (colour-class passes over a
 *      greedy colouring of the neighbour list) with the same counter-based
 *      Philox4x32 draws (10 rounds; 7 for the Heisenberg update and the
 *      batched threshold planes), the same integer Delta-E index and the same
 *      acceptance-threshold table.  Ising results are bit-exact against the
 *      CUDA kernels; Heisenberg runs in FP64 and is compared with tolerances.
 *
 *  (b) ref_cpu -- a faithful restatement of the reference's single-threaded
 *      Metropolis: N random-site attempts per sweep, two per-site energy calls
 *      per attempt, accept if dE < 0 or u < exp(-dE/T), restore otherwise
 *      (src/integrator.rs:66-137), per-site energies with the reference's
 *      signs (src/energy.rs:45-257), the per-sweep state clone
 *      (src/machine.rs:91-101) and the CLI's per-sweep total_energy +
 *      magnetization (src/instrument.rs:133-141).  The reference draws from
 *      rand_pcg's Pcg64; this restatement uses the same PCG XSL-RR 128/64
 *      generator family but does not replicate the seeded stream (rand_core's
 *      seed expansion is in an absent dependency), so its parity with the GPU
 *      is statistical.
 *
 * Pinning: Philox4x32-10 is checked against the published Random123
 * known-answer vectors; the energy terms against every known answer in the
 * reference's own unit tests (src/energy.rs:292-376, src/state.rs:320-383).
 * The lattice geometry restates vegas-lattice 0.13 (absent from the reference
 * tree); its edge semantics are NOT pinned by any reference test.
 */
#ifndef VEGAS_ORACLE_H
#define VEGAS_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- Philox */
void vo_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
/* Philox4x32 with the given number of rounds (1..10); the batched
 * multi-spin-coded threshold planes use VO_MSC_ROUNDS, the Heisenberg
 * update draws (proposal and acceptance) VO_HEIS_ROUNDS.  Salmon et al.
 * (SC'11) report Philox4x32 passing TestU01's Crush batteries from 7
 * rounds on; initial states, Ising draws and exchange decisions keep 10. */
void vo_philox4x32_r(const uint32_t ctr[4], const uint32_t key[2], int rounds, uint32_t out[4]);
enum { VO_MSC_ROUNDS = 7, VO_HEIS_ROUNDS = 7 };

/* Draw-stream tags (bits 24..31 of the third counter word). */
enum {
  VO_TAG_ISING_ACCEPT = 1,
  VO_TAG_ISING_PROPOSE = 2,
  VO_TAG_HEIS = 3,
  VO_TAG_INIT_ISING = 4,
  VO_TAG_INIT_HEIS = 5
};

/* ---------------------------------------------------------------- lattice */
enum { VO_CELL_SC = 0, VO_CELL_BCC = 1, VO_CELL_FCC = 2 };

typedef struct {
  int32_t cell;           /* VO_CELL_* */
  int32_t nx, ny, nz;     /* unit cells along each axis (expand(x, y, z)) */
  int32_t pbc_x, pbc_y, pbc_z;
} vo_lattice;

int32_t vo_basis_size(int32_t cell);
int32_t vo_coordination(int32_t cell);
int64_t vo_num_sites(const vo_lattice* lat);
/* nbr[i*zmax + k] = k-th neighbour of site i (or -1).  Returns 0 on success. */
int vo_build_neighbours(const vo_lattice* lat, int32_t* nbr);
/* Greedy sequential colouring in site order.  Returns the colour count. */
int vo_greedy_colouring(int64_t n, int32_t zmax, const int32_t* nbr, int32_t* colour);
/* 1 if no neighbour pair shares a colour, else 0. */
int vo_colouring_valid(int64_t n, int32_t zmax, const int32_t* nbr, const int32_t* colour);

/* ------------------------------------------------ (a) colour_cpu: Ising */
enum { VO_PROPOSE_FLIP = 0, VO_PROPOSE_RANDOM = 1 };

/* Acceptance threshold: accept iff U < thr with U a 32-bit uniform integer.
 * thr >= 2^32 means "always" (dE <= 0). */
uint64_t vo_ising_threshold(double J, double hz, double T, int s, int nsum);

/* Runs nsweeps colour-class sweeps in place on spin[] (+1/-1, site order).
 * obs[2*t] = sum over bonds s_i s_j, obs[2*t+1] = sum s_i after sweep t. */
int vo_ising_colour_sweeps(int64_t n, int32_t zmax, const int32_t* nbr, const int32_t* colour,
                           int32_t ncolours, int8_t* spin, double J, double hz, double T,
                           int proposal, uint64_t seed, uint32_t replica, uint32_t sweep0,
                           int32_t nsweeps, int64_t* obs);

/* Random initial state (State::rand_with_size): spin[i] = +1 iff u < 0.5. */
void vo_ising_init(int64_t n, uint64_t seed, uint32_t replica, int8_t* spin);

/* --------------------------------------------- (a) colour_cpu: Heisenberg */
typedef struct {
  double J;               /* exchange constant (uniform) */
  double K;               /* uniaxial anisotropy strength, per-site +K (s.e)^2 */
  double axis[3];         /* anisotropy axis e */
  double hz;              /* per-site Zeeman coefficient: E_i += hz * (s . b) */
  double b[3];            /* field orientation b */
  double Kc;              /* cubic anisotropy (extension): E_i += -Kc (sx^4+sy^4+sz^4) */
  double T;
} vo_heis_params;

/* proposal uniform on the sphere from two 32-bit draws (Archimedes map). */
void vo_heis_proposal(uint32_t w0, uint32_t w1, double out[3]);
void vo_heis_init(int64_t n, uint64_t seed, uint32_t replica, double* spin /* n*3 */);
/* Single-site dE for replacing s by p given neighbour sum h (= sum_j s_j). */
double vo_heis_delta(const vo_heis_params* P, const double s[3], const double p[3], const double h[3]);
/* obs[8*t + 0..7] = {bond sum s_i.s_j, sum (s.e)^2, sum s.b, sum(sx^4+sy^4+sz^4), Mx, My, Mz, accepted} */
int vo_heis_colour_sweeps(int64_t n, int32_t zmax, const int32_t* nbr, const int32_t* colour,
                          int32_t ncolours, double* spin, const vo_heis_params* P, int proposal,
                          uint64_t seed, uint32_t replica, uint32_t sweep0, int32_t nsweeps,
                          double* obs);

/* Per-bond exchange constants (Exchange's CSR with arbitrary J_ij):
 * jb[i * zmax + k] is the constant of the bond to neighbour k of site i.
 * Ising: obs[2 t] = sum over bonds of J_ij s_i s_j, obs[2 t + 1] = M.
 * Heisenberg: P->J must be 1 (the constants carry the exchange); obs as
 * vo_heis_colour_sweeps with the bond sum weighted by J_ij. */
int vo_ising_colour_sweeps_bonds(int64_t n, int32_t zmax, const int32_t* nbr, const double* jb,
                                 const int32_t* colour, int32_t ncol, int8_t* spin, double hz, double T,
                                 int proposal, uint64_t seed, uint32_t replica, uint32_t sweep0, int32_t nsweeps,
                                 double* obs);
int vo_heis_colour_sweeps_bonds(int64_t n, int32_t zmax, const int32_t* nbr, const double* jb,
                                const int32_t* colour, int32_t ncol, double* spin, const vo_heis_params* P,
                                int proposal, uint64_t seed, uint32_t replica, uint32_t sweep0, int32_t nsweeps,
                                double* obs);

/* Wolff cluster steps with the GPU's draws (tags 9: source, 10: bonds).
 * obs[3 t .. 3 t + 2] = {bond sum, magnetisation, cluster size}. */
enum { VO_TAG_WOLFF_SOURCE = 9, VO_TAG_WOLFF_BOND = 10 };
int vo_wolff_steps(int64_t n, int32_t zmax, const int32_t* nbr, int8_t* spin, double J, double T, uint64_t seed,
                   uint32_t replica, uint32_t step0, int32_t nsteps, double* obs);

/* ------------------------------------------------ (b) ref_cpu (faithful) */
typedef struct {
  int32_t has_exchange; double J;
  int32_t has_anisotropy; double K; double axis[3];
  int32_t has_zeeman; double zeeman_sign;   /* +1 = reference per-site sign */
  int32_t has_gauge; double gauge;
  int32_t compound;       /* 1: total = sum_i energy(i) (Compound); 0: single term's own total */
} vo_hamiltonian;

typedef struct {
  uint64_t state_hi, state_lo, inc_hi, inc_lo;
} vo_pcg64;

void vo_pcg64_seed(vo_pcg64* rng, uint64_t seed);
uint64_t vo_pcg64_next(vo_pcg64* rng);

/* Runs nsweeps reference sweeps (N random-site attempts each).
 * spin_kind 0 = Ising (int8 +-1 in spin_i8), 1 = Heisenberg (double xyz in spin_f64).
 * b[3], bmag: thermostat field.  If measure, obs[2*t] = total energy and
 * obs[2*t+1] = |M| after sweep t (the CLI instruments' per-sweep work).
 * clone: copy the whole state every sweep as Machine::run does. */
int vo_ref_sweeps(int64_t n, int32_t zmax, const int32_t* nbr, int32_t spin_kind, int32_t proposal,
                  int8_t* spin_i8, double* spin_f64, const vo_hamiltonian* H, double T,
                  const double b[3], double bmag, vo_pcg64* rng, int32_t nsweeps, int32_t measure,
                  int32_t clone, double* obs);

/* Total energy and |M| with the reference's semantics. */
double vo_ref_total_energy(int64_t n, int32_t zmax, const int32_t* nbr, int32_t spin_kind,
                           const int8_t* spin_i8, const double* spin_f64, const vo_hamiltonian* H,
                           const double b[3], double bmag);
double vo_ref_magnetization(int64_t n, int32_t spin_kind, const int8_t* spin_i8, const double* spin_f64);
/* Hamiltonian::energy(i) of every site, the reference's per-site semantics. */
void vo_ref_site_energies(int64_t n, int32_t zmax, const int32_t* nbr, int32_t spin_kind, const int8_t* spin_i8,
                          const double* spin_f64, const vo_hamiltonian* H, const double b[3], double bmag,
                          double* out);

/* Independent reference chains on nthreads host threads (one lattice each),
 * for the multi-core CPU baseline: nwarm untimed sweeps, then nsweeps timed
 * ones.  Returns the timed attempted flips; *seconds receives the slowest
 * chain's timed sweep time (setup and warm-up excluded). */
int64_t vo_ref_parallel(const vo_lattice* lat, int32_t spin_kind, int32_t proposal,
                        const vo_hamiltonian* H, double T, double bmag, int32_t nwarm, int32_t nsweeps,
                        int32_t measure, int32_t nthreads, uint64_t seed, double* seconds);
/* The same chains walking a temperature schedule: nwarm untimed sweeps at
 * temps[0], then sweeps_per_temp timed sweeps at each temperature in turn,
 * the state carried over as CoolDown::run carries it (src/program.rs:182-214). */
int64_t vo_ref_parallel_ladder(const vo_lattice* lat, int32_t spin_kind, int32_t proposal,
                               const vo_hamiltonian* H, const double* temps, int32_t ntemps, double bmag,
                               int32_t nwarm, int32_t sweeps_per_temp, int32_t measure, int32_t nthreads,
                               uint64_t seed, double* seconds);

/* --------------------------------- (a) colour_cpu: batched multi-spin coding */
/* A replica group: n_rep replicas (a multiple of 32) of one sc lattice that
 * is periodic on every axis, or 2D (nz = 1, open z).  Replica r = 32 w + l is
 * lane l of replica word w; its random numbers come from the Philox stream of
 * word id (seg_base + w).  temperatures[i] is ladder entry i; replica r starts
 * at ladder entry r.  spins: n_rep x N int8 (+1/-1), site order. */
typedef struct {
  vo_lattice lat;
  int32_t n_rep;
  const double* temperatures;
  uint32_t seg_base;
  int8_t* spins;
  int32_t* tau;        /* ladder entry of each replica (in/out) */
} vo_msc_group;

enum { VO_TAG_MSC = 6, VO_TAG_MSC_INIT = 7, VO_TAG_EXCHANGE = 8 };

void vo_msc_init(vo_msc_group* g, uint64_t seed);
/* rounds x every sweeps; after each round the per-replica anti-aligned bond
 * and up-spin counts are recorded (obs[round][rep][2], may be NULL) and, if
 * exchange, adjacent ladder entries swap with probability
 * min(1, exp((b_i - b_j)(E_i - E_j))).  accepted[i] counts swaps of (i, i+1). */
int vo_msc_run(vo_msc_group* groups, int32_t n_groups, double J, uint64_t seed, uint32_t sweep0, uint32_t round0,
               int32_t every, int32_t rounds, int32_t exchange, int64_t* obs, int64_t* accepted);

/* ------------------------------------------------ programs and statistics */
/* CoolDown temperatures (src/program.rs:202-211).  Returns count (<= cap). */
int32_t vo_cooldown_temperatures(double tmax, double tmin, double rate, double* out, int32_t cap);
/* HysteresisLoop field magnitudes, all three legs (src/program.rs:302-332). */
int32_t vo_hysteresis_fields(double max_field, double step, double* out, int32_t cap);
/* Accumulator (src/accumulator.rs:42-63): out = {mean, variance, binder}. */
void vo_accumulate(const double* x, int64_t n, double out[3]);

#ifdef __cplusplus
}
#endif
#endif
