/*
 * vegas_oracle.c -- CPU oracle for the vegas Metropolis hot path.
 *
 * TEST INFRASTRUCTURE ONLY (see vegas_oracle.h): the checker for the CUDA
 * kernels and the timed CPU baseline.  Nothing in the product links it.
 *
 * Pinned against the Random123 Philox4x32-10 known-answer vectors and the
 * known answers of the reference's unit tests; lattice edge semantics
 * (vegas-lattice 0.13, absent from the reference tree) are unpinned.
 */
#include "vegas_oracle.h"

#include <math.h>
#include <pthread.h>
#include <unistd.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

/* ================================================================ Philox */
/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), as published with the
 * Random123 library: 10 rounds of two 32x32->64 multiplies, Weyl key bumps. */
void vo_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  vo_philox4x32_r(ctr, key, 10, out);
}

/* Philox4x32 with `rounds` rounds (the first rounds of the 10-round
 * function: same multipliers and Weyl key increments). */
void vo_philox4x32_r(const uint32_t ctr[4], const uint32_t key[2], int rounds, uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < rounds; ++r) {
    if (r) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
    uint32_t n1 = (uint32_t)p1;
    uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
    uint32_t n3 = (uint32_t)p0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

static void draw(uint64_t seed, uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t out[4]) {
  uint32_t ctr[4] = {c0, c1, c2, c3};
  uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  vo_philox4x32_10(ctr, key, out);
}

/* byte k (0..15) of a 128-bit Philox block */
static inline uint32_t block_byte(const uint32_t w[4], int k) {
  return (w[k >> 2] >> (8 * (k & 3))) & 0xFFu;
}

/* =============================================================== lattice */
/* Positions in half-cell integer units.  Basis and nearest-neighbour vectors
 * of the cubic unit cells (Lattice::sc/bcc/fcc(1.0), src/input.rs:296-302). */
static const int SC_BASIS[1][3] = {{0, 0, 0}};
static const int BCC_BASIS[2][3] = {{0, 0, 0}, {1, 1, 1}};
static const int FCC_BASIS[4][3] = {{0, 0, 0}, {1, 1, 0}, {1, 0, 1}, {0, 1, 1}};
static const int SC_NN[6][3] = {{2, 0, 0}, {-2, 0, 0}, {0, 2, 0}, {0, -2, 0}, {0, 0, 2}, {0, 0, -2}};
static const int BCC_NN[8][3] = {{1, 1, 1},   {-1, 1, 1},  {1, -1, 1},  {-1, -1, 1},
                                 {1, 1, -1},  {-1, 1, -1}, {1, -1, -1}, {-1, -1, -1}};
static const int FCC_NN[12][3] = {{1, 1, 0},  {-1, 1, 0},  {1, -1, 0},  {-1, -1, 0},
                                  {1, 0, 1},  {-1, 0, 1},  {1, 0, -1},  {-1, 0, -1},
                                  {0, 1, 1},  {0, -1, 1},  {0, 1, -1},  {0, -1, -1}};

int32_t vo_basis_size(int32_t cell) { return cell == VO_CELL_SC ? 1 : cell == VO_CELL_BCC ? 2 : 4; }
int32_t vo_coordination(int32_t cell) { return cell == VO_CELL_SC ? 6 : cell == VO_CELL_BCC ? 8 : 12; }

int64_t vo_num_sites(const vo_lattice* L) {
  return (int64_t)L->nx * L->ny * L->nz * vo_basis_size(L->cell);
}

static const int (*basis_of(int cell))[3] {
  return cell == VO_CELL_SC ? SC_BASIS : cell == VO_CELL_BCC ? BCC_BASIS : FCC_BASIS;
}
static const int (*nn_of(int cell))[3] {
  return cell == VO_CELL_SC ? SC_NN : cell == VO_CELL_BCC ? BCC_NN : FCC_NN;
}

static int basis_index(int cell, int hx, int hy, int hz) {
  const int(*B)[3] = basis_of(cell);
  int nb = vo_basis_size(cell);
  for (int b = 0; b < nb; ++b)
    if (B[b][0] == hx && B[b][1] == hy && B[b][2] == hz) return b;
  return -1;
}

static int floordiv2(int v) { return v >= 0 ? v / 2 : -((-v + 1) / 2); }

/* Neighbour k of every site: the site at position + d_k, wrapped on periodic
 * axes, absent (-1) across an open axis (drop_x/y/z, src/input.rs:311-320). */
int vo_build_neighbours(const vo_lattice* L, int32_t* nbr) {
  int nb = vo_basis_size(L->cell), z = vo_coordination(L->cell);
  const int(*B)[3] = basis_of(L->cell);
  const int(*D)[3] = nn_of(L->cell);
  int ext[3] = {L->nx, L->ny, L->nz};
  int per[3] = {L->pbc_x, L->pbc_y, L->pbc_z};
  for (int a = 0; a < 3; ++a) {
    if (ext[a] < 1) return -1;
    if (per[a] && ext[a] < 2 && L->cell == VO_CELL_SC) return -2; /* self-bond */
  }
  int64_t i = 0;
  for (int cz = 0; cz < L->nz; ++cz)
    for (int cy = 0; cy < L->ny; ++cy)
      for (int cx = 0; cx < L->nx; ++cx)
        for (int b = 0; b < nb; ++b, ++i) {
          int c[3] = {cx, cy, cz};
          for (int k = 0; k < z; ++k) {
            int q[3], cell[3], h[3], ok = 1;
            for (int a = 0; a < 3; ++a) {
              q[a] = 2 * c[a] + B[b][a] + D[k][a];
              cell[a] = floordiv2(q[a]);
              h[a] = q[a] - 2 * cell[a];
              if (cell[a] < 0 || cell[a] >= ext[a]) {
                if (!per[a]) ok = 0;
                cell[a] = ((cell[a] % ext[a]) + ext[a]) % ext[a];
              }
            }
            int bb = basis_index(L->cell, h[0], h[1], h[2]);
            if (!ok || bb < 0) {
              nbr[i * z + k] = -1;
            } else {
              nbr[i * z + k] =
                  (int32_t)((((int64_t)cell[2] * L->ny + cell[1]) * L->nx + cell[0]) * nb + bb);
            }
          }
        }
  return 0;
}

int vo_greedy_colouring(int64_t n, int32_t zmax, const int32_t* nbr, int32_t* colour) {
  int ncol = 0;
  for (int64_t i = 0; i < n; ++i) colour[i] = -1;
  for (int64_t i = 0; i < n; ++i) {
    uint64_t used = 0;
    for (int k = 0; k < zmax; ++k) {
      int32_t j = nbr[i * zmax + k];
      if (j >= 0 && j != i && colour[j] >= 0) used |= 1ull << colour[j];
    }
    int c = 0;
    while (used & (1ull << c)) ++c;
    colour[i] = c;
    if (c + 1 > ncol) ncol = c + 1;
  }
  return ncol;
}

int vo_colouring_valid(int64_t n, int32_t zmax, const int32_t* nbr, const int32_t* colour) {
  for (int64_t i = 0; i < n; ++i)
    for (int k = 0; k < zmax; ++k) {
      int32_t j = nbr[i * zmax + k];
      if (j >= 0 && colour[j] == colour[i]) return 0;
    }
  return 1;
}

/* rank of each site within its colour class (ascending site order) */
static int64_t* class_ranks(int64_t n, const int32_t* colour, int32_t ncol) {
  int64_t* rank = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
  int64_t cnt[64] = {0};
  for (int64_t i = 0; i < n; ++i) rank[i] = cnt[colour[i]]++;
  (void)ncol;
  return rank;
}

/* ========================================================== Ising oracle */
/* dE of flipping s given the neighbour sum: E_i(s) = -J s nsum + hz s
 * (Exchange::energy src/energy.rs:194-206, Zeeman::energy :147-151), so
 * dE = E_i(-s) - E_i(s).  Reference accept rule (src/integrator.rs:127-133):
 * accept if dE < 0, else if u < exp(-dE/T).  With u = U / 2^32 for a 32-bit
 * integer U, u < p  <=>  U < ceil(p 2^32).  dE <= 0 always accepts. */
uint64_t vo_ising_threshold(double J, double hz, double T, int s, int nsum) {
  double e_old = -J * (double)s * (double)nsum + hz * (double)s;
  double e_new = -J * (double)(-s) * (double)nsum + hz * (double)(-s);
  double de = e_new - e_old;
  if (de <= 0.0) return 1ull << 32;
  double p = exp(-de / T);
  double x = ceil(p * 4294967296.0);
  if (x >= 4294967296.0) return 1ull << 32;
  if (x <= 0.0) return 0;
  return (uint64_t)x;
}

/* 32-bit acceptance uniform of class entry j: byte (j & 15) of four Philox
 * blocks, most significant byte first (digit d = 0..3 in counter word 2). */
static uint32_t ising_uniform(uint64_t seed, uint32_t replica, uint32_t sweep, int colour, int64_t j) {
  uint32_t u = 0;
  for (int d = 0; d < 4; ++d) {
    uint32_t w[4];
    draw(seed, (uint32_t)(j >> 4), sweep, ((uint32_t)VO_TAG_ISING_ACCEPT << 24) | ((uint32_t)colour << 8) | (uint32_t)d,
         replica, w);
    u = (u << 8) | block_byte(w, (int)(j & 15));
  }
  return u;
}

void vo_ising_init(int64_t n, uint64_t seed, uint32_t replica, int8_t* spin) {
  for (int64_t i = 0; i < n; ++i) {
    uint32_t w[4];
    draw(seed, (uint32_t)(i >> 4), 0, (uint32_t)VO_TAG_INIT_ISING << 24, replica, w);
    spin[i] = block_byte(w, (int)(i & 15)) < 128 ? 1 : -1;
  }
}

int vo_ising_colour_sweeps(int64_t n, int32_t zmax, const int32_t* nbr, const int32_t* colour,
                           int32_t ncol, int8_t* spin, double J, double hz, double T, int proposal,
                           uint64_t seed, uint32_t replica, uint32_t sweep0, int32_t nsweeps,
                           int64_t* obs) {
  if (T < 2.220446049250313e-16) T = 2.220446049250313e-16; /* Thermostat clamp */
  int64_t* rank = class_ranks(n, colour, ncol);
  /* thr[s][nsum + zmax] */
  uint64_t* thr = (uint64_t*)malloc(sizeof(uint64_t) * 2 * (2 * zmax + 1));
  for (int s = 0; s < 2; ++s)
    for (int ns = -zmax; ns <= zmax; ++ns)
      thr[s * (2 * zmax + 1) + ns + zmax] = vo_ising_threshold(J, hz, T, s ? 1 : -1, ns);
  for (int32_t t = 0; t < nsweeps; ++t) {
    uint32_t sweep = sweep0 + (uint32_t)t;
    int64_t bond = 0, mag = 0;
    for (int c = 0; c < ncol; ++c) {
      for (int64_t i = 0; i < n; ++i) {
        if (colour[i] != c) continue;
        int64_t j = rank[i];
        int s = spin[i];
        int nsum = 0;
        for (int k = 0; k < zmax; ++k) {
          int32_t q = nbr[i * zmax + k];
          if (q >= 0) nsum += spin[q];
        }
        int propose_flip = 1;
        if (proposal == VO_PROPOSE_RANDOM) {
          uint32_t w[4];
          draw(seed, (uint32_t)(j >> 4), sweep, ((uint32_t)VO_TAG_ISING_PROPOSE << 24) | ((uint32_t)c << 8),
               replica, w);
          int up = block_byte(w, (int)(j & 15)) < 128;
          propose_flip = (up ? 1 : -1) != s;
        }
        if (propose_flip) {
          uint64_t th = thr[(s > 0) * (2 * zmax + 1) + nsum + zmax];
          int accept = th >= (1ull << 32) ? 1 : (uint64_t)ising_uniform(seed, replica, sweep, c, j) < th;
          if (accept) spin[i] = (int8_t)(-s);
        }
        int sn = spin[i];
        mag += sn;
        int low = 0;
        for (int k = 0; k < zmax; ++k) {
          int32_t q = nbr[i * zmax + k];
          if (q >= 0 && colour[q] < c) low += spin[q];
        }
        bond += (int64_t)sn * low;
      }
    }
    if (obs) {
      obs[2 * t] = bond;
      obs[2 * t + 1] = mag;
    }
  }
  free(thr);
  free(rank);
  return 0;
}

/* Per-bond exchange constants (Exchange's CSR with arbitrary J_ij,
 * src/energy.rs:169-206): jb[i * zmax + k] is the constant of the bond to
 * neighbour k of site i.  hJ = sum_k jb s_k in k order; dE of s -> -s is
 * (-(-s) hJ + hz (-s)) - (-s hJ + hz s), thr = ceil(exp(-dE / T) 2^32) as in
 * vo_ising_threshold; obs[2 t] = sum over bonds of J_ij s_i s_j (each bond
 * once, from its higher-colour end), obs[2 t + 1] = magnetisation. */
static uint64_t thr_of(double de, double T) {
  if (de <= 0.0) return 1ull << 32;
  double x = ceil(exp(-de / T) * 4294967296.0);
  if (x >= 4294967296.0) return 1ull << 32;
  if (x <= 0.0) return 0;
  return (uint64_t)x;
}

int vo_ising_colour_sweeps_bonds(int64_t n, int32_t zmax, const int32_t* nbr, const double* jb,
                                 const int32_t* colour, int32_t ncol, int8_t* spin, double hz, double T,
                                 int proposal, uint64_t seed, uint32_t replica, uint32_t sweep0, int32_t nsweeps,
                                 double* obs) {
  if (T < 2.220446049250313e-16) T = 2.220446049250313e-16;
  int64_t* rank = class_ranks(n, colour, ncol);
  for (int32_t t = 0; t < nsweeps; ++t) {
    uint32_t sweep = sweep0 + (uint32_t)t;
    double bond = 0.0;
    int64_t mag = 0;
    for (int c = 0; c < ncol; ++c) {
      for (int64_t i = 0; i < n; ++i) {
        if (colour[i] != c) continue;
        int64_t j = rank[i];
        int s = spin[i];
        double hj = 0.0;
        for (int k = 0; k < zmax; ++k) {
          int32_t q = nbr[i * zmax + k];
          if (q >= 0) hj += jb[i * zmax + k] * (double)spin[q];
        }
        int propose_flip = 1;
        if (proposal == VO_PROPOSE_RANDOM) {
          uint32_t w[4];
          draw(seed, (uint32_t)(j >> 4), sweep, ((uint32_t)VO_TAG_ISING_PROPOSE << 24) | ((uint32_t)c << 8),
               replica, w);
          int up = block_byte(w, (int)(j & 15)) < 128;
          propose_flip = (up ? 1 : -1) != s;
        }
        if (propose_flip) {
          const double sd = (double)s;
          const double e_old = -sd * hj + hz * sd;
          const double e_new = -(-sd) * hj + hz * (-sd);
          uint64_t th = thr_of(e_new - e_old, T);
          int accept = th >= (1ull << 32) ? 1 : (uint64_t)ising_uniform(seed, replica, sweep, c, j) < th;
          if (accept) spin[i] = (int8_t)(-s);
        }
        int sn = spin[i];
        mag += sn;
        double low = 0.0;
        for (int k = 0; k < zmax; ++k) {
          int32_t q = nbr[i * zmax + k];
          if (q >= 0 && colour[q] < c) low += jb[i * zmax + k] * (double)spin[q];
        }
        bond += (double)sn * low;
      }
    }
    if (obs) {
      obs[2 * t] = bond;
      obs[2 * t + 1] = (double)mag;
    }
  }
  free(rank);
  return 0;
}

/* Wolff cluster steps (WolffIntegrator::step, src/integrator.rs:140-230)
 * with the GPU's draws: source = (Philox(step, 0, TAG_WOLFF_SOURCE << 24,
 * replica).w0 * n) >> 32; the bond k of site i to j = nbr[i][k] (occurrence
 * o among the repeated bonds of that pair) is active iff Philox(min(i, j),
 * max(i, j), TAG_WOLFF_BOND << 24 | o << 20 | replica, step).w0 < thr, thr =
 * ceil((1 - exp(-2 J / T)) 2^32).  The cluster is grown with a queue as the
 * reference does; obs[3 t .. 3 t + 2] = {bond sum, magnetisation, cluster
 * size} after step t. */
int vo_wolff_steps(int64_t n, int32_t zmax, const int32_t* nbr, int8_t* spin, double J, double T, uint64_t seed,
                   uint32_t replica, uint32_t step0, int32_t nsteps, double* obs) {
  if (T < 2.220446049250313e-16) T = 2.220446049250313e-16;
  const double p = 1.0 - exp(-2.0 * J / T);
  uint64_t thr = 0;
  if (p > 0.0) {
    double x = ceil(p * 4294967296.0);
    thr = x >= 4294967296.0 ? (1ull << 32) : (uint64_t)x;
  }
  uint8_t* in = (uint8_t*)malloc((size_t)n);
  int64_t* queue = (int64_t*)malloc(sizeof(int64_t) * (size_t)n);
  for (int32_t t = 0; t < nsteps; ++t) {
    uint32_t step = step0 + (uint32_t)t;
    uint32_t w[4];
    draw(seed, step, 0, (uint32_t)VO_TAG_WOLFF_SOURCE << 24, replica, w);
    int64_t src = (int64_t)(((uint64_t)w[0] * (uint64_t)n) >> 32);
    memset(in, 0, (size_t)n);
    int8_t ref = spin[src];
    int64_t head = 0, tail = 0;
    queue[tail++] = src;
    in[src] = 1;
    while (head < tail) {
      int64_t i = queue[head++];
      for (int k = 0; k < zmax; ++k) {
        int32_t j = nbr[i * zmax + k];
        if (j < 0 || in[j] || spin[j] != ref) continue;
        uint32_t o = 0;
        for (int q = 0; q < k; ++q) o += nbr[i * zmax + q] == j;
        uint32_t lo = (uint32_t)(i < j ? i : j), hi = (uint32_t)(i < j ? j : i);
        draw(seed, lo, hi, ((uint32_t)VO_TAG_WOLFF_BOND << 24) | (o << 20) | (replica & 0xFFFFFu), step, w);
        if ((uint64_t)w[0] < thr) {
          in[j] = 1;
          queue[tail++] = j;
        }
      }
    }
    for (int64_t i = 0; i < n; ++i)
      if (in[i]) spin[i] = (int8_t)(-spin[i]);
    if (obs) {
      int64_t bond = 0, mag = 0;
      for (int64_t i = 0; i < n; ++i) {
        mag += spin[i];
        for (int k = 0; k < zmax; ++k) {
          int32_t j = nbr[i * zmax + k];
          if (j > i) bond += (int64_t)spin[i] * spin[j];
        }
      }
      obs[3 * t] = (double)bond;
      obs[3 * t + 1] = (double)mag;
      obs[3 * t + 2] = (double)tail;
    }
  }
  free(in);
  free(queue);
  return 0;
}

/* ===================================================== Heisenberg oracle */
/* Uniform point on S^2 (Archimedes: z uniform in (-1,1), azimuth uniform):
 * z = (2k + 1 - 2^24) / 2^24 with k = w0 >> 8, azimuth = pi * (w1 >> 8) / 2^23.
 * Stands in for util::marsaglia (src/util.rs:21-34): same distribution,
 * no rejection loop. */
void vo_heis_proposal(uint32_t w0, uint32_t w1, double out[3]) {
  double z = ((double)(w0 >> 8) * 2.0 + 1.0 - 16777216.0) * (1.0 / 16777216.0);
  double t = (double)(w1 >> 8) * (1.0 / 8388608.0);
  double r = sqrt((1.0 - z) * (1.0 + z));
  out[0] = r * cos(M_PI * t);
  out[1] = r * sin(M_PI * t);
  out[2] = z;
}

void vo_heis_init(int64_t n, uint64_t seed, uint32_t replica, double* spin) {
  for (int64_t i = 0; i < n; ++i) {
    uint32_t w[4];
    draw(seed, (uint32_t)i, 0, (uint32_t)VO_TAG_INIT_HEIS << 24, replica, w);
    vo_heis_proposal(w[0], w[1], spin + 3 * i);
  }
}

static inline double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static inline double quart(const double* s) {
  double x2 = s[0] * s[0], y2 = s[1] * s[1], z2 = s[2] * s[2];
  return x2 * x2 + y2 * y2 + z2 * z2;
}

double vo_heis_delta(const vo_heis_params* P, const double s[3], const double p[3], const double h[3]) {
  double d[3] = {p[0] - s[0], p[1] - s[1], p[2] - s[2]};
  double pe = dot3(p, P->axis), se = dot3(s, P->axis);
  double de = -P->J * dot3(d, h);
  de += P->K * (pe * pe - se * se);
  de += P->hz * dot3(d, P->b);
  de += -P->Kc * (quart(p) - quart(s));
  return de;
}

/* jb = NULL: uniform exchange P->J; else per-bond constants jb[i * zmax + k]
 * weigh the neighbour field and the bond sum, and P->J must be 1. */
static int heis_sweeps(int64_t n, int32_t zmax, const int32_t* nbr, const double* jb, const int32_t* colour,
                       int32_t ncol, double* spin, const vo_heis_params* P, int proposal, uint64_t seed,
                       uint32_t replica, uint32_t sweep0, int32_t nsweeps, double* obs) {
  double T = P->T < 2.220446049250313e-16 ? 2.220446049250313e-16 : P->T;
  int64_t* rank = class_ranks(n, colour, ncol);
  for (int32_t t = 0; t < nsweeps; ++t) {
    uint32_t sweep = sweep0 + (uint32_t)t;
    double acc[8] = {0};
    for (int c = 0; c < ncol; ++c) {
      for (int64_t i = 0; i < n; ++i) {
        if (colour[i] != c) continue;
        int64_t j = rank[i];
        double* s = spin + 3 * i;
        double h[3] = {0, 0, 0};
        for (int k = 0; k < zmax; ++k) {
          int32_t q = nbr[i * zmax + k];
          if (q >= 0) {
            const double wq = jb ? jb[i * zmax + k] : 1.0;
            h[0] += wq * spin[3 * q];
            h[1] += wq * spin[3 * q + 1];
            h[2] += wq * spin[3 * q + 2];
          }
        }
        uint32_t w[4];
        {
          const uint32_t ctr[4] = {(uint32_t)j, sweep, ((uint32_t)VO_TAG_HEIS << 24) | ((uint32_t)c << 8), replica};
          const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
          vo_philox4x32_r(ctr, key, VO_HEIS_ROUNDS, w);
        }
        double p[3];
        if (proposal == VO_PROPOSE_RANDOM) {
          vo_heis_proposal(w[0], w[1], p);
        } else {
          p[0] = -s[0]; p[1] = -s[1]; p[2] = -s[2];
        }
        double de = vo_heis_delta(P, s, p, h);
        double u = (double)(w[2] >> 8) * (1.0 / 16777216.0);
        if (de <= 0.0 || u < exp(-de / T)) {
          s[0] = p[0]; s[1] = p[1]; s[2] = p[2];
          acc[7] += 1.0;
        }
        double low[3] = {0, 0, 0};
        for (int k = 0; k < zmax; ++k) {
          int32_t q = nbr[i * zmax + k];
          if (q >= 0 && colour[q] < c) {
            const double wq = jb ? jb[i * zmax + k] : 1.0;
            low[0] += wq * spin[3 * q];
            low[1] += wq * spin[3 * q + 1];
            low[2] += wq * spin[3 * q + 2];
          }
        }
        double se = dot3(s, P->axis);
        acc[0] += dot3(s, low);
        acc[1] += se * se;
        acc[2] += dot3(s, P->b);
        acc[3] += quart(s);
        acc[4] += s[0];
        acc[5] += s[1];
        acc[6] += s[2];
      }
    }
    if (obs) memcpy(obs + 8 * t, acc, sizeof(acc));
  }
  free(rank);
  return 0;
}

int vo_heis_colour_sweeps(int64_t n, int32_t zmax, const int32_t* nbr, const int32_t* colour,
                          int32_t ncol, double* spin, const vo_heis_params* P, int proposal,
                          uint64_t seed, uint32_t replica, uint32_t sweep0, int32_t nsweeps,
                          double* obs) {
  return heis_sweeps(n, zmax, nbr, NULL, colour, ncol, spin, P, proposal, seed, replica, sweep0, nsweeps, obs);
}

int vo_heis_colour_sweeps_bonds(int64_t n, int32_t zmax, const int32_t* nbr, const double* jb,
                                const int32_t* colour, int32_t ncol, double* spin, const vo_heis_params* P,
                                int proposal, uint64_t seed, uint32_t replica, uint32_t sweep0, int32_t nsweeps,
                                double* obs) {
  return heis_sweeps(n, zmax, nbr, jb, colour, ncol, spin, P, proposal, seed, replica, sweep0, nsweeps, obs);
}

/* ============================================================== ref_cpu */
/* PCG XSL-RR 128/64 (O'Neill 2014), the generator family of rand_pcg::Pcg64
 * (src/main.rs:27-30).  The 128-bit LCG multiplier is PCG's default. */
typedef unsigned __int128 u128;
static u128 pcg_state(const vo_pcg64* r) { return ((u128)r->state_hi << 64) | r->state_lo; }
static u128 pcg_inc(const vo_pcg64* r) { return ((u128)r->inc_hi << 64) | r->inc_lo; }
static const u128 PCG_MULT = (((u128)0x2360ED051FC65DA4ull) << 64) | 0x4385DF649FCCF645ull;

static uint64_t splitmix64(uint64_t* x) {
  uint64_t z = (*x += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

void vo_pcg64_seed(vo_pcg64* r, uint64_t seed) {
  uint64_t x = seed;
  r->state_hi = splitmix64(&x);
  r->state_lo = splitmix64(&x);
  r->inc_hi = splitmix64(&x);
  r->inc_lo = splitmix64(&x) | 1ull;
}

uint64_t vo_pcg64_next(vo_pcg64* r) {
  u128 s = pcg_state(r);
  u128 ns = s * PCG_MULT + pcg_inc(r);
  r->state_hi = (uint64_t)(ns >> 64);
  r->state_lo = (uint64_t)ns;
  uint64_t xsl = (uint64_t)(s >> 64) ^ (uint64_t)s;
  unsigned rot = (unsigned)(s >> 122);
  return (xsl >> rot) | (xsl << ((64 - rot) & 63));
}

/* Uniform::new(0, n).sample: unbiased widening-multiply rejection (Lemire). */
static uint64_t pcg_below(vo_pcg64* r, uint64_t range) {
  u128 m = (u128)vo_pcg64_next(r) * range;
  uint64_t lo = (uint64_t)m;
  if (lo < range) {
    uint64_t thresh = (0 - range) % range;
    while (lo < thresh) {
      m = (u128)vo_pcg64_next(r) * range;
      lo = (uint64_t)m;
    }
  }
  return (uint64_t)(m >> 64);
}
/* rng.random::<f64>(): 53 random bits in [0, 1). */
static double pcg_f64(vo_pcg64* r) { return (double)(vo_pcg64_next(r) >> 11) * (1.0 / 9007199254740992.0); }
/* Uniform::new(-1.0, 1.0).sample: 52 random bits scaled into [-1, 1). */
static double pcg_sym(vo_pcg64* r) {
  double u = (double)(vo_pcg64_next(r) >> 12) * (1.0 / 4503599627370496.0);
  return u * 2.0 - 1.0;
}

/* util::marsaglia (src/util.rs:21-34) */
static void marsaglia(vo_pcg64* r, double* out) {
  for (;;) {
    double x1 = pcg_sym(r), x2 = pcg_sym(r);
    double q = x1 * x1 + x2 * x2;
    if (q >= 1.0) continue;
    double root = sqrt(1.0 - x1 * x1 - x2 * x2);
    out[0] = 2.0 * x1 * root;
    out[1] = 2.0 * x2 * root;
    out[2] = 1.0 - 2.0 * q;
    return;
  }
}

/* Exchange::from_lattice (src/energy.rs:176-187) builds a CSR with J on
 * (s, t) and (t, s); to_csr sums duplicates and sorts columns.  The row walk
 * of Exchange::energy (src/energy.rs:194-206) therefore visits each distinct
 * neighbour once, in ascending order, with J times its multiplicity. */
typedef struct {
  int64_t* off;
  int32_t* col;
  double* w;
} csr_t;

static int cmp_i32(const void* a, const void* b) {
  int32_t x = *(const int32_t*)a, y = *(const int32_t*)b;
  return (x > y) - (x < y);
}

static csr_t build_csr(int64_t n, int32_t zmax, const int32_t* nbr, double J) {
  csr_t m;
  m.off = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n + 1));
  m.col = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n * zmax + 1));
  m.w = (double*)malloc(sizeof(double) * (size_t)(n * zmax + 1));
  int32_t tmp[64];
  int64_t pos = 0;
  for (int64_t i = 0; i < n; ++i) {
    m.off[i] = pos;
    int cnt = 0;
    for (int k = 0; k < zmax; ++k)
      if (nbr[i * zmax + k] >= 0) tmp[cnt++] = nbr[i * zmax + k];
    qsort(tmp, (size_t)cnt, sizeof(int32_t), cmp_i32);
    for (int k = 0; k < cnt; ++k) {
      if (pos > m.off[i] && m.col[pos - 1] == tmp[k]) {
        m.w[pos - 1] += J;
      } else {
        m.col[pos] = tmp[k];
        m.w[pos] = J;
        ++pos;
      }
    }
  }
  m.off[n] = pos;
  return m;
}

static void free_csr(csr_t* m) {
  free(m->off);
  free(m->col);
  free(m->w);
}

typedef struct {
  int32_t kind;
  const csr_t* X;
  const vo_hamiltonian* H;
  double b[3];
  double bmag;
} ref_ctx;

/* Compound::energy (src/energy.rs:248-257) over the terms in the order the
 * hamiltonian! macro nests them: ((Exchange + Anisotropy) + Zeeman) + Gauge. */
static double site_energy(const ref_ctx* R, const int8_t* si, const double* sf, int64_t i) {
  const vo_hamiltonian* H = R->H;
  double e = 0.0;
  int first = 1;
  if (H->has_exchange) {
    double acc = 0.0;
    for (int64_t p = R->X->off[i]; p < R->X->off[i + 1]; ++p) {
      int32_t q = R->X->col[p];
      double d = R->kind == 0 ? (double)(si[i] * si[q]) : dot3(sf + 3 * i, sf + 3 * q);
      acc = acc + (-R->X->w[p] * d);
    }
    e = acc;
    first = 0;
  }
  if (H->has_anisotropy) {
    double d = R->kind == 0 ? (double)si[i] * (H->axis[2] >= 0 ? 1.0 : -1.0) : dot3(sf + 3 * i, H->axis);
    double a = d * d * H->K;
    e = first ? a : e + a;
    first = 0;
  }
  if (H->has_zeeman) {
    double d = R->kind == 0 ? (double)si[i] * (R->b[2] >= 0 ? 1.0 : -1.0) : dot3(sf + 3 * i, R->b);
    double zz = H->zeeman_sign * d * R->bmag;
    e = first ? zz : e + zz;
    first = 0;
  }
  if (H->has_gauge) {
    e = first ? H->gauge : e + H->gauge;
  }
  return e;
}

static double total_energy(const ref_ctx* R, int64_t n, const int8_t* si, const double* sf) {
  const vo_hamiltonian* H = R->H;
  if (H->compound) {
    /* Hamiltonian::total_energy default (src/energy.rs:55-59) */
    double s = 0.0;
    for (int64_t i = 0; i < n; ++i) s += site_energy(R, si, sf, i);
    return s;
  }
  if (H->has_exchange) { /* Exchange::total_energy (src/energy.rs:208-213) */
    double s = 0.0;
    for (int64_t i = 0; i < n; ++i) s = s + site_energy(R, si, sf, i);
    return s / 2.0;
  }
  if (H->has_anisotropy) { /* UniaxialAnisotropy::total_energy omits K (src/energy.rs:114-120) */
    double s = 0.0;
    for (int64_t i = 0; i < n; ++i) {
      double d = R->kind == 0 ? 1.0 : dot3(sf + 3 * i, H->axis);
      s += d * d;
    }
    return s;
  }
  if (H->has_zeeman) { /* Zeeman::total_energy (src/energy.rs:153-160) */
    double s = 0.0;
    for (int64_t i = 0; i < n; ++i)
      s += R->kind == 0 ? (double)si[i] * (R->b[2] >= 0 ? 1.0 : -1.0) : dot3(sf + 3 * i, R->b);
    return -R->bmag * s;
  }
  if (H->has_gauge) return (double)n * H->gauge;
  return 0.0;
}

/* State::magnetization().magnitude() (src/state.rs:291-297, :86-92, :150-160, :219-221) */
double vo_ref_magnetization(int64_t n, int32_t kind, const int8_t* si, const double* sf) {
  if (kind == 0) {
    double m = 0.0;
    for (int64_t i = 0; i < n; ++i) m += (double)si[i];
    return fabs(m);
  }
  double m[3] = {0, 0, 0};
  for (int64_t i = 0; i < n; ++i) {
    m[0] += sf[3 * i];
    m[1] += sf[3 * i + 1];
    m[2] += sf[3 * i + 2];
  }
  double mag = sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]);
  return fabs(mag) < 2.220446049250313e-16 ? 0.0 : mag;
}

double vo_ref_total_energy(int64_t n, int32_t zmax, const int32_t* nbr, int32_t kind, const int8_t* si,
                           const double* sf, const vo_hamiltonian* H, const double b[3], double bmag) {
  csr_t X = build_csr(n, zmax, nbr, H->J);
  ref_ctx R = {kind, &X, H, {b[0], b[1], b[2]}, fabs(bmag)};
  double e = total_energy(&R, n, si, sf);
  free_csr(&X);
  return e;
}

/* Hamiltonian::energy(i) of every site (src/energy.rs:45-52; Compound sums
 * the terms' site energies, src/energy.rs:254-256). */
void vo_ref_site_energies(int64_t n, int32_t zmax, const int32_t* nbr, int32_t kind, const int8_t* si,
                          const double* sf, const vo_hamiltonian* H, const double b[3], double bmag, double* out) {
  csr_t X = build_csr(n, zmax, nbr, H->J);
  ref_ctx R = {kind, &X, H, {b[0], b[1], b[2]}, fabs(bmag)};
  for (int64_t i = 0; i < n; ++i) out[i] = site_energy(&R, si, sf, i);
  free_csr(&X);
}

/* MetropolisFlipIntegrator / MetropolisIntegrator::step
 * (src/integrator.rs:66-92, :113-137) followed by the instruments. */
int vo_ref_sweeps(int64_t n, int32_t zmax, const int32_t* nbr, int32_t kind, int32_t proposal,
                  int8_t* si, double* sf, const vo_hamiltonian* H, double T, const double b[3], double bmag,
                  vo_pcg64* rng, int32_t nsweeps, int32_t measure, int32_t clone, double* obs) {
  if (T < 2.220446049250313e-16) T = 2.220446049250313e-16;
  csr_t X = build_csr(n, zmax, nbr, H->J);
  ref_ctx R = {kind, &X, H, {b[0], b[1], b[2]}, fabs(bmag)};
  int8_t* ci = NULL;
  double* cf = NULL;
  if (clone) {
    if (kind == 0) ci = (int8_t*)malloc((size_t)n);
    else cf = (double*)malloc(sizeof(double) * 3 * (size_t)n);
  }
  for (int32_t t = 0; t < nsweeps; ++t) {
    if (clone) { /* self.state.clone() every sweep (src/machine.rs:91-93) */
      if (kind == 0) memcpy(ci, si, (size_t)n);
      else memcpy(cf, sf, sizeof(double) * 3 * (size_t)n);
    }
    for (int64_t a = 0; a < n; ++a) {
      int64_t site = (int64_t)pcg_below(rng, (uint64_t)n);
      double old_e = site_energy(&R, si, sf, site);
      int8_t old_i = 0;
      double old_f[3] = {0, 0, 0};
      if (kind == 0) {
        old_i = si[site];
        if (proposal == VO_PROPOSE_FLIP) si[site] = (int8_t)(-old_i);
        else si[site] = pcg_f64(rng) < 0.5 ? 1 : -1; /* IsingSpin::rand (src/state.rs:76-84) */
      } else {
        memcpy(old_f, sf + 3 * site, sizeof(old_f));
        if (proposal == VO_PROPOSE_FLIP) {
          sf[3 * site] = -old_f[0];
          sf[3 * site + 1] = -old_f[1];
          sf[3 * site + 2] = -old_f[2];
        } else {
          marsaglia(rng, sf + 3 * site);
        }
      }
      double new_e = site_energy(&R, si, sf, site);
      double delta = new_e - old_e;
      if (delta < 0.0) continue;
      if (pcg_f64(rng) < exp(-delta / T)) continue;
      if (kind == 0) si[site] = old_i;
      else memcpy(sf + 3 * site, old_f, sizeof(old_f));
    }
    if (measure && obs) {
      obs[2 * t] = total_energy(&R, n, si, sf);
      obs[2 * t + 1] = vo_ref_magnetization(n, kind, si, sf);
    }
  }
  free(ci);
  free(cf);
  free_csr(&X);
  return 0;
}

typedef struct {
  const vo_lattice* lat;
  int32_t kind, proposal, nsweeps, measure, nwarm;
  const vo_hamiltonian* H;
  const double* temps; /* nsweeps measured sweeps at each of ntemps temperatures */
  int32_t ntemps;
  double bmag;
  uint64_t seed;
  int64_t flips;
  pthread_barrier_t* start;
  double seconds;
} par_job;

static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static void* par_worker(void* arg) {
  par_job* J = (par_job*)arg;
  int64_t n = vo_num_sites(J->lat);
  int32_t z = vo_coordination(J->lat->cell);
  int32_t* nbr = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n * z));
  vo_build_neighbours(J->lat, nbr);
  vo_pcg64 rng;
  vo_pcg64_seed(&rng, J->seed);
  int8_t* si = NULL;
  double* sf = NULL;
  if (J->kind == 0) {
    si = (int8_t*)malloc((size_t)n);
    for (int64_t i = 0; i < n; ++i) si[i] = pcg_f64(&rng) < 0.5 ? 1 : -1;
  } else {
    sf = (double*)malloc(sizeof(double) * 3 * (size_t)n);
    for (int64_t i = 0; i < n; ++i) marsaglia(&rng, sf + 3 * i);
  }
  double* obs = (double*)malloc(sizeof(double) * 2 * (size_t)(J->nsweeps > 0 ? J->nsweeps : 1));
  double b[3] = {0, 0, 1};
  if (J->nwarm > 0) { /* untimed warm-up sweeps at the first temperature */
    double* wo = (double*)malloc(sizeof(double) * 2 * (size_t)J->nwarm);
    vo_ref_sweeps(n, z, nbr, J->kind, J->proposal, si, sf, J->H, J->temps[0], b, J->bmag, &rng, J->nwarm,
                  J->measure, 1, wo);
    free(wo);
  }
  pthread_barrier_wait(J->start); /* all chains set up: time the sweeps only */
  double t0 = now_s();
  for (int32_t k = 0; k < J->ntemps; ++k) /* the chain carries its state from temperature to temperature */
    vo_ref_sweeps(n, z, nbr, J->kind, J->proposal, si, sf, J->H, J->temps[k], b, J->bmag, &rng, J->nsweeps,
                  J->measure, 1, obs);
  J->seconds = now_s() - t0;
  J->flips = n * (int64_t)J->nsweeps * J->ntemps;
  free(obs);
  free(si);
  free(sf);
  free(nbr);
  return NULL;
}

int64_t vo_ref_parallel(const vo_lattice* lat, int32_t kind, int32_t proposal, const vo_hamiltonian* H,
                        double T, double bmag, int32_t nwarm, int32_t nsweeps, int32_t measure, int32_t nthreads,
                        uint64_t seed, double* seconds) {
  return vo_ref_parallel_ladder(lat, kind, proposal, H, &T, 1, bmag, nwarm, nsweeps, measure, nthreads, seed,
                                seconds);
}

int64_t vo_ref_parallel_ladder(const vo_lattice* lat, int32_t kind, int32_t proposal, const vo_hamiltonian* H,
                               const double* temps, int32_t ntemps, double bmag, int32_t nwarm,
                               int32_t sweeps_per_temp, int32_t measure, int32_t nthreads, uint64_t seed,
                               double* seconds) {
  const int32_t nsweeps = sweeps_per_temp;
  if (nthreads < 1) nthreads = 1;
  if (ntemps < 1) return 0;
  pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)nthreads);
  par_job* jobs = (par_job*)malloc(sizeof(par_job) * (size_t)nthreads);
  pthread_barrier_t start;
  pthread_barrier_init(&start, NULL, (unsigned)nthreads);
  for (int k = 0; k < nthreads; ++k) {
    par_job j = {lat, kind, proposal, nsweeps, measure, nwarm, H, temps, ntemps, bmag, seed + 7919ull * (uint64_t)k,
                 0, &start, 0.0};
    jobs[k] = j;
    pthread_create(&th[k], NULL, par_worker, &jobs[k]);
  }
  int64_t total = 0;
  double worst = 0.0;
  for (int k = 0; k < nthreads; ++k) {
    pthread_join(th[k], NULL);
    total += jobs[k].flips;
    if (jobs[k].seconds > worst) worst = jobs[k].seconds;
  }
  pthread_barrier_destroy(&start);
  if (seconds) *seconds = worst;
  free(th);
  free(jobs);
  return total;
}

/* ======================================== batched multi-spin-coded oracle */
/* The GPU packs 32 replicas per 32-bit word; here every replica is its own
 * int8 lattice, updated with the draws the packed kernel uses:
 *   plane p (0 = most significant) of class entry j in sweep t, colour c, is
 *   word (p & 3) of Philox(j, t, TAG_MSC<<24 | c<<8 | p>>2, word id);
 *   replica lane l's 32-bit uniform takes bit l of plane p as its bit 31-p.
 * A move with dE = 2 J (z - 2 n_anti) <= 0 always accepts; otherwise accept
 * iff U < thr(T, n_anti) (the Ising threshold rule above). */
static int msc_z(const vo_lattice* L) { return L->nz == 1 && !L->pbc_z ? 4 : 6; }

void vo_msc_init(vo_msc_group* g, uint64_t seed) {
  int64_t n = vo_num_sites(&g->lat);
  for (int32_t r = 0; r < g->n_rep; ++r) {
    uint32_t word = g->seg_base + (uint32_t)(r / 32), lane = (uint32_t)(r % 32);
    for (int64_t i = 0; i < n; ++i) {
      uint32_t w[4];
      draw(seed, (uint32_t)i, 0, (uint32_t)VO_TAG_MSC_INIT << 24, word, w);
      g->spins[(int64_t)r * n + i] = (w[0] >> lane) & 1u ? 1 : -1;
    }
    g->tau[r] = r;
  }
}

/* Decision of "U < th" for lane `lane` of the 32-replica word `word` at class
 * entry j: U's bit 31-p is bit `lane` of plane p, plane p is word p & 3 of
 * the Philox4x32-7 block p >> 2 (drawn once per word and kept in blk / have, so
 * the 32 lanes of a word share their blocks).  Planes are compared most
 * significant first, and only until they differ, which gives exactly
 * U < th. */
static int msc_accept(uint64_t seed, uint32_t word, uint32_t sweep, int colour, int64_t j, uint32_t lane,
                      uint64_t th, uint32_t blk[8][4], int have[8]) {
  for (int p = 0; p < 32; ++p) {
    const int b = p >> 2;
    if (!have[b]) {
      const uint32_t ctr[4] = {(uint32_t)j, sweep, ((uint32_t)VO_TAG_MSC << 24) | ((uint32_t)colour << 8) | (uint32_t)b,
                               word};
      const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
      vo_philox4x32_r(ctr, key, VO_MSC_ROUNDS, blk[b]);
      have[b] = 1;
    }
    const uint32_t ub = (blk[b][p & 3] >> lane) & 1u;
    const uint32_t tb = (uint32_t)(th >> (31 - p)) & 1u;
    if (ub != tb) return ub < tb;
  }
  return 0; /* U == th */
}

/* One colour pass of one replica group over the class entries of colour c,
 * the sites split across host threads (sites of one colour share no bond). */
typedef struct {
  vo_msc_group* g;
  int64_t n, lo, hi;
  const int32_t* nbr;
  const int32_t* colour;
  const int64_t* rank;
  const uint64_t* thr;
  int z, c;
  uint64_t seed;
  uint32_t sweep;
} msc_pass_job;

static void* msc_pass_worker(void* arg) {
  const msc_pass_job* J = (const msc_pass_job*)arg;
  vo_msc_group* g = J->g;
  for (int64_t i = J->lo; i < J->hi; ++i) {
    if (J->colour[i] != J->c) continue;
    for (int32_t w0 = 0; w0 < g->n_rep; w0 += 32) {
      uint32_t blk[8][4];
      int have[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      for (int32_t r = w0; r < w0 + 32; ++r) {
        int8_t* sp = g->spins + (int64_t)r * J->n;
        int na = 0;
        for (int k = 0; k < 6; ++k) {
          const int32_t q = J->nbr[i * 6 + k];
          if (q >= 0 && sp[q] != sp[i]) ++na;
        }
        const uint64_t th = J->thr[(size_t)g->tau[r] * (J->z + 1) + na];
        const int acc = th >= (1ull << 32) ? 1
                                           : msc_accept(J->seed, g->seg_base + (uint32_t)(r / 32), J->sweep, J->c,
                                                        J->rank[i], (uint32_t)(r % 32), th, blk, have);
        if (acc) sp[i] = (int8_t)(-sp[i]);
      }
    }
  }
  return NULL;
}

static int host_threads(void) {
  long k = sysconf(_SC_NPROCESSORS_ONLN);
  return k < 1 ? 1 : k > 32 ? 32 : (int)k;
}

static void msc_pass(vo_msc_group* g, int64_t n, const int32_t* nbr, const int32_t* colour, const int64_t* rank,
                     const uint64_t* thr, int z, int c, uint64_t seed, uint32_t sweep) {
  int nt = host_threads();
  if (n < 4096) nt = 1;
  pthread_t th[32];
  msc_pass_job jobs[32];
  for (int k = 0; k < nt; ++k) {
    msc_pass_job J = {g, n, n * k / nt, n * (k + 1) / nt, nbr, colour, rank, thr, z, c, seed, sweep};
    jobs[k] = J;
  }
  for (int k = 1; k < nt; ++k) pthread_create(&th[k], NULL, msc_pass_worker, &jobs[k]);
  msc_pass_worker(&jobs[0]);
  for (int k = 1; k < nt; ++k) pthread_join(th[k], NULL);
}

int vo_msc_run(vo_msc_group* G, int32_t ng, double J, uint64_t seed, uint32_t sweep0, uint32_t round0, int32_t every,
               int32_t rounds, int32_t exchange, int64_t* obs, int64_t* accepted) {
  int64_t total_rep = 0;
  for (int32_t gi = 0; gi < ng; ++gi) total_rep += G[gi].n_rep;
  int64_t rep_off = 0;
  for (int32_t gi = 0; gi < ng; ++gi) {
    vo_msc_group* g = &G[gi];
    const int64_t n = vo_num_sites(&g->lat);
    const int z = msc_z(&g->lat);
    int32_t* nbr = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n * 6));
    vo_build_neighbours(&g->lat, nbr);
    int32_t* colour = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
    const int ncol = vo_greedy_colouring(n, 6, nbr, colour);
    int64_t* rank = class_ranks(n, colour, ncol);
    uint64_t* thr = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)g->n_rep * (size_t)(z + 1));
    for (int32_t i = 0; i < g->n_rep; ++i) {
      const double T = g->temperatures[i] < 2.220446049250313e-16 ? 2.220446049250313e-16 : g->temperatures[i];
      for (int na = 0; na <= z; ++na) thr[(size_t)i * (z + 1) + na] = vo_ising_threshold(J, 0.0, T, 1, z - 2 * na);
    }
    int32_t* rep_at = (int32_t*)malloc(sizeof(int32_t) * (size_t)g->n_rep);
    double* E = (double*)malloc(sizeof(double) * (size_t)g->n_rep);
    for (int32_t r = 0; r < g->n_rep; ++r) rep_at[g->tau[r]] = r;
    for (int32_t rd = 0; rd < rounds; ++rd) {
      for (int32_t t = 0; t < every; ++t) {
        const uint32_t sweep = sweep0 + (uint32_t)(rd * every + t);
        for (int c = 0; c < 2; ++c) msc_pass(g, n, nbr, colour, rank, thr, z, c, seed, sweep);
      }
      /* measurement: anti-aligned bonds and up spins of every replica */
      for (int32_t r = 0; r < g->n_rep; ++r) {
        const int8_t* sp = g->spins + (int64_t)r * n;
        int64_t anti2 = 0, ups = 0, nb2 = 0;
        for (int64_t i = 0; i < n; ++i) {
          ups += sp[i] > 0;
          for (int k = 0; k < 6; ++k) {
            const int32_t q = nbr[i * 6 + k];
            if (q >= 0) {
              ++nb2;
              anti2 += sp[q] != sp[i];
            }
          }
        }
        E[r] = -J * (double)(nb2 / 2 - 2 * (anti2 / 2));
        if (obs) {
          int64_t* o = obs + ((int64_t)rd * total_rep + rep_off + r) * 2;
          o[0] = anti2 / 2;
          o[1] = ups;
        }
      }
      /* replica exchange between adjacent ladder entries (i, i+1) */
      if (exchange) {
        const uint32_t round = round0 + (uint32_t)rd;
        for (int32_t i = (int32_t)(round & 1u); i + 1 < g->n_rep; i += 2) {
          const int32_t r1 = rep_at[i], r2 = rep_at[i + 1];
          const double x = (1.0 / g->temperatures[i] - 1.0 / g->temperatures[i + 1]) * (E[r1] - E[r2]);
          uint32_t w[4];
          draw(seed, (uint32_t)i, round, ((uint32_t)VO_TAG_EXCHANGE << 24) | (uint32_t)gi, 0, w);
          const double u = (double)w[0] * (1.0 / 4294967296.0);
          if (x >= 0.0 || u < exp(x)) {
            rep_at[i] = r2;
            rep_at[i + 1] = r1;
            g->tau[r1] = i + 1;
            g->tau[r2] = i;
            if (accepted) accepted[rep_off + i] += 1;
          }
        }
      }
    }
    free(E);
    free(rep_at);
    free(thr);
    free(rank);
    free(colour);
    free(nbr);
    rep_off += g->n_rep;
  }
  return 0;
}

/* ================================================ programs and statistics */
int32_t vo_cooldown_temperatures(double tmax, double tmin, double rate, double* out, int32_t cap) {
  int32_t n = 0;
  double t = tmax;
  for (;;) {
    if (n < cap) out[n] = t;
    ++n;
    t -= rate;
    if (t < tmin) break;
  }
  return n;
}

int32_t vo_hysteresis_fields(double max_field, double step, double* out, int32_t cap) {
  int32_t n = 0;
  double m = 0.0;
  for (;;) {
    if (n < cap) out[n] = m;
    ++n;
    m += step;
    if (m > max_field) break;
  }
  for (;;) {
    if (n < cap) out[n] = m;
    ++n;
    m -= step;
    if (m < -max_field) break;
  }
  for (;;) {
    if (n < cap) out[n] = m;
    ++n;
    m += step;
    if (m > max_field) break;
  }
  return n;
}

void vo_accumulate(const double* x, int64_t n, double out[3]) {
  double s = 0.0, s2 = 0.0, s4 = 0.0;
  for (int64_t i = 0; i < n; ++i) {
    s += x[i];
    s2 += x[i] * x[i];
    s4 += x[i] * x[i] * x[i] * x[i];
  }
  double mean = s / (double)n;
  out[0] = mean;
  out[1] = s2 / (double)n - mean * mean;
  out[2] = 1.0 - (s4 / (double)n) / (3.0 * (s2 / (double)n) * (s2 / (double)n));
}
