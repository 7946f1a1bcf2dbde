"""CPU oracle for the vegas Metropolis hot path -- TEST INFRASTRUCTURE ONLY.

This package is the checker.  Only ``tests/``, ``__graft_entry__.smoke()`` and
the CPU-baseline legs of ``bench.py`` may import it; the product (the CUDA
library and its host mirror) never does.

It wraps ``oracle/build/libvegas_oracle.so`` (built from ``vegas_oracle.c`` by
``build()``):

* colour_cpu -- the GPU's colour-class update order with the same Philox
  draws (bit-exact for Ising, FP64 for Heisenberg);
* ref_cpu -- a faithful restatement of the reference's random-site
  Metropolis (src/integrator.rs:66-137) with its energy semantics
  (src/energy.rs:45-257) and per-sweep measurement (src/instrument.rs:133-141);
* the CoolDown / HysteresisLoop schedules (src/program.rs:182-335) and the
  Accumulator statistics (src/accumulator.rs:42-63).
"""
from __future__ import annotations

import ctypes as C  # noqa: N812

import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "build", "libvegas_oracle.so")

CELL = {"sc": 0, "bcc": 1, "fcc": 2}
PROPOSE_FLIP, PROPOSE_RANDOM = 0, 1


def build() -> str:
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


class Lattice(C.Structure):
    _fields_ = [("cell", C.c_int32), ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
                ("pbc_x", C.c_int32), ("pbc_y", C.c_int32), ("pbc_z", C.c_int32)]


class HeisParams(C.Structure):
    _fields_ = [("J", C.c_double), ("K", C.c_double), ("axis", C.c_double * 3), ("hz", C.c_double),
                ("b", C.c_double * 3), ("Kc", C.c_double), ("T", C.c_double)]


class Hamiltonian(C.Structure):
    _fields_ = [("has_exchange", C.c_int32), ("J", C.c_double),
                ("has_anisotropy", C.c_int32), ("K", C.c_double), ("axis", C.c_double * 3),
                ("has_zeeman", C.c_int32), ("zeeman_sign", C.c_double),
                ("has_gauge", C.c_int32), ("gauge", C.c_double),
                ("compound", C.c_int32)]


class MscGroup(C.Structure):
    _fields_ = [("lat", Lattice), ("n_rep", C.c_int32), ("temperatures", C.POINTER(C.c_double)),
                ("seg_base", C.c_uint32), ("spins", C.POINTER(C.c_int8)), ("tau", C.POINTER(C.c_int32))]


class Pcg64(C.Structure):
    _fields_ = [("state_hi", C.c_uint64), ("state_lo", C.c_uint64),
                ("inc_hi", C.c_uint64), ("inc_lo", C.c_uint64)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        P = C.POINTER
        L.vo_philox4x32_10.argtypes = [P(C.c_uint32), P(C.c_uint32), P(C.c_uint32)]
        L.vo_philox4x32_r.argtypes = [P(C.c_uint32), P(C.c_uint32), C.c_int, P(C.c_uint32)]
        L.vo_num_sites.argtypes = [P(Lattice)]
        L.vo_num_sites.restype = C.c_int64
        L.vo_coordination.argtypes = [C.c_int32]
        L.vo_coordination.restype = C.c_int32
        L.vo_build_neighbours.argtypes = [P(Lattice), P(C.c_int32)]
        L.vo_greedy_colouring.argtypes = [C.c_int64, C.c_int32, P(C.c_int32), P(C.c_int32)]
        L.vo_colouring_valid.argtypes = [C.c_int64, C.c_int32, P(C.c_int32), P(C.c_int32)]
        L.vo_ising_threshold.argtypes = [C.c_double, C.c_double, C.c_double, C.c_int, C.c_int]
        L.vo_ising_threshold.restype = C.c_uint64
        L.vo_ising_colour_sweeps.argtypes = [C.c_int64, C.c_int32, P(C.c_int32), P(C.c_int32), C.c_int32,
                                             P(C.c_int8), C.c_double, C.c_double, C.c_double, C.c_int,
                                             C.c_uint64, C.c_uint32, C.c_uint32, C.c_int32, P(C.c_int64)]
        L.vo_ising_init.argtypes = [C.c_int64, C.c_uint64, C.c_uint32, P(C.c_int8)]
        L.vo_heis_proposal.argtypes = [C.c_uint32, C.c_uint32, P(C.c_double)]
        L.vo_heis_init.argtypes = [C.c_int64, C.c_uint64, C.c_uint32, P(C.c_double)]
        L.vo_heis_delta.argtypes = [P(HeisParams), P(C.c_double), P(C.c_double), P(C.c_double)]
        L.vo_heis_delta.restype = C.c_double
        L.vo_heis_colour_sweeps.argtypes = [C.c_int64, C.c_int32, P(C.c_int32), P(C.c_int32), C.c_int32,
                                            P(C.c_double), P(HeisParams), C.c_int, C.c_uint64, C.c_uint32,
                                            C.c_uint32, C.c_int32, P(C.c_double)]
        L.vo_ising_colour_sweeps_bonds.argtypes = [C.c_int64, C.c_int32, P(C.c_int32), P(C.c_double),
                                                   P(C.c_int32), C.c_int32, P(C.c_int8), C.c_double, C.c_double,
                                                   C.c_int, C.c_uint64, C.c_uint32, C.c_uint32, C.c_int32,
                                                   P(C.c_double)]
        L.vo_heis_colour_sweeps_bonds.argtypes = [C.c_int64, C.c_int32, P(C.c_int32), P(C.c_double),
                                                  P(C.c_int32), C.c_int32, P(C.c_double), P(HeisParams), C.c_int,
                                                  C.c_uint64, C.c_uint32, C.c_uint32, C.c_int32, P(C.c_double)]
        L.vo_wolff_steps.argtypes = [C.c_int64, C.c_int32, P(C.c_int32), P(C.c_int8), C.c_double, C.c_double,
                                     C.c_uint64, C.c_uint32, C.c_uint32, C.c_int32, P(C.c_double)]
        L.vo_pcg64_seed.argtypes = [P(Pcg64), C.c_uint64]
        L.vo_pcg64_next.argtypes = [P(Pcg64)]
        L.vo_pcg64_next.restype = C.c_uint64
        L.vo_ref_sweeps.argtypes = [C.c_int64, C.c_int32, P(C.c_int32), C.c_int32, C.c_int32, P(C.c_int8),
                                    P(C.c_double), P(Hamiltonian), C.c_double, P(C.c_double), C.c_double,
                                    P(Pcg64), C.c_int32, C.c_int32, C.c_int32, P(C.c_double)]
        L.vo_ref_total_energy.argtypes = [C.c_int64, C.c_int32, P(C.c_int32), C.c_int32, P(C.c_int8),
                                          P(C.c_double), P(Hamiltonian), P(C.c_double), C.c_double]
        L.vo_ref_total_energy.restype = C.c_double
        L.vo_ref_site_energies.argtypes = [C.c_int64, C.c_int32, P(C.c_int32), C.c_int32, P(C.c_int8),
                                           P(C.c_double), P(Hamiltonian), P(C.c_double), C.c_double, P(C.c_double)]
        L.vo_ref_site_energies.restype = None
        L.vo_ref_magnetization.argtypes = [C.c_int64, C.c_int32, P(C.c_int8), P(C.c_double)]
        L.vo_ref_magnetization.restype = C.c_double
        L.vo_ref_parallel.argtypes = [P(Lattice), C.c_int32, C.c_int32, P(Hamiltonian), C.c_double, C.c_double,
                                      C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_uint64, P(C.c_double)]
        L.vo_ref_parallel.restype = C.c_int64
        L.vo_ref_parallel_ladder.argtypes = [P(Lattice), C.c_int32, C.c_int32, P(Hamiltonian), P(C.c_double),
                                             C.c_int32, C.c_double, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                             C.c_uint64, P(C.c_double)]
        L.vo_ref_parallel_ladder.restype = C.c_int64
        L.vo_cooldown_temperatures.argtypes = [C.c_double, C.c_double, C.c_double, P(C.c_double), C.c_int32]
        L.vo_cooldown_temperatures.restype = C.c_int32
        L.vo_hysteresis_fields.argtypes = [C.c_double, C.c_double, P(C.c_double), C.c_int32]
        L.vo_hysteresis_fields.restype = C.c_int32
        L.vo_accumulate.argtypes = [P(C.c_double), C.c_int64, P(C.c_double)]
        L.vo_msc_init.argtypes = [P(MscGroup), C.c_uint64]
        L.vo_msc_run.argtypes = [P(MscGroup), C.c_int32, C.c_double, C.c_uint64, C.c_uint32, C.c_uint32, C.c_int32,
                                 C.c_int32, C.c_int32, P(C.c_int64), P(C.c_int64)]
        _lib = L
    return _lib


def _p(a, ct):
    return a.ctypes.data_as(C.POINTER(ct))


def philox(ctr, key, rounds=10):
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    if rounds == 10:
        lib().vo_philox4x32_10(c, k, o)
    else:
        lib().vo_philox4x32_r(c, k, rounds, o)
    return list(o)


MSC_ROUNDS = 7  # Philox rounds of the batched threshold planes
HEIS_ROUNDS = 7  # Philox rounds of the Heisenberg update draws


def lattice(cell="sc", nx=4, ny=4, nz=4, pbc=(True, True, True)) -> Lattice:
    return Lattice(CELL[cell], nx, ny, nz, int(pbc[0]), int(pbc[1]), int(pbc[2]))


class Graph:
    """Neighbour table + greedy colouring of a lattice, as the oracle builds them."""

    def __init__(self, lat: Lattice):
        L = lib()
        self.lat = lat
        self.n = int(L.vo_num_sites(C.byref(lat)))
        self.zmax = int(L.vo_coordination(lat.cell))
        self.nbr = np.empty(self.n * self.zmax, dtype=np.int32)
        rc = L.vo_build_neighbours(C.byref(lat), _p(self.nbr, C.c_int32))
        if rc != 0:
            raise ValueError(f"unsupported lattice (code {rc})")
        self.colour = np.empty(self.n, dtype=np.int32)
        self.ncolours = int(L.vo_greedy_colouring(self.n, self.zmax, _p(self.nbr, C.c_int32),
                                                   _p(self.colour, C.c_int32)))

    def neighbours(self) -> np.ndarray:
        return self.nbr.reshape(self.n, self.zmax)

    def colouring_valid(self, colour=None) -> bool:
        col = self.colour if colour is None else np.ascontiguousarray(colour, dtype=np.int32)
        return bool(lib().vo_colouring_valid(self.n, self.zmax, _p(self.nbr, C.c_int32), _p(col, C.c_int32)))

    # ---- colour_cpu (bit-exact GPU update order)
    def ising_init(self, seed, replica=0):
        s = np.empty(self.n, dtype=np.int8)
        lib().vo_ising_init(self.n, seed, replica, _p(s, C.c_int8))
        return s

    def ising_sweeps(self, spin, J, hz, T, seed, sweep0, nsweeps, replica=0, proposal=PROPOSE_FLIP):
        spin = np.ascontiguousarray(spin, dtype=np.int8).copy()
        obs = np.zeros((max(nsweeps, 1), 2), dtype=np.int64)
        lib().vo_ising_colour_sweeps(self.n, self.zmax, _p(self.nbr, C.c_int32), _p(self.colour, C.c_int32),
                                     self.ncolours, _p(spin, C.c_int8), J, hz, T, proposal, seed, replica,
                                     sweep0, nsweeps, _p(obs, C.c_int64))
        return spin, obs[:nsweeps]

    def heis_init(self, seed, replica=0):
        s = np.empty((self.n, 3), dtype=np.float64)
        lib().vo_heis_init(self.n, seed, replica, _p(s, C.c_double))
        return s

    def heis_sweeps(self, spin, params: HeisParams, seed, sweep0, nsweeps, replica=0, proposal=PROPOSE_RANDOM):
        spin = np.ascontiguousarray(spin, dtype=np.float64).copy()
        obs = np.zeros((max(nsweeps, 1), 8), dtype=np.float64)
        lib().vo_heis_colour_sweeps(self.n, self.zmax, _p(self.nbr, C.c_int32), _p(self.colour, C.c_int32),
                                    self.ncolours, _p(spin, C.c_double), C.byref(params), proposal, seed,
                                    replica, sweep0, nsweeps, _p(obs, C.c_double))
        return spin, obs[:nsweeps]

    # ---- per-bond exchange constants (jb: n x zmax, entries of absent neighbours ignored)
    def ising_sweeps_bonds(self, spin, jb, hz, T, seed, sweep0, nsweeps, replica=0, proposal=PROPOSE_FLIP):
        spin = np.ascontiguousarray(spin, dtype=np.int8).copy()
        jb = np.ascontiguousarray(jb, dtype=np.float64).reshape(self.n, self.zmax)
        obs = np.zeros((max(nsweeps, 1), 2), dtype=np.float64)
        lib().vo_ising_colour_sweeps_bonds(self.n, self.zmax, _p(self.nbr, C.c_int32), _p(jb, C.c_double),
                                           _p(self.colour, C.c_int32), self.ncolours, _p(spin, C.c_int8), hz, T,
                                           proposal, seed, replica, sweep0, nsweeps, _p(obs, C.c_double))
        return spin, obs[:nsweeps]

    def heis_sweeps_bonds(self, spin, jb, params: HeisParams, seed, sweep0, nsweeps, replica=0,
                          proposal=PROPOSE_RANDOM):
        spin = np.ascontiguousarray(spin, dtype=np.float64).copy()
        jb = np.ascontiguousarray(jb, dtype=np.float64).reshape(self.n, self.zmax)
        obs = np.zeros((max(nsweeps, 1), 8), dtype=np.float64)
        lib().vo_heis_colour_sweeps_bonds(self.n, self.zmax, _p(self.nbr, C.c_int32), _p(jb, C.c_double),
                                          _p(self.colour, C.c_int32), self.ncolours, _p(spin, C.c_double),
                                          C.byref(params), proposal, seed, replica, sweep0, nsweeps,
                                          _p(obs, C.c_double))
        return spin, obs[:nsweeps]

    def wolff_steps(self, spin, J, T, seed, step0, nsteps, replica=0):
        """Wolff cluster steps with the GPU's draws; obs rows (bond sum, M, cluster size)."""
        spin = np.ascontiguousarray(spin, dtype=np.int8).copy()
        obs = np.zeros((max(nsteps, 1), 3), dtype=np.float64)
        lib().vo_wolff_steps(self.n, self.zmax, _p(self.nbr, C.c_int32), _p(spin, C.c_int8), J, T, seed, replica,
                             step0, nsteps, _p(obs, C.c_double))
        return spin, obs[:nsteps]

    def symmetric_bonds(self, rng, values=(0.5, 1.0, 1.5)):
        """Random symmetric per-bond constants drawn from `values`
        (J_ij = J_ji for every bond, duplicates of a pair share one value)."""
        nb = self.neighbours()
        jb = np.zeros((self.n, self.zmax))
        for i in range(self.n):
            for k in range(self.zmax):
                t = int(nb[i, k])
                if t < 0 or jb[i, k] != 0.0:
                    continue
                v = float(rng.choice(values))
                for kk in range(self.zmax):
                    if nb[i, kk] == t:
                        jb[i, kk] = v
                for kk in range(self.zmax):
                    if nb[t, kk] == i:
                        jb[t, kk] = v
        return jb

    # ---- ref_cpu (faithful restatement of the reference)
    def ref_sweeps(self, kind, spin, H: Hamiltonian, T, nsweeps, rng: Pcg64, b=(0.0, 0.0, 1.0), bmag=0.0,
                   proposal=PROPOSE_FLIP, measure=True, clone=True):
        bb = (C.c_double * 3)(*b)
        obs = np.zeros((max(nsweeps, 1), 2), dtype=np.float64)
        if kind == 0:
            si = np.ascontiguousarray(spin, dtype=np.int8).copy()
            sf = np.zeros(3, dtype=np.float64)
        else:
            si = np.zeros(1, dtype=np.int8)
            sf = np.ascontiguousarray(spin, dtype=np.float64).copy()
        lib().vo_ref_sweeps(self.n, self.zmax, _p(self.nbr, C.c_int32), kind, proposal, _p(si, C.c_int8),
                            _p(sf, C.c_double), C.byref(H), T, bb, bmag, C.byref(rng), nsweeps, int(measure),
                            int(clone), _p(obs, C.c_double))
        return (si if kind == 0 else sf), obs[:nsweeps]

    def ref_total_energy(self, kind, spin, H: Hamiltonian, b=(0.0, 0.0, 1.0), bmag=0.0):
        bb = (C.c_double * 3)(*b)
        if kind == 0:
            si = np.ascontiguousarray(spin, dtype=np.int8)
            sf = np.zeros(3, dtype=np.float64)
        else:
            si = np.zeros(1, dtype=np.int8)
            sf = np.ascontiguousarray(spin, dtype=np.float64)
        return lib().vo_ref_total_energy(self.n, self.zmax, _p(self.nbr, C.c_int32), kind, _p(si, C.c_int8),
                                         _p(sf, C.c_double), C.byref(H), bb, bmag)


    def ref_site_energies(self, kind, spin, H: Hamiltonian, b=(0.0, 0.0, 1.0), bmag=0.0):
        """Hamiltonian::energy(i) of every site (src/energy.rs:45-52)."""
        bb = (C.c_double * 3)(*b)
        if kind == 0:
            si = np.ascontiguousarray(spin, dtype=np.int8)
            sf = np.zeros(3, dtype=np.float64)
        else:
            si = np.zeros(1, dtype=np.int8)
            sf = np.ascontiguousarray(spin, dtype=np.float64)
        out = np.zeros(max(self.n, 1))
        lib().vo_ref_site_energies(self.n, self.zmax, _p(self.nbr, C.c_int32), kind, _p(si, C.c_int8),
                                   _p(sf, C.c_double), C.byref(H), bb, bmag, _p(out, C.c_double))
        return out[:self.n]


class MscBatch:
    """Replica groups for the batched multi-spin-coded oracle (one int8 lattice per replica)."""

    def __init__(self, groups):
        # groups: list of (Lattice, temperatures array); word ids are assigned in order
        self.groups = []
        base = 0
        for lat, temps in groups:
            temps = np.ascontiguousarray(temps, dtype=np.float64)
            n_rep = temps.size
            assert n_rep % 32 == 0
            n = int(lib().vo_num_sites(C.byref(lat)))
            spins = np.zeros((n_rep, n), dtype=np.int8)
            tau = np.arange(n_rep, dtype=np.int32)
            self.groups.append(dict(lat=lat, temps=temps, spins=spins, tau=tau, base=base, n=n))
            base += n_rep // 32
        self.total = sum(g["temps"].size for g in self.groups)

    def _structs(self):
        arr = (MscGroup * len(self.groups))()
        for k, g in enumerate(self.groups):
            arr[k] = MscGroup(g["lat"], g["temps"].size, _p(g["temps"], C.c_double), g["base"],
                              _p(g["spins"], C.c_int8), _p(g["tau"], C.c_int32))
        return arr

    def init(self, seed):
        arr = self._structs()
        for k in range(len(self.groups)):
            lib().vo_msc_init(C.byref(arr[k]), seed)

    def run(self, J, seed, sweep0, round0, every, rounds, exchange=True):
        arr = self._structs()
        obs = np.zeros((max(rounds, 1), self.total, 2), dtype=np.int64)
        acc = np.zeros(self.total, dtype=np.int64)
        lib().vo_msc_run(arr, len(self.groups), J, seed, sweep0, round0, every, rounds, int(exchange),
                         _p(obs, C.c_int64), _p(acc, C.c_int64))
        return obs[:rounds], acc


def pcg64(seed: int) -> Pcg64:
    r = Pcg64()
    lib().vo_pcg64_seed(C.byref(r), seed)
    return r


def ising_threshold(J, hz, T, s, nsum) -> int:
    return int(lib().vo_ising_threshold(J, hz, T, s, nsum))


def heis_proposal(w0, w1):
    o = (C.c_double * 3)()
    lib().vo_heis_proposal(w0, w1, o)
    return np.array(list(o))


def heis_delta(params: HeisParams, s, p, h):
    a = (C.c_double * 3)(*s)
    b = (C.c_double * 3)(*p)
    c = (C.c_double * 3)(*h)
    return lib().vo_heis_delta(C.byref(params), a, b, c)


def cooldown_temperatures(tmax, tmin, rate):
    n = lib().vo_cooldown_temperatures(tmax, tmin, rate, None, 0)
    out = np.zeros(n, dtype=np.float64)
    lib().vo_cooldown_temperatures(tmax, tmin, rate, _p(out, C.c_double), n)
    return out


def hysteresis_fields(max_field, step):
    n = lib().vo_hysteresis_fields(max_field, step, None, 0)
    out = np.zeros(n, dtype=np.float64)
    lib().vo_hysteresis_fields(max_field, step, _p(out, C.c_double), n)
    return out


def accumulate(x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = (C.c_double * 3)()
    lib().vo_accumulate(_p(x, C.c_double), x.size, out)
    return tuple(out)


def ref_parallel(lat: Lattice, kind, H: Hamiltonian, T, nsweeps, nthreads, seed=1, proposal=PROPOSE_FLIP,
                 measure=True, bmag=0.0, warmup=0):
    """Independent reference chains, one per thread (field bmag along z):
    `warmup` untimed sweeps, then `nsweeps` timed ones; returns (flips,
    seconds of timed sweeping)."""
    sec = C.c_double()
    flips = int(lib().vo_ref_parallel(C.byref(lat), kind, proposal, C.byref(H), T, bmag, warmup, nsweeps,
                                      int(measure), nthreads, seed, C.byref(sec)))
    return flips, sec.value


def ref_parallel_ladder(lat: Lattice, kind, H: Hamiltonian, temps, sweeps_per_temp, nthreads, seed=1,
                        proposal=PROPOSE_FLIP, measure=True, bmag=0.0, warmup=0):
    """Independent reference chains, one per thread, each walking `temps`
    (`warmup` untimed sweeps at temps[0], then `sweeps_per_temp` timed sweeps
    per temperature, state carried over); returns (flips, seconds)."""
    t = np.ascontiguousarray(temps, dtype=np.float64)
    sec = C.c_double()
    flips = int(lib().vo_ref_parallel_ladder(C.byref(lat), kind, proposal, C.byref(H), _p(t, C.c_double), t.size,
                                             bmag, warmup, sweeps_per_temp, int(measure), nthreads, seed,
                                             C.byref(sec)))
    return flips, sec.value
