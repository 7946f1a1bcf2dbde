"""Python binding of the vegas GB300 Metropolis engine (libvegas_gpu.so).

Mirrors the pieces of the vegas API the engine replaces, with the same names
and meaning:

* ``Lattice.sc/bcc/fcc`` + ``expand`` + per-axis PBC (src/input.rs:296-322);
* the energy terms ``Exchange``, ``UniaxialAnisotropy``, ``Zeeman``,
  ``Gauge`` and the ``hamiltonian(...)`` builder, which nests terms into a
  Compound exactly like the ``hamiltonian!`` macro (src/energy.rs:273-290);
* ``Engine``: the device-resident state + Metropolis integrator
  (MetropolisFlipIntegrator / MetropolisIntegrator, src/integrator.rs:56-138),
  with ``set_thermostat`` (src/thermostat.rs) and per-sweep E / |M|.

All compute runs in the CUDA library; this module only marshals arguments.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field
from typing import Optional, Sequence, Tuple

import numpy as np

from . import _abi
from ._abi import (CELL_BCC, CELL_FCC, CELL_SC, FP32, FP64, PATH_AUTO, PATH_GENERIC, PATH_RESIDENT, PATH_STRUCTURED, PATH_TILED,
                   PROPOSE_FLIP, PROPOSE_RANDOM, SPIN_HEISENBERG, SPIN_ISING, Sums, VegasGpuError)

__all__ = [
    "Lattice", "Exchange", "UniaxialAnisotropy", "Zeeman", "Gauge", "CubicAnisotropy", "hamiltonian",
    "Engine", "Sums", "VegasGpuError", "lib", "SPIN_ISING", "SPIN_HEISENBERG", "PROPOSE_FLIP",
    "PROPOSE_RANDOM", "PATH_AUTO", "PATH_GENERIC", "PATH_STRUCTURED", "PATH_RESIDENT", "PATH_TILED", "FP32", "FP64", "Batch",
    "HeisReplica", "HysteresisBatch", "hysteresis_fields", "loop_area", "coercive_fields",
]

_lib = None


def lib() -> C.CDLL:
    """The loaded CUDA library (raises if it is not built)."""
    global _lib
    if _lib is None:
        _lib = _abi.load()
    return _lib


def _check(rc: int, ctx=None):
    if rc != _abi.VG_OK:
        msg = lib().vg_last_error(ctx)
        raise VegasGpuError(rc, (msg or b"").decode() or lib().vg_status_string(rc).decode())


# ------------------------------------------------------------------ lattice
@dataclass(frozen=True)
class Lattice:
    """``Lattice::<cell>(1.0).expand(nx, ny, nz)`` with drop_x/y/z on open axes."""

    cell: int
    nx: int
    ny: int
    nz: int
    pbc: Tuple[bool, bool, bool] = (True, True, True)

    @staticmethod
    def sc(nx, ny=None, nz=None, pbc=(True, True, True)):
        return Lattice(CELL_SC, nx, ny if ny is not None else nx, nz if nz is not None else nx, tuple(pbc))

    @staticmethod
    def bcc(nx, ny=None, nz=None, pbc=(True, True, True)):
        return Lattice(CELL_BCC, nx, ny if ny is not None else nx, nz if nz is not None else nx, tuple(pbc))

    @staticmethod
    def fcc(nx, ny=None, nz=None, pbc=(True, True, True)):
        return Lattice(CELL_FCC, nx, ny if ny is not None else nx, nz if nz is not None else nx, tuple(pbc))

    def desc(self) -> _abi.LatticeDesc:
        return _abi.LatticeDesc(self.cell, self.nx, self.ny, self.nz, int(self.pbc[0]), int(self.pbc[1]),
                                int(self.pbc[2]))

    @property
    def basis(self) -> int:
        return {CELL_SC: 1, CELL_BCC: 2, CELL_FCC: 4}[self.cell]

    @property
    def n_sites(self) -> int:
        return self.nx * self.ny * self.nz * self.basis

    def neighbours(self) -> np.ndarray:
        d = self.desc()
        n, z = C.c_int64(), C.c_int32()
        _check(lib().vg_lattice_neighbours(C.byref(d), None, 0, C.byref(n), C.byref(z)))
        out = np.empty(n.value * z.value, dtype=np.int32)
        _check(lib().vg_lattice_neighbours(C.byref(d), out.ctypes.data_as(C.POINTER(C.c_int32)), out.size,
                                           C.byref(n), C.byref(z)))
        return out.reshape(n.value, z.value)

    def colouring(self) -> Tuple[np.ndarray, int]:
        d = self.desc()
        out = np.empty(self.n_sites, dtype=np.int32)
        nc = C.c_int32()
        _check(lib().vg_lattice_colouring(C.byref(d), out.ctypes.data_as(C.POINTER(C.c_int32)), out.size,
                                          C.byref(nc)))
        return out, nc.value


# ------------------------------------------------------------------ energies
@dataclass
class Exchange:
    """Exchange::from_lattice(J, lattice): per site -J sum_j s_i.s_j."""
    J: float = 1.0


@dataclass
class UniaxialAnisotropy:
    """UniaxialAnisotropy::new(axis, K): per site +K (s.axis)^2."""
    axis: Sequence[float] = (0.0, 0.0, 1.0)
    K: float = 1.0


@dataclass
class Zeeman:
    """Zeeman::new(): per site +|B| (s.b) with the thermostat's field."""
    sign: float = 1.0


@dataclass
class Gauge:
    """Gauge::new(g): per site g."""
    value: float = 0.0


@dataclass
class CubicAnisotropy:
    """Extension without a reference counterpart: per site -Kc (sx^4+sy^4+sz^4)."""
    Kc: float = 0.0


def hamiltonian(*terms) -> _abi.HamiltonianDesc:
    """Flatten terms as the ``hamiltonian!`` macro nests them.

    One term keeps that term's own ``total_energy``; two or more form a
    Compound whose total is sum_i energy(i).  Repeated terms of one kind add
    their per-site coefficients.
    """
    if not terms:
        raise ValueError("hamiltonian needs at least one term")
    h = _abi.HamiltonianDesc()
    h.zeeman_sign = 0.0
    for t in terms:
        if isinstance(t, Exchange):
            h.has_exchange = 1
            h.exchange += t.J
        elif isinstance(t, UniaxialAnisotropy):
            if h.has_anisotropy and tuple(h.anisotropy_axis) != tuple(t.axis):
                raise ValueError("two anisotropy terms with different axes are not supported")
            h.has_anisotropy = 1
            h.anisotropy += t.K
            for i in range(3):
                h.anisotropy_axis[i] = t.axis[i]
        elif isinstance(t, Zeeman):
            h.has_zeeman = 1
            h.zeeman_sign += t.sign
        elif isinstance(t, Gauge):
            h.has_gauge = 1
            h.gauge += t.value
        elif isinstance(t, CubicAnisotropy):
            h.has_cubic = 1
            h.cubic += t.Kc
        else:
            raise TypeError(f"unknown energy term {t!r}")
    h.compound = 1 if len(terms) >= 2 else 0
    return h


# ------------------------------------------------------------------ engine
class Engine:
    """A device-resident lattice state driven by the GPU Metropolis integrator.

    `path` picks the kernel family (PATH_AUTO chooses): PATH_STRUCTURED runs
    implicit neighbour stencils -- sc checkerboard classes, and one array per
    basis sublattice for bcc / fcc (Ising when x is a multiple of 16,
    Heisenberg always); PATH_GENERIC runs neighbour tables on any lattice and
    is the one per-bond exchange constants need; PATH_RESIDENT keeps a small
    sc Ising lattice in one block's shared memory; PATH_TILED runs each sweep
    of a fully periodic sc Ising lattice as one launch over shared-memory
    tiles with halos.  All paths draw the same random numbers for the same
    site, sweep and seed.
    """

    def __init__(self, lattice: Lattice, ham: _abi.HamiltonianDesc, spin: int = SPIN_ISING, seed: int = 0,
                 proposal: Optional[int] = None, path: int = PATH_AUTO, precision: int = FP32, replica: int = 0,
                 threads_per_block: int = 0, blocks_per_sm: int = 0, device: int = -1, max_device_bytes: int = 0):
        L = lib()
        o = _abi.Options()
        _check(L.vg_options_default(spin, C.byref(o)))
        if proposal is not None:
            o.proposal = proposal
        o.path, o.precision, o.replica = path, precision, replica
        o.threads_per_block, o.blocks_per_sm, o.device = threads_per_block, blocks_per_sm, device
        o.max_device_bytes = max_device_bytes
        self.lattice, self.ham, self.spin_kind = lattice, ham, spin
        d = lattice.desc()
        h = C.c_void_p()
        _check(L.vg_ctx_create_ex(C.byref(d), C.byref(ham), C.byref(o), C.c_uint64(seed), C.byref(h)))
        self._h = h
        self.n = lattice.n_sites

    # lifecycle
    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            lib().vg_ctx_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def info(self) -> _abi.Info:
        i = _abi.Info()
        _check(lib().vg_ctx_info(self._h, C.byref(i)), self._h)
        return i

    # state
    def init_random(self):
        _check(lib().vg_init_random(self._h), self._h)

    def set_state(self, spins: np.ndarray):
        if self.spin_kind == SPIN_ISING:
            a = np.ascontiguousarray(spins, dtype=np.int8)
        else:
            a = np.ascontiguousarray(spins, dtype=np.float64)
        _check(lib().vg_set_state(self._h, a.ctypes.data, C.c_int64(self.n)), self._h)

    def get_state(self) -> np.ndarray:
        if self.spin_kind == SPIN_ISING:
            out = np.empty(self.n, dtype=np.int8)
        else:
            out = np.empty((self.n, 3), dtype=np.float64)
        _check(lib().vg_get_state(self._h, out.ctypes.data, C.c_int64(self.n)), self._h)
        return out

    def set_thermostat(self, temperature: float, b=(0.0, 0.0, 1.0), magnitude: float = 0.0):
        bb = (C.c_double * 3)(*b)
        _check(lib().vg_set_thermostat(self._h, temperature, bb, magnitude), self._h)

    @property
    def sweep_index(self) -> int:
        v = C.c_uint64()
        _check(lib().vg_get_sweep_index(self._h, C.byref(v)), self._h)
        return v.value

    @sweep_index.setter
    def sweep_index(self, v: int):
        _check(lib().vg_set_sweep_index(self._h, C.c_uint64(v)), self._h)

    # sweeps
    def sweeps(self, n: int, measure: bool = True):
        """Run n sweeps; returns (E, |M|) arrays per sweep when measuring."""
        if not measure:
            _check(lib().vg_sweeps(self._h, C.c_uint64(n), 0, None, None), self._h)
            return None
        E = np.empty(max(n, 1), dtype=np.float64)
        M = np.empty(max(n, 1), dtype=np.float64)
        dp = C.POINTER(C.c_double)
        _check(lib().vg_sweeps(self._h, C.c_uint64(n), 1, E.ctypes.data_as(dp), M.ctypes.data_as(dp)), self._h)
        return E[:n], M[:n]

    def sweeps_sums(self, n: int) -> np.ndarray:
        out = (Sums * max(n, 1))()
        _check(lib().vg_sweeps_sums(self._h, C.c_uint64(n), out), self._h)
        return np.frombuffer(out, dtype=np.float64).reshape(-1, 8)[:n].copy()

    def sweeps_async(self, n: int, measure: bool = True):
        _check(lib().vg_sweeps_async(self._h, C.c_uint64(n), int(measure)), self._h)

    def read_sums(self, n: int) -> np.ndarray:
        out = (Sums * max(n, 1))()
        _check(lib().vg_read_sums(self._h, C.c_uint64(n), out), self._h)
        return np.frombuffer(out, dtype=np.float64).reshape(-1, 8)[:n].copy()

    def synchronize(self):
        _check(lib().vg_synchronize(self._h), self._h)

    def stream(self) -> int:
        s = C.c_void_p()
        _check(lib().vg_get_stream(self._h, C.byref(s)), self._h)
        return s.value or 0

    def set_stream(self, stream_ptr: int):
        _check(lib().vg_set_stream(self._h, C.c_void_p(stream_ptr)), self._h)

    def time_passes(self, n: int, measure: bool = True) -> Tuple[float, float]:
        """Mean colour-pass and sweep durations (ms) over n real sweeps (CUDA events)."""
        a, b = C.c_double(), C.c_double()
        _check(lib().vg_time_passes(self._h, C.c_uint64(n), int(measure), C.byref(a), C.byref(b)), self._h)
        return a.value, b.value

    def wolff_steps(self, n: int, measure: bool = True):
        """n Wolff cluster steps (WolffIntegrator); returns (E, |M|) per step."""
        E = np.zeros(max(n, 1))
        M = np.zeros(max(n, 1))
        _check(lib().vg_wolff_steps(self._h, C.c_uint64(n), int(measure), E.ctypes.data_as(C.POINTER(C.c_double)),
                                    M.ctypes.data_as(C.POINTER(C.c_double))), self._h)
        return E[:n], M[:n]

    def set_exchange_bonds(self, J: Optional[np.ndarray]):
        """Per-bond exchange constants (n_sites x coordination, the order of
        Lattice.neighbours()); None restores the uniform constant."""
        if J is None:
            _check(lib().vg_set_exchange_bonds(self._h, None, 0), self._h)
            return
        a = np.ascontiguousarray(J, dtype=np.float64)
        _check(lib().vg_set_exchange_bonds(self._h, a.ctypes.data_as(C.POINTER(C.c_double)), a.size), self._h)

    # observables
    def current_sums(self) -> np.ndarray:
        s = Sums()
        _check(lib().vg_current_sums(self._h, C.byref(s)), self._h)
        return np.frombuffer(s, dtype=np.float64).copy()

    def total_energy(self) -> float:
        e = C.c_double()
        _check(lib().vg_total_energy(self._h, C.byref(e)), self._h)
        return e.value

    def site_energies(self) -> np.ndarray:
        """Hamiltonian::energy(i) for every site of the current state (FP64)."""
        n = self.lattice.n_sites
        out = np.zeros(max(n, 1))
        _check(lib().vg_site_energies(self._h, out.ctypes.data_as(C.POINTER(C.c_double)), n), self._h)
        return out[:n]

    def delta_energies(self, proposals: np.ndarray) -> np.ndarray:
        """Energy change of replacing each site's spin by proposals[i] (n x 3),
        the others fixed, in the context's precision (Heisenberg)."""
        n = self.lattice.n_sites
        p = np.ascontiguousarray(proposals, dtype=np.float64).reshape(n, 3)
        out = np.zeros(max(n, 1))
        _check(lib().vg_delta_energies(self._h, p.ctypes.data_as(C.POINTER(C.c_double)),
                                       out.ctypes.data_as(C.POINTER(C.c_double)), n), self._h)
        return out[:n]

    def magnetization(self):
        m = (C.c_double * 3)()
        mag = C.c_double()
        _check(lib().vg_magnetization(self._h, m, C.byref(mag)), self._h)
        return np.array(list(m)), mag.value

    def energy_from_sums(self, sums_row) -> Tuple[float, float]:
        s = Sums(*[float(v) for v in sums_row])
        e, m = C.c_double(), C.c_double()
        _check(lib().vg_energy_from_sums(self._h, C.byref(s), C.byref(e), C.byref(m)), self._h)
        return e.value, m.value


class Batch:
    """Replica groups of multi-spin-coded Ising lattices with on-device replica exchange.

    groups: list of (Lattice, temperatures); each group's replica count is
    len(temperatures) (a multiple of 32).  One round = sweeps_per_round
    sweeps, then per-replica measurement and (if exchange) ladder swaps.
    """

    def __init__(self, groups, J: float = 1.0, seed: int = 0, sweeps_per_round: int = 10, exchange: bool = True):
        L = lib()
        self._temps = [np.ascontiguousarray(t, dtype=np.float64) for _, t in groups]
        arr = (_abi.ReplicaGroup * len(groups))()
        for k, (lat, _) in enumerate(groups):
            arr[k] = _abi.ReplicaGroup(lat.desc(), self._temps[k].size,
                                       self._temps[k].ctypes.data_as(C.POINTER(C.c_double)))
        h = C.c_void_p()
        rc = L.vg_batch_create(arr, len(groups), J, C.c_uint64(seed), sweeps_per_round, int(exchange), C.byref(h))
        if rc:
            raise VegasGpuError(rc, L.vg_last_error(None).decode())
        self._h = h
        self.lattices = [lat for lat, _ in groups]
        self.J = J

    def _chk(self, rc):
        if rc:
            raise VegasGpuError(rc, lib().vg_batch_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            lib().vg_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def info(self) -> _abi.BatchInfo:
        i = _abi.BatchInfo()
        self._chk(lib().vg_batch_get_info(self._h, C.byref(i)))
        return i

    def stream(self) -> int:
        s = C.c_void_p()
        self._chk(lib().vg_batch_get_stream(self._h, C.byref(s)))
        return s.value or 0

    def init_random(self):
        self._chk(lib().vg_batch_init_random(self._h))

    def run(self, rounds: int):
        self._chk(lib().vg_batch_run(self._h, C.c_uint64(rounds)))

    def run_async(self, rounds: int):
        self._chk(lib().vg_batch_run_async(self._h, C.c_uint64(rounds)))

    def synchronize(self):
        self._chk(lib().vg_batch_synchronize(self._h))

    def observables(self, round_index: int):
        n = self.info().total_replicas
        counts = np.zeros((n, 2), dtype=np.int64)
        tau = np.zeros(n, dtype=np.int32)
        self._chk(lib().vg_batch_observables(self._h, C.c_uint64(round_index),
                                             counts.ctypes.data_as(C.POINTER(C.c_int64)),
                                             tau.ctypes.data_as(C.POINTER(C.c_int32))))
        return counts, tau

    def ladder(self, group: int) -> np.ndarray:
        out = np.zeros(self._temps[group].size, dtype=np.int32)
        self._chk(lib().vg_batch_ladder(self._h, group, out.ctypes.data_as(C.POINTER(C.c_int32))))
        return out

    def swap_stats(self, group: int):
        n = self._temps[group].size
        acc = np.zeros(n, dtype=np.int64)
        att = np.zeros(n, dtype=np.int64)
        self._chk(lib().vg_batch_swap_stats(self._h, group, acc.ctypes.data_as(C.POINTER(C.c_int64)),
                                            att.ctypes.data_as(C.POINTER(C.c_int64))))
        return acc, att

    # launch shape of the multi-spin-coded passes (results do not depend on it)
    def tuning(self) -> Tuple[int, int, int]:
        t = _abi.BatchTuning()
        self._chk(lib().vg_batch_get_tuning(self._h, C.byref(t)))
        return (t.threads_per_block, t.words_per_thread, t.words_in_flight)

    def set_tuning(self, threads_per_block: int, words_per_thread: int, words_in_flight: int):
        t = _abi.BatchTuning(threads_per_block, words_per_thread, words_in_flight)
        self._chk(lib().vg_batch_set_tuning(self._h, C.byref(t)))

    def signature(self) -> str:
        """Shape of the batch as a tuning-cache key: per group the lattice
        extents, periodicity and replica count."""
        parts = []
        for lat, temps in zip(self.lattices, self._temps):
            d = lat.desc()
            parts.append(f"sc{d.nx}x{d.ny}x{d.nz}p{d.pbc_x}{d.pbc_y}{d.pbc_z}r{temps.size}")
        return "+".join(parts)

    def autotune(self, rounds: int = 3, cache: Optional[str] = None):
        """Pick the fastest launch shape for this batch on this device.

        With `cache` (a JSON file), a shape stored for the same device name and
        batch signature is applied without timing; otherwise every shape is
        timed (vg_batch_autotune, which restores the batch's state afterwards)
        and the winner is stored.  Returns (shape, ms per round or None)."""
        import json

        key = f"{device_name()}|{self.signature()}"
        table = {}
        if cache and os.path.exists(cache):
            try:
                with open(cache) as f:
                    table = json.load(f)
            except (OSError, ValueError):
                table = {}
        if key in table:
            self.set_tuning(*table[key]["shape"])
            return tuple(table[key]["shape"]), None
        best = _abi.BatchTuning()
        ms = C.c_double()
        self._chk(lib().vg_batch_autotune(self._h, rounds, C.byref(best), C.byref(ms)))
        shape = (best.threads_per_block, best.words_per_thread, best.words_in_flight)
        if cache:
            table[key] = {"shape": list(shape), "ms_per_round": ms.value}
            d = os.path.dirname(os.path.abspath(cache))
            os.makedirs(d, exist_ok=True)
            tmp = cache + ".tmp"
            with open(tmp, "w") as f:
                json.dump(table, f, indent=1, sort_keys=True)
            os.replace(tmp, cache)
        return shape, ms.value

    def get_replica(self, group: int, replica: int) -> np.ndarray:
        out = np.empty(self.lattices[group].n_sites, dtype=np.int8)
        self._chk(lib().vg_batch_get_replica(self._h, group, replica, out.ctypes.data_as(C.POINTER(C.c_int8))))
        return out

    def set_replica(self, group: int, replica: int, spins: np.ndarray):
        a = np.ascontiguousarray(spins, dtype=np.int8)
        self._chk(lib().vg_batch_set_replica(self._h, group, replica, a.ctypes.data_as(C.POINTER(C.c_int8))))


class HeisReplica:
    """One replica of a HysteresisBatch: seed and Philox stream id, temperature
    and energy constants (exchange J, uniaxial K, cubic Kc)."""

    def __init__(self, seed: int, replica: int = 0, temperature: float = 1.0, exchange: float = 1.0,
                 anisotropy: float = 0.0, cubic: float = 0.0):
        self.seed, self.replica, self.temperature = seed, replica, temperature
        self.exchange, self.anisotropy, self.cubic = exchange, anisotropy, cubic

    def _c(self) -> _abi.HeisReplica:
        return _abi.HeisReplica(C.c_uint64(self.seed).value, self.replica, 0, self.temperature, self.exchange,
                                self.anisotropy, self.cubic)


class HysteresisBatch:
    """Heisenberg replicas of one bcc or fcc lattice swept through a shared
    field schedule (the vg_hbatch_* ABI).

    Per-site energy -J sum s.s_j + K (s.e)^2 + zeeman_sign h (s.b) - Kc sum s_a^4;
    zeeman_sign = +1 is the reference's per-site sign, -1 aligns the spins with
    the field.  run(fields, relax, measure) returns the per-point sums
    (points x replicas x 12, see VG_HB_NSUMS in vegas_gpu.h).
    """

    def __init__(self, lattice: "Lattice", replicas: Sequence[HeisReplica], anisotropy_axis=(0.0, 0.0, 1.0),
                 field_axis=(0.0, 0.0, 1.0), zeeman_sign: float = 1.0, precision: int = FP32,
                 proposal: int = PROPOSE_RANDOM):
        L = lib()
        d = _abi.HBatchDesc()
        d.lattice = lattice.desc()
        d.anisotropy_axis[:] = tuple(float(v) for v in anisotropy_axis)
        d.field_axis[:] = tuple(float(v) for v in field_axis)
        d.zeeman_sign = zeeman_sign
        d.precision = precision
        d.proposal = proposal
        arr = (_abi.HeisReplica * len(replicas))(*[r._c() for r in replicas])
        h = C.c_void_p()
        rc = L.vg_hbatch_create(C.byref(d), arr, len(replicas), C.byref(h))
        if rc:
            raise VegasGpuError(rc, L.vg_last_error(None).decode())
        self._h = h
        self.lattice = lattice
        self.replicas = list(replicas)
        self.zeeman_sign = zeeman_sign

    def _chk(self, rc):
        if rc:
            raise VegasGpuError(rc, lib().vg_hbatch_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            lib().vg_hbatch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def info(self) -> _abi.HBatchInfo:
        i = _abi.HBatchInfo()
        self._chk(lib().vg_hbatch_get_info(self._h, C.byref(i)))
        return i

    def stream(self) -> int:
        s = C.c_void_p()
        self._chk(lib().vg_hbatch_get_stream(self._h, C.byref(s)))
        return s.value or 0

    def init_random(self):
        self._chk(lib().vg_hbatch_init_random(self._h))

    def get_replica(self, r: int) -> np.ndarray:
        n = self.lattice.n_sites
        out = np.empty((n, 3), dtype=np.float64)
        self._chk(lib().vg_hbatch_get_replica(self._h, r, out.ctypes.data_as(C.POINTER(C.c_double)), n))
        return out

    def set_replica(self, r: int, xyz: np.ndarray):
        a = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        self._chk(lib().vg_hbatch_set_replica(self._h, r, a.ctypes.data_as(C.POINTER(C.c_double)), a.shape[0]))

    def run_async(self, fields, relax: int, measure: int):
        f = np.ascontiguousarray(fields, dtype=np.float64)
        self._fields = f
        self._chk(lib().vg_hbatch_run_async(self._h, f.ctypes.data_as(C.POINTER(C.c_double)), f.size, relax,
                                            measure))

    def synchronize(self):
        self._chk(lib().vg_hbatch_synchronize(self._h))

    def point_sums(self) -> np.ndarray:
        n = self._fields.size * len(self.replicas) * _abi.HB_NSUMS
        out = np.empty(n, dtype=np.float64)
        self._chk(lib().vg_hbatch_point_sums(self._h, out.ctypes.data_as(C.POINTER(C.c_double)), n))
        return out.reshape(self._fields.size, len(self.replicas), _abi.HB_NSUMS)

    def run(self, fields, relax: int, measure: int) -> np.ndarray:
        self.run_async(fields, relax, measure)
        self.synchronize()
        return self.point_sums()

    def time_passes(self, n_sweeps: int) -> float:
        ms = C.c_double()
        self._chk(lib().vg_hbatch_time_passes(self._h, n_sweeps, C.byref(ms)))
        return ms.value


def hysteresis_fields(max_field: float, step: float) -> np.ndarray:
    """Signed field values of a closed loop +max -> -max -> +max in steps of
    `step` (2 n + 1 points for n = max / step; each value is computed as
    max - k step, so the schedule does not drift).  The reference's own
    HysteresisLoop (src/program.rs:281-335, magnitude 0 -> max -> -max -> max
    with accumulated steps) is mirrored by the C++ host's HysteresisLoop."""
    n = int(round(max_field / step))
    down = max_field - step * np.arange(0, 2 * n + 1)
    up = -max_field + step * np.arange(1, 2 * n + 1)
    return np.concatenate([down, up])


def loop_area(fields: np.ndarray, m: np.ndarray) -> float:
    """Area enclosed by the closed loop (h, m): |trapezoid integral of m dh|."""
    h = np.append(fields, fields[0])
    mm = np.append(m, m[0])
    return float(abs(np.sum(0.5 * (mm[1:] + mm[:-1]) * np.diff(h))))


def coercive_fields(fields: np.ndarray, m: np.ndarray):
    """Fields where m changes sign on the descending and the ascending branch
    (linear interpolation between the bracketing points; NaN if none)."""
    res = []
    for sgn in (-1.0, 1.0):
        hc = float("nan")
        for i in range(len(fields) - 1):
            if np.sign(fields[i + 1] - fields[i]) != sgn:
                continue
            a, b = m[i], m[i + 1]
            if a == 0.0 or a * b < 0.0:
                hc = float(fields[i] if a == 0.0 else fields[i] + (fields[i + 1] - fields[i]) * a / (a - b))
                break
        res.append(hc)
    return tuple(res)


def device_name(device: int = 0) -> str:
    buf = C.create_string_buffer(256)
    _check(lib().vg_device_name(device, buf, 256))
    return buf.value.decode()


def device_count() -> int:
    n = C.c_int32()
    lib().vg_device_count(C.byref(n))
    return n.value
