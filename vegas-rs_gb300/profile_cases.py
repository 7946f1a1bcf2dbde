"""Small, self-contained workloads of each hot kernel, for profilers.

Each case builds one engine, runs a few sweeps and exits; the commands in
profiles/*.md run these under ncu (one kernel filtered with -k, a few
launches with -c), after the same command has run without the profiler.

    python vegas-rs_gb300/profile_cases.py ising L SWEEPS      # sc L^3 Ising, checkerboard passes
    python vegas-rs_gb300/profile_cases.py ising_sizes N       # pass time for sc 64^3 .. 512^3
    python vegas-rs_gb300/profile_cases.py sub CELL L SWEEPS   # bcc / fcc L^3-cell Ising, sublattice passes
    python vegas-rs_gb300/profile_cases.py heis L SWEEPS       # sc L^3 Heisenberg, FP32
    python vegas-rs_gb300/profile_cases.py heis_sub CELL L SWEEPS  # bcc / fcc L^3-cell Heisenberg, FP32
    python vegas-rs_gb300/profile_cases.py hbatch L REPLICAS   # fcc L^3 cells x replicas, field points
    python vegas-rs_gb300/profile_cases.py msc ROUNDS          # the 256-replica multi-spin-coded batch
"""
import os
import sys
import time

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

import vegas_gb300 as V  # noqa: E402


def ising(L, sweeps):
    with V.Engine(V.Lattice.sc(L, L, L), V.hamiltonian(V.Exchange(1.0)), seed=1) as eng:
        eng.init_random()
        eng.set_thermostat(4.5)
        t0 = time.perf_counter()
        eng.sweeps(sweeps)
        dt = time.perf_counter() - t0
        print(f"ising sc {L}^3: {sweeps} measured sweeps, {L ** 3 * sweeps / (dt * 1e9):.1f} flips/ns (wall)")


def ising_sizes(sweeps_at_256):
    """Pass time against lattice size (unmeasured sweeps): the intercept is
    the fixed cost of a colour-pass launch boundary."""
    for L in (64, 128, 192, 256, 320, 384, 512):
        with V.Engine(V.Lattice.sc(L, L, L), V.hamiltonian(V.Exchange(1.0)), seed=1, path=V.PATH_STRUCTURED) as eng:
            eng.init_random()
            eng.set_thermostat(4.5)
            n = max(20, int(sweeps_at_256 * (256 / L) ** 3)) if L >= 128 else 10 * sweeps_at_256
            eng.sweeps_async(n, measure=False)
            eng.synchronize()
            t0 = time.perf_counter()
            eng.sweeps_async(n, measure=False)
            eng.synchronize()
            us = (time.perf_counter() - t0) / n * 1e6
            print(f"sc {L}^3: pass {us / 2:.2f} us, {L ** 3 / (us * 1e3):.1f} flips/ns, grid {eng.info().grid_blocks}")


def sub(cell, L, sweeps):
    lat = getattr(V.Lattice, cell)(L, L, L)
    with V.Engine(lat, V.hamiltonian(V.Exchange(1.0)), seed=1, path=V.PATH_STRUCTURED) as eng:
        eng.init_random()
        eng.set_thermostat(3.0)
        t0 = time.perf_counter()
        eng.sweeps(sweeps)
        dt = time.perf_counter() - t0
        print(f"ising {cell} {L}^3 cells: {sweeps} measured sweeps, {lat.n_sites * sweeps / (dt * 1e9):.1f} flips/ns (wall)")


def heis(L, sweeps):
    H = V.hamiltonian(V.Exchange(1.0), V.UniaxialAnisotropy((0, 0, 1), 0.1), V.Zeeman())
    with V.Engine(V.Lattice.sc(L, L, L), H, spin=V.SPIN_HEISENBERG, seed=1) as eng:
        eng.init_random()
        eng.set_thermostat(1.0, (0, 0, 1), 0.05)
        t0 = time.perf_counter()
        eng.sweeps(sweeps)
        dt = time.perf_counter() - t0
        print(f"heisenberg sc {L}^3: {sweeps} measured sweeps, {L ** 3 * sweeps / (dt * 1e9):.1f} flips/ns (wall)")


def heis_sub(cell, L, sweeps):
    lat = getattr(V.Lattice, cell)(L, L, L)
    H = V.hamiltonian(V.Exchange(1.0), V.UniaxialAnisotropy((0, 0, 1), 0.1), V.Zeeman())
    with V.Engine(lat, H, spin=V.SPIN_HEISENBERG, seed=1, path=V.PATH_STRUCTURED) as eng:
        eng.init_random()
        eng.set_thermostat(1.0, (0, 0, 1), 0.05)
        t0 = time.perf_counter()
        eng.sweeps(sweeps)
        dt = time.perf_counter() - t0
        print(f"heisenberg {cell} {L}^3 cells: {sweeps} measured sweeps, "
              f"{lat.n_sites * sweeps / (dt * 1e9):.1f} flips/ns (wall)")


def hbatch(L, nrep):
    lat = V.Lattice.fcc(L, L, L)
    reps = [V.HeisReplica(seed=11 + r, replica=r, temperature=0.5, cubic=0.05) for r in range(nrep)]
    with V.HysteresisBatch(lat, reps, zeeman_sign=-1.0) as hb:
        hb.init_random()
        t0 = time.perf_counter()
        hb.run([1.0, 0.5], 2, 3)
        dt = time.perf_counter() - t0
        print(f"hysteresis batch fcc {L}^3 x {nrep}: 2 points x 5 sweeps, "
              f"{lat.n_sites * nrep * 10 / (dt * 1e9):.1f} flips/ns (wall, incl. graph capture)")


def msc(rounds):
    import numpy as np

    t2 = np.geomspace(2.0, 2.6, 64)
    t3 = np.geomspace(4.2, 4.8, 64)
    groups = [(V.Lattice.sc(64, 64, 1, pbc=(True, True, False)), t2),
              (V.Lattice.sc(512, 512, 1, pbc=(True, True, False)), t2),
              (V.Lattice.sc(32, 32, 32), t3), (V.Lattice.sc(128, 128, 128), t3)]
    with V.Batch(groups, J=1.0, seed=1, sweeps_per_round=10, exchange=True) as b:
        b.init_random()
        t0 = time.perf_counter()
        b.run(rounds)
        dt = time.perf_counter() - t0
        print(f"msc batch: {rounds} rounds, {b.info().replica_sites * 10 * rounds / (dt * 1e9):.1f} flips/ns (wall)")


if __name__ == "__main__":
    case, args = sys.argv[1], [a if a in ("bcc", "fcc") else int(a) for a in sys.argv[2:]]
    {"ising": ising, "ising_sizes": ising_sizes, "sub": sub, "heis": heis, "heis_sub": heis_sub, "hbatch": hbatch, "msc": msc}[case](*args)
