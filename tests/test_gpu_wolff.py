"""Wolff cluster steps (WolffIntegrator, src/integrator.rs:140-230) on the
GPU, against the oracle's cluster steps with the same draws, and against
Metropolis sweeps in equilibrium."""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = [
    ("sc", (10, 10, 10), (1, 1, 1)),   # docs/wolff.toml's lattice
    ("sc", (32, 32, 1), (1, 1, 0)),    # 2D, open z
    ("sc", (4, 2, 4), (1, 1, 1)),      # a periodic axis of extent 2: repeated bonds
    ("bcc", (4, 4, 4), (1, 1, 1)),
    ("fcc", (3, 3, 3), (1, 0, 1)),
]


@pytest.mark.parametrize("cell,ext,pbc", CASES)
@pytest.mark.parametrize("T", [6.0, 4.0, 2.0])
def test_wolff_steps_bit_exact(V, O, cell, ext, pbc, T):
    seed, J, n = 5, 1.0, 300
    lat = getattr(V.Lattice, cell)(*ext, pbc=tuple(bool(p) for p in pbc))
    g = O.Graph(O.lattice(cell, *ext, pbc))
    with V.Engine(lat, V.hamiltonian(V.Exchange(J)), seed=seed) as eng:
        eng.init_random()
        s0 = eng.get_state()
        eng.set_thermostat(T)
        E, M = eng.wolff_steps(n)
        ref, obs = g.wolff_steps(s0, J, T, seed, 0, n)
        assert np.array_equal(eng.get_state(), ref)
        np.testing.assert_array_equal(E, -J * obs[:, 0])     # Exchange::total_energy
        np.testing.assert_array_equal(M, np.abs(obs[:, 1]))
        assert eng.info().sweep_index == n


# beyond 16,384 sites: spins and cluster marks as bits in one block
MID_CASES = [
    ("sc", (32, 32, 32), (1, 1, 1)),
    ("sc", (256, 256, 1), (1, 1, 0)),
    ("sc", (64, 2, 256), (1, 1, 1)),   # repeated bonds along y
    ("bcc", (24, 24, 24), (1, 1, 1)),
    ("fcc", (18, 18, 18), (1, 0, 1)),
]


# beyond 786,432 sites: the multi-block kernel (grid barrier per level)
GRID_CASES = [
    ("sc", (96, 96, 96), (1, 1, 1)),
    ("fcc", (60, 60, 60), (1, 1, 0)),
]


def _wolff_bit_exact(V, O, cell, ext, pbc, T, n):
    seed, J = 9, 1.0
    lat = getattr(V.Lattice, cell)(*ext, pbc=tuple(bool(p) for p in pbc))
    g = O.Graph(O.lattice(cell, *ext, pbc))
    with V.Engine(lat, V.hamiltonian(V.Exchange(J)), seed=seed) as eng:
        eng.init_random()
        s0 = eng.get_state()
        eng.set_thermostat(T)
        E, M = eng.wolff_steps(n)
        ref, obs = g.wolff_steps(s0, J, T, seed, 0, n)
        assert np.array_equal(eng.get_state(), ref)
        np.testing.assert_array_equal(E, -J * obs[:, 0])
        np.testing.assert_array_equal(M, np.abs(obs[:, 1]))
        # unmeasured steps continue the same stream
        eng.wolff_steps(5, measure=False)
        ref2, _ = g.wolff_steps(ref, J, T, seed, n, 5)
        assert np.array_equal(eng.get_state(), ref2)
    return lat.n_sites


@pytest.mark.parametrize("cell,ext,pbc", MID_CASES)
@pytest.mark.parametrize("T", [8.0, 4.5, 2.0])
def test_wolff_mid_steps_bit_exact(V, O, cell, ext, pbc, T):
    assert 16384 < _wolff_bit_exact(V, O, cell, ext, pbc, T, 60) <= 786432


@pytest.mark.parametrize("cell,ext,pbc", GRID_CASES)
@pytest.mark.parametrize("T", [4.5, 2.0])
def test_wolff_grid_steps_bit_exact(V, O, cell, ext, pbc, T):
    assert _wolff_bit_exact(V, O, cell, ext, pbc, T, 12) > 786432


def test_wolff_then_metropolis_continue_one_stream(V, O):
    """Wolff steps and Metropolis sweeps share the context's counter."""
    lat = V.Lattice.sc(10, 10, 10)
    g = O.Graph(O.lattice("sc", 10, 10, 10))
    with V.Engine(lat, V.hamiltonian(V.Exchange(1.0)), seed=2, path=V.PATH_GENERIC) as eng:
        eng.init_random()
        s0 = eng.get_state()
        eng.set_thermostat(4.4)
        eng.wolff_steps(7)
        eng.sweeps(3)
        s1, _ = g.wolff_steps(s0, 1.0, 4.4, 2, 0, 7)
        s2, _ = g.ising_sweeps(s1, 1.0, 0.0, 4.4, 2, 7, 3)
        assert np.array_equal(eng.get_state(), s2)


def test_wolff_equilibrium_matches_metropolis(V):
    """<E> and <|M|> of the 3D Ising model from cluster steps and from
    Metropolis sweeps agree within their statistical errors."""
    lat = V.Lattice.sc(10, 10, 10)
    H = V.hamiltonian(V.Exchange(1.0))
    out = {}
    for how in ("wolff", "metropolis"):
        with V.Engine(lat, H, seed=11) as eng:
            eng.init_random()
            eng.set_thermostat(4.0)
            run = eng.wolff_steps if how == "wolff" else eng.sweeps
            run(2000)
            E, M = run(40000 if how == "wolff" else 20000)
            n = 1000
            e, m = E / n, M / n
            blocks = 40
            be = e[: len(e) // blocks * blocks].reshape(blocks, -1).mean(axis=1)
            bm = m[: len(m) // blocks * blocks].reshape(blocks, -1).mean(axis=1)
            out[how] = (be.mean(), be.std() / np.sqrt(blocks), bm.mean(), bm.std() / np.sqrt(blocks))
    (ew, sew, mw, smw), (em, sem, mm, smm) = out["wolff"], out["metropolis"]
    assert abs(ew - em) < 4 * np.hypot(sew, sem) + 1e-3
    assert abs(mw - mm) < 4 * np.hypot(smw, smm) + 2e-3


def test_wolff_rejections(V):
    with V.Engine(V.Lattice.sc(8, 8, 8), V.hamiltonian(V.Exchange(1.0)), spin=V.SPIN_HEISENBERG, seed=1) as eng:
        with pytest.raises(V.VegasGpuError) as e:
            eng.wolff_steps(1)
        assert e.value.status == 5
    lat = V.Lattice.bcc(4, 4, 4)
    with V.Engine(lat, V.hamiltonian(V.Exchange(1.0)), seed=1, path=V.PATH_GENERIC) as eng:
        eng.set_exchange_bonds(np.ones((lat.n_sites, 8)))
        with pytest.raises(V.VegasGpuError) as e:
            eng.wolff_steps(1)
        assert e.value.status == 5 and "uniform exchange" in str(e.value)


def test_cli_runs_the_wolff_input(tmp_path):
    """docs/wolff.toml's shape (sc 10^3, Relax, CoolDown) with short stages."""
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    cli = os.path.join(repo, "vegas-rs_gb300", "_build", "bin", "vegas_gpu_cli")
    toml = tmp_path / "wolff.toml"
    toml.write_text(
        'model = "Ising"\nalgorithm = "Wolff"\n[sample.unitcell]\nname = "sc"\n'
        "[sample.size]\nx = 10\ny = 10\nz = 10\n[sample.pbc]\nx = true\ny = true\nz = true\n"
        '[[stages]]\nprogram = "Relax"\nsteps = 100\ntemperature = 6.0\n'
        '[[stages]]\nprogram = "CoolDown"\nmax_temperature = 6.0\nmin_temperature = 1.0\ncool_rate = 0.5\n'
        "relax = 50\nsteps = 200\n"
        f'[output]\nobservables = "{tmp_path}/obs.parquet"\n')
    r = subprocess.run([cli, "run", str(toml), "-s", "3"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    rows = [list(map(float, ln.split())) for ln in r.stdout.strip().splitlines()]
    assert len(rows) == 11  # CoolDown(6.0, 1.0, 0.5)
    # ordered at T = 1: energy per spin near the ground state of the Compound total (-6)
    assert rows[-1][2] / 1000 < -5.5 and rows[-1][4] / 1000 > 0.95
    assert (tmp_path / "obs.parquet").exists()


def test_grid_barrier_wait_runs_out_and_context_stays_usable(V):
    """A grid barrier one block never reaches: the others' bounded waits end
    after 2 s with VG_ERR_TIMEOUT (no fault, no hang); the same context then
    completes a barrier and runs multi-block Wolff steps bit-exactly."""
    import time

    lib = V.lib()
    with V.Engine(V.Lattice.sc(8, 8, 8), V.hamiltonian(V.Exchange(1.0)), seed=3) as eng:
        assert lib.vg_selftest_grid_barrier(eng._h, -1) == 0
        t0 = time.perf_counter()
        assert lib.vg_selftest_grid_barrier(eng._h, 2) == 3  # VG_ERR_TIMEOUT
        assert 1.5 < time.perf_counter() - t0 < 30.0
        assert b"ran out" in lib.vg_last_error(eng._h)
        assert lib.vg_selftest_grid_barrier(eng._h, -1) == 0
        eng.init_random()
        eng.set_thermostat(4.5)
        eng.sweeps(2)


def test_grid_wolff_after_barrier_self_test(V, O):
    """The self-test's barrier block does not stand in for the multi-block
    kernel's other buffers: a grid Wolff run on the same context is exact."""
    lat = V.Lattice.sc(96, 96, 96)
    with V.Engine(lat, V.hamiltonian(V.Exchange(1.0)), seed=12) as eng:
        assert V.lib().vg_selftest_grid_barrier(eng._h, 1) == 3
        eng.init_random()
        s0 = eng.get_state()
        eng.set_thermostat(4.5)
        eng.wolff_steps(3)
        g = O.Graph(O.lattice("sc", 96, 96, 96))
        ref, _ = g.wolff_steps(s0, 1.0, 4.5, 12, 0, 3)
        assert np.array_equal(eng.get_state(), ref)
