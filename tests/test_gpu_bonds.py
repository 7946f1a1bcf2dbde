"""Per-bond exchange constants (Exchange's CSR with arbitrary J_ij) on the
generic path, against the oracle's per-bond sweeps (same draws)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LATS = [("bcc", (4, 4, 4), (1, 1, 1)), ("fcc", (3, 3, 3), (1, 1, 0)), ("sc", (16, 4, 4), (1, 1, 1))]


def _setup(V, O, cell, ext, pbc, spin, seed, **kw):
    lat = getattr(V.Lattice, cell)(*ext, pbc=tuple(bool(p) for p in pbc))
    g = O.Graph(O.lattice(cell, *ext, pbc))
    jb = g.symmetric_bonds(np.random.default_rng(seed))
    H = V.hamiltonian(V.Exchange(1.0), V.Zeeman()) if spin == V.SPIN_ISING else \
        V.hamiltonian(V.Exchange(1.0), V.UniaxialAnisotropy((0, 0, 1), 0.1), V.Zeeman())
    eng = V.Engine(lat, H, spin=spin, seed=seed, path=V.PATH_GENERIC, **kw)
    return eng, g, jb


@pytest.mark.parametrize("cell,ext,pbc", LATS)
@pytest.mark.parametrize("proposal", [0, 1])
def test_ising_bonds_bit_exact(V, O, cell, ext, pbc, proposal):
    seed, T, mag, n = 41, 2.7, 0.3, 5
    eng, g, jb = _setup(V, O, cell, ext, pbc, V.SPIN_ISING, seed, proposal=proposal)
    with eng:
        eng.set_exchange_bonds(jb)
        eng.init_random()
        s0 = eng.get_state()
        eng.set_thermostat(T, (0, 0, -1), mag)
        sums = eng.sweeps_sums(n)
        ref, obs = g.ising_sweeps_bonds(s0, jb, -mag, T, seed, 0, n, proposal=proposal)
        assert np.array_equal(eng.get_state(), ref)
        np.testing.assert_allclose(sums[:, 0], obs[:, 0], rtol=0, atol=1e-9)   # sum J_ij s_i s_j
        np.testing.assert_array_equal(sums[:, 6], obs[:, 1])                  # magnetisation
        E = eng.total_energy()
        # Compound total: -2 sum J_ij s_i s_j + |B| sum s.b (b down)
        bond, m = obs[-1]
        assert abs(E - (-2.0 * bond + mag * (-m))) < 1e-9


@pytest.mark.parametrize("cell,ext,pbc", [("bcc", (9, 30, 30), (1, 1, 1)), ("fcc", (9, 40, 40), (1, 1, 0))])
def test_ising_bonds_entry_batches_bit_exact(V, O, cell, ext, pbc):
    """A grid narrower than the class (152 x 64 threads): two entries per
    thread at a time, the last pair partly past the class's end."""
    seed, T, mag, n = 43, 2.9, 0.25, 3
    eng, g, jb = _setup(V, O, cell, ext, pbc, V.SPIN_ISING, seed, threads_per_block=64, blocks_per_sm=1)
    with eng:
        eng.set_exchange_bonds(jb)
        eng.init_random()
        s0 = eng.get_state()
        eng.set_thermostat(T, (0, 0, 1), mag)
        sums = eng.sweeps_sums(n)
        ref, obs = g.ising_sweeps_bonds(s0, jb, mag, T, seed, 0, n)
        assert np.array_equal(eng.get_state(), ref)
        np.testing.assert_allclose(sums[:, 0], obs[:, 0], rtol=0, atol=1e-9)
        np.testing.assert_array_equal(sums[:, 6], obs[:, 1])


def test_uniform_bonds_equal_the_uniform_constant(V, O):
    lat = V.Lattice.bcc(4, 4, 4)
    H = V.hamiltonian(V.Exchange(1.0))
    out = []
    for bonds in (False, True):
        with V.Engine(lat, H, seed=3, path=V.PATH_GENERIC) as eng:
            if bonds:
                eng.set_exchange_bonds(np.ones((lat.n_sites, 8)))
            eng.init_random()
            eng.set_thermostat(3.0)
            E, M = eng.sweeps(6)
            out.append((eng.get_state(), E, M))
    assert np.array_equal(out[0][0], out[1][0])
    np.testing.assert_allclose(out[0][1], out[1][1], rtol=1e-12)
    np.testing.assert_array_equal(out[0][2], out[1][2])


@pytest.mark.parametrize("cell,ext,pbc", LATS[:2])
def test_heisenberg_bonds_match_oracle_fp64(V, O, cell, ext, pbc):
    seed, T, mag, n = 9, 1.1, 0.2, 3
    eng, g, jb = _setup(V, O, cell, ext, pbc, V.SPIN_HEISENBERG, seed, precision=V.FP64)
    with eng:
        eng.set_exchange_bonds(jb)
        eng.init_random()
        s0 = eng.get_state()
        eng.set_thermostat(T, (0, 0, 1), mag)
        sums = eng.sweeps_sums(n)
        P = O.HeisParams(J=1.0, K=0.1, hz=mag, Kc=0.0, T=T)
        P.axis[:] = (0, 0, 1)
        P.b[:] = (0, 0, 1)
        ref, obs = g.heis_sweeps_bonds(s0, jb, P, seed, 0, n)
        got = eng.get_state()
        same = np.all(np.abs(got - ref) < 1e-9, axis=1)
        assert same.mean() > 0.999
        if same.all():
            np.testing.assert_allclose(sums[:, 0], obs[:, 0], rtol=1e-9, atol=1e-9)


def test_bonds_are_validated(V, O):
    lat = V.Lattice.bcc(3, 3, 3)
    H = V.hamiltonian(V.Exchange(1.0))
    with V.Engine(V.Lattice.sc(64, 16, 10), H, seed=1) as eng:  # structured path
        with pytest.raises(V.VegasGpuError) as e:
            eng.set_exchange_bonds(np.ones((64 * 16 * 10, 6)))
        assert e.value.status == 5
    with V.Engine(lat, H, seed=1, path=V.PATH_GENERIC) as eng:
        with pytest.raises(V.VegasGpuError) as e:
            eng.set_exchange_bonds(np.ones((lat.n_sites, 7)))
        assert e.value.status == 1
        jb = np.ones((lat.n_sites, 8))
        jb[0, 0] = 2.0  # breaks J_ij == J_ji
        with pytest.raises(V.VegasGpuError) as e:
            eng.set_exchange_bonds(jb)
        assert "symmetric" in str(e.value)
        eng.set_exchange_bonds(np.full((lat.n_sites, 8), 0.5))
        eng.set_exchange_bonds(None)
        eng.init_random()
        eng.sweeps(2)
