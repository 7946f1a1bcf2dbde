"""Per-site energies (Hamiltonian::energy, src/energy.rs:45-52) and energy
changes of single-site proposals through the C ABI.

Site energies are FP64 and compared with the oracle's restatement of the
reference's site energies to 1e-12.  Energy changes run the sweeps' own
function in the context's precision: FP64 matches the oracle's FP64 energy
change to 1e-12 of the sum of the absolute terms, FP32 to 1e-6 of it
(|dE32 - dE64| <= 1e-6 sum|terms|, the terms being -J (p - s).s_j per
neighbour, K (p.e)^2, K (s.e)^2, |B| (p - s).b, Kc quart(p), Kc quart(s)).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LATS = [("sc", (8, 8, 8), (1, 1, 1)), ("sc", (8, 6, 5), (1, 1, 0)), ("bcc", (4, 4, 4), (1, 1, 1)),
        ("fcc", (3, 3, 3), (1, 0, 1))]
J, K, AXIS, G, MAG = 1.3, 0.2, (0.0, 0.6, 0.8), 0.5, 0.4


def _engine(V, cell, ext, pbc, spin, **kw):
    lat = getattr(V.Lattice, cell)(*ext, pbc=tuple(bool(p) for p in pbc))
    H = V.hamiltonian(V.Exchange(J), V.UniaxialAnisotropy(AXIS if spin == V.SPIN_HEISENBERG else (0, 0, 1), K),
                      V.Zeeman(), V.Gauge(G))
    return V.Engine(lat, H, spin=spin, seed=17, **kw)


def _oracle_H(O, spin_heis):
    H = O.Hamiltonian(has_exchange=1, J=J, has_anisotropy=1, K=K, has_zeeman=1, zeeman_sign=1.0, has_gauge=1,
                      gauge=G, compound=1)
    H.axis[:] = AXIS if spin_heis else (0.0, 0.0, 1.0)
    return H


def _unit(rng, n):
    v = rng.normal(size=(n, 3))
    return v / np.linalg.norm(v, axis=1, keepdims=True)


@pytest.mark.parametrize("cell,ext,pbc", LATS)
@pytest.mark.parametrize("heis", [False, True])
def test_site_energies_match_reference_restatement(V, O, cell, ext, pbc, heis):
    spin = V.SPIN_HEISENBERG if heis else V.SPIN_ISING
    b = (0.0, 0.6, 0.8) if heis else (0.0, 0.0, -1.0)
    with _engine(V, cell, ext, pbc, spin) as eng:
        eng.init_random()
        eng.set_thermostat(1.5, b, MAG)
        eng.sweeps(3)
        s = eng.get_state()
        e = eng.site_energies()
        total = eng.total_energy()
    g = O.Graph(O.lattice(cell, *ext, pbc))
    ref = g.ref_site_energies(1 if heis else 0, s, _oracle_H(O, heis), b, MAG)
    np.testing.assert_allclose(e, ref, rtol=0, atol=1e-12)
    # Compound: the total is the sum of the site energies (src/energy.rs:55-59);
    # the FP32 context forms its total from FP32 block sums
    tol = 1e-6 if heis else 1e-12
    assert abs(e.sum() - total) <= tol * max(1.0, np.abs(e).sum())


def _oracle_delta(O, g, s, p, b, Kc=0.0, jb=None, Jc=J):
    """FP64 energy changes and the sum of absolute terms, per site."""
    P = O.HeisParams(J=Jc, K=K, hz=MAG, Kc=Kc, T=1.0)
    P.axis[:] = AXIS
    P.b[:] = b
    n, z = g.n, g.zmax
    nbr = g.nbr.reshape(n, z)
    ax, bb = np.array(AXIS), np.array(b)
    de = np.empty(n)
    scale = np.empty(n)
    for i in range(n):
        h = np.zeros(3)
        ex = 0.0
        d = p[i] - s[i]
        for k in range(z):
            q = nbr[i, k]
            if q < 0:
                continue
            w = jb[i, k] if jb is not None else 1.0
            h += w * s[q]
            ex += abs(Jc * w * (d @ s[q]))
        de[i] = O.heis_delta(P, s[i], p[i], h)
        quart = lambda v: float((v ** 4).sum())  # noqa: E731
        scale[i] = (ex + K * ((p[i] @ ax) ** 2 + (s[i] @ ax) ** 2) + MAG * abs(d @ bb)
                    + abs(Kc) * (quart(p[i]) + quart(s[i])))
    return de, scale


@pytest.mark.parametrize("cell,ext,pbc", LATS)
@pytest.mark.parametrize("fp64", [False, True])
def test_delta_energies_against_fp64_oracle(V, O, cell, ext, pbc, fp64):
    b = (0.0, 0.6, 0.8)
    rng = np.random.default_rng(5)
    with _engine(V, cell, ext, pbc, V.SPIN_HEISENBERG, precision=V.FP64 if fp64 else V.FP32) as eng:
        n = eng.lattice.n_sites
        eng.set_state(_unit(rng, n))
        eng.set_thermostat(1.0, b, MAG)
        s = eng.get_state()  # the state as the context holds it (FP32 values exactly)
        p = _unit(rng, n)
        if not fp64:
            p = p.astype(np.float32).astype(np.float64)
        got = eng.delta_energies(p)
    g = O.Graph(O.lattice(cell, *ext, pbc))
    ref, scale = _oracle_delta(O, g, s, p, b)
    tol = 1e-12 if fp64 else 1e-6
    err = np.abs(got - ref)
    assert np.all(err <= tol * scale), (err / scale).max()


def test_delta_energies_with_cubic_term(V, O):
    b = (0.0, 0.0, 1.0)
    lat = V.Lattice.fcc(3, 3, 3)
    H = V.hamiltonian(V.Exchange(J), V.UniaxialAnisotropy(AXIS, K), V.Zeeman(), V.CubicAnisotropy(0.05))
    rng = np.random.default_rng(8)
    with V.Engine(lat, H, spin=V.SPIN_HEISENBERG, seed=3) as eng:
        eng.set_state(_unit(rng, lat.n_sites))
        eng.set_thermostat(0.5, b, MAG)
        s = eng.get_state()
        p = _unit(rng, lat.n_sites).astype(np.float32).astype(np.float64)
        got = eng.delta_energies(p)
    g = O.Graph(O.lattice("fcc", 3, 3, 3, (1, 1, 1)))
    ref, scale = _oracle_delta(O, g, s, p, b, Kc=0.05)
    assert np.all(np.abs(got - ref) <= 1e-6 * scale)


def test_delta_equals_change_of_site_energy(V):
    """dE of one site's proposal = that site's energy after minus before."""
    rng = np.random.default_rng(2)
    with _engine(V, "bcc", (4, 4, 4), (1, 1, 1), V.SPIN_HEISENBERG, precision=V.FP64) as eng:
        n = eng.lattice.n_sites
        eng.set_state(_unit(rng, n))
        eng.set_thermostat(1.0, (0.0, 0.6, 0.8), MAG)
        s = eng.get_state()
        p = _unit(rng, n)
        de = eng.delta_energies(p)
        before = eng.site_energies()
        for i in (0, 17, n - 1):
            t = s.copy()
            t[i] = p[i]
            eng.set_state(t)
            after = eng.site_energies()
            assert after[i] - before[i] == pytest.approx(de[i], abs=1e-12)


@pytest.mark.parametrize("heis", [False, True])
def test_site_energies_and_delta_with_bond_constants(V, O, heis):
    cell, ext, pbc = "bcc", (4, 4, 4), (1, 1, 1)
    spin = V.SPIN_HEISENBERG if heis else V.SPIN_ISING
    b = (0.0, 0.6, 0.8) if heis else (0.0, 0.0, 1.0)
    g = O.Graph(O.lattice(cell, *ext, pbc))
    jb = g.symmetric_bonds(np.random.default_rng(4)).reshape(g.n, g.zmax)
    with _engine(V, cell, ext, pbc, spin, path=V.PATH_GENERIC, precision=V.FP64) as eng:
        eng.set_exchange_bonds(jb)
        eng.init_random()
        eng.set_thermostat(1.0, b, MAG)
        s = eng.get_state()
        e = eng.site_energies()
        nbr = g.nbr.reshape(g.n, g.zmax)
        sv = s.astype(np.float64) if heis else s.astype(np.float64)[:, None] * np.array([0.0, 0.0, 1.0])
        ax = np.array(AXIS if heis else (0.0, 0.0, 1.0))
        ref = np.array([-sum(jb[i, k] * (sv[i] @ sv[nbr[i, k]]) for k in range(g.zmax) if nbr[i, k] >= 0)
                        for i in range(g.n)])
        ref += K * (sv @ ax) ** 2 + MAG * (sv @ np.array(b)) + G
        np.testing.assert_allclose(e, ref, rtol=0, atol=1e-12)
        if heis:
            p = _unit(np.random.default_rng(6), g.n)
            got = eng.delta_energies(p)
            de, scale = _oracle_delta(O, g, s, p, b, jb=jb, Jc=1.0)
            assert np.all(np.abs(got - de) <= 1e-12 * scale)


def test_delta_energies_rejected_for_ising(V):
    with _engine(V, "sc", (8, 8, 8), (1, 1, 1), V.SPIN_ISING) as eng:
        with pytest.raises(V.VegasGpuError) as e:
            eng.delta_energies(np.zeros((512, 3)))
        assert e.value.status == 5
