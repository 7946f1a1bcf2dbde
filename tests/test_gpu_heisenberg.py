"""Heisenberg colour-class sweeps on the GPU against the FP64 CPU oracle.

Tolerances: the FP64 kernels follow the oracle to 1e-12 per spin component
(acceptance decisions may differ only where u ~ exp(-dE/T) to ~1e-15, allowed
for at most 0.1% of sites); the FP32 kernels to 2e-6 per component for sites
that took the same decision, with at most 0.1% of decisions differing.
Lattice sums in FP32 agree with FP64 sums of the same state to 1e-6 relative
(of the sum of |terms|).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LATTICES = [
    ("sc", (8, 8, 8), (1, 1, 1)),        # structured checkerboard
    ("sc", (8, 6, 5), (1, 1, 0)),        # structured, open z
    ("sc", (7, 4, 4), (1, 1, 1)),        # generic (odd x)
    ("bcc", (4, 4, 4), (1, 1, 1)),       # sublattice planes, runs of 4 cells
    ("fcc", (3, 3, 3), (1, 1, 1)),       # sublattice planes, runs of 1 cell
    ("bcc", (8, 4, 3), (1, 0, 1)),       # runs of 4, open y
    ("fcc", (5, 3, 4), (0, 1, 1)),       # runs of 1, open x
    ("fcc", (4, 2, 3), (1, 1, 0)),       # runs of 4, open z
]


def _params(O, J, K, axis, hz, b, Kc, T):
    P = O.HeisParams(J=J, K=K, hz=hz, Kc=Kc, T=T)
    P.axis[:] = axis
    P.b[:] = b
    return P


def _run(V, O, cell, ext, pbc, precision, proposal, n=2, seed=21, **opts):
    J, K, axis, mag, b, T = 1.0, 0.1, (0.0, 0.0, 1.0), 0.05, (0.0, 0.6, 0.8), 0.9
    H = V.hamiltonian(V.Exchange(J), V.UniaxialAnisotropy(axis, K), V.Zeeman())
    lat = getattr(V.Lattice, cell)(*ext, pbc=tuple(bool(p) for p in pbc))
    with V.Engine(lat, H, spin=V.SPIN_HEISENBERG, seed=seed, precision=precision, proposal=proposal, **opts) as eng:
        if opts:  # a grid of one warp per SM: threads walk several runs of four cells
            assert lat.n_sites // (4 * (2 if cell == "bcc" else 4)) > eng.info().sm_count * 32
        eng.init_random()
        s0 = eng.get_state()
        eng.set_thermostat(T, b, mag)
        sums = eng.sweeps_sums(n)
        s1 = eng.get_state()
        path = eng.info().path
    g = O.Graph(O.lattice(cell, *ext, pbc))
    ref0 = g.heis_init(seed)
    P = _params(O, J, K, axis, mag, b, 0.0, T)
    ref1, obs = g.heis_sweeps(s0, P, seed, 0, n, proposal=proposal)
    return s0, ref0, s1, ref1, sums, obs, path


@pytest.mark.parametrize("cell,ext,pbc", LATTICES)
@pytest.mark.parametrize("proposal", [1, 0])
def test_fp64_follows_oracle(V, O, cell, ext, pbc, proposal):
    s0, ref0, s1, ref1, sums, obs, _ = _run(V, O, cell, ext, pbc, V.FP64, proposal)
    assert np.abs(s0 - ref0).max() < 1e-12
    same = np.all(np.abs(s1 - ref1) < 1e-12, axis=1)
    assert same.mean() >= 0.999
    if same.all():
        np.testing.assert_allclose(sums[-1, :7], obs[-1, :7], rtol=0, atol=1e-9)


@pytest.mark.parametrize("cell,ext,pbc", [("bcc", (32, 16, 40), (1, 1, 1)), ("fcc", (32, 24, 26), (1, 0, 1))])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_sublattice_runs_of_four_follow_oracle(V, O, cell, ext, pbc, precision):
    """bcc / fcc with x a multiple of 4 (float4 / double2 runs of four cells),
    on a grid of one warp per SM so that threads walk several runs."""
    fp64 = precision == "fp64"
    s0, ref0, s1, ref1, sums, obs, path = _run(V, O, cell, ext, pbc, V.FP64 if fp64 else V.FP32, 1, n=1,
                                               threads_per_block=32, blocks_per_sm=1)
    assert path == V.PATH_STRUCTURED
    tol = 1e-12 if fp64 else 2e-6
    same = np.all(np.abs(s1 - ref1) < tol, axis=1)
    assert same.mean() >= 0.999
    if fp64 and same.all():
        np.testing.assert_allclose(sums[-1, :7], obs[-1, :7], rtol=0, atol=1e-8)


@pytest.mark.parametrize("cell,ext,pbc", [("sc", (33, 24, 30), (1, 1, 1)), ("fcc", (9, 40, 40), (1, 1, 0))])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_generic_entry_batches_follow_oracle(V, O, cell, ext, pbc, precision):
    """The neighbour-table kernel on a grid narrower than its classes (152 x 64
    threads): two entries per thread at a time, the last pair partly past the
    class's end."""
    J, K, axis, mag, b, T, seed = 1.0, 0.1, (0.0, 0.0, 1.0), 0.05, (0.0, 0.6, 0.8), 0.9, 21
    fp64 = precision == "fp64"
    H = V.hamiltonian(V.Exchange(J), V.UniaxialAnisotropy(axis, K), V.Zeeman())
    lat = getattr(V.Lattice, cell)(*ext, pbc=tuple(bool(p) for p in pbc))
    with V.Engine(lat, H, spin=V.SPIN_HEISENBERG, seed=seed, precision=V.FP64 if fp64 else V.FP32, proposal=1,
                  path=V.PATH_GENERIC, threads_per_block=64, blocks_per_sm=1) as eng:
        assert eng.info().path == V.PATH_GENERIC
        eng.init_random()
        s0 = eng.get_state()
        eng.set_thermostat(T, b, mag)
        sums = eng.sweeps_sums(1)
        s1 = eng.get_state()
    g = O.Graph(O.lattice(cell, *ext, pbc))
    ref1, obs = g.heis_sweeps(s0, _params(O, J, K, axis, mag, b, 0.0, T), seed, 0, 1, proposal=1)
    same = np.all(np.abs(s1 - ref1) < (1e-12 if fp64 else 2e-6), axis=1)
    assert same.mean() >= 0.999
    if fp64 and same.all():
        np.testing.assert_allclose(sums[-1, :7], obs[-1, :7], rtol=0, atol=1e-8)


@pytest.mark.parametrize("cell,ext,pbc", [("sc", (2, 2, 2), (1, 1, 1)), ("sc", (3, 2, 1), (1, 1, 0)),
                                          ("bcc", (1, 1, 1), (1, 1, 1)), ("fcc", (1, 1, 1), (1, 1, 1)),
                                          ("fcc", (1, 2, 1), (1, 0, 1))])
def test_tiny_periodic_lattices_follow_oracle(V, O, cell, ext, pbc):
    """Periodic axes of extent 1 or 2 (neighbour lists that repeat a site,
    three- or four-class colourings): FP64 against the oracle."""
    s0, ref0, s1, ref1, sums, obs, _ = _run(V, O, cell, ext, pbc, V.FP64, 1, n=4)
    assert np.abs(s0 - ref0).max() < 1e-12
    assert np.abs(s1 - ref1).max() < 1e-12
    np.testing.assert_allclose(sums[-1, :7], obs[-1, :7], rtol=0, atol=1e-9)


@pytest.mark.parametrize("cell,ext,pbc", LATTICES)
def test_fp32_follows_oracle(V, O, cell, ext, pbc):
    s0, ref0, s1, ref1, sums, obs, _ = _run(V, O, cell, ext, pbc, V.FP32, 1, n=1)
    assert np.abs(s0 - ref0).max() < 2e-6
    # re-run the oracle from the FP32 start state so only the sweep itself is compared
    d = np.abs(s1 - ref1).max(axis=1)
    assert (d < 2e-6).mean() >= 0.999
    norms = np.linalg.norm(s1, axis=1)
    assert np.abs(norms - 1).max() < 1e-6


@pytest.mark.parametrize("cell,ext,pbc", [("bcc", (8, 6, 4), (1, 1, 1)), ("fcc", (4, 5, 3), (1, 0, 1)),
                                          ("fcc", (3, 4, 4), (0, 1, 1))])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_sublattice_and_generic_paths_agree(V, cell, ext, pbc, precision):
    """bcc / fcc Heisenberg: the sublattice kernel and the ELL kernel draw the
    same numbers; their fields differ only in FP summation order."""
    prec = V.FP64 if precision == "fp64" else V.FP32
    tol = 1e-12 if precision == "fp64" else 2e-6
    H = V.hamiltonian(V.Exchange(1.0), V.UniaxialAnisotropy((0.0, 0.6, 0.8), 0.2), V.Zeeman(), V.CubicAnisotropy(0.05))
    lat = getattr(V.Lattice, cell)(*ext, pbc=tuple(bool(p) for p in pbc))
    out = []
    for path in (V.PATH_STRUCTURED, V.PATH_GENERIC):
        with V.Engine(lat, H, spin=V.SPIN_HEISENBERG, seed=9, precision=prec, path=path,
                      proposal=V.PROPOSE_RANDOM) as eng:
            assert eng.info().path == path
            eng.init_random()
            eng.set_thermostat(0.8, (0.0, 0.0, 1.0), 0.3)
            sums = eng.sweeps_sums(3)
            out.append((eng.get_state(), sums, eng.current_sums()))
    same = np.all(np.abs(out[0][0] - out[1][0]) < tol, axis=1)
    assert same.mean() >= 0.999
    if same.all():
        n = lat.n_sites
        scale = np.array([12 * n, n, n, n, n, n, n, n])
        assert np.all(np.abs(out[0][1] - out[1][1]) <= 1e-5 * scale)
        assert np.all(np.abs(out[0][2][:7] - out[1][2][:7]) <= 1e-5 * scale[:7])


def test_fp32_sums_match_fp64_on_same_state(V):
    H = V.hamiltonian(V.Exchange(1.0), V.UniaxialAnisotropy((0, 0, 1), 0.1), V.Zeeman())
    lat = V.Lattice.sc(16, 16, 16)
    rng = np.random.default_rng(3)
    s = rng.normal(size=(lat.n_sites, 3))
    s /= np.linalg.norm(s, axis=1, keepdims=True)
    out = {}
    for prec in (V.FP32, V.FP64):
        with V.Engine(lat, H, spin=V.SPIN_HEISENBERG, seed=1, precision=prec) as eng:
            eng.set_state(s)
            eng.set_thermostat(1.0, (0, 0, 1), 0.05)
            out[prec] = eng.current_sums()
    scale = np.array([3 * lat.n_sites, lat.n_sites, lat.n_sites, lat.n_sites] + [lat.n_sites] * 3)
    assert np.all(np.abs(out[V.FP32][:7] - out[V.FP64][:7]) <= 1e-6 * scale)


def test_norms_do_not_drift(V):
    H = V.hamiltonian(V.Exchange(1.0))
    with V.Engine(V.Lattice.sc(32, 16, 16), H, spin=V.SPIN_HEISENBERG, seed=4) as eng:
        eng.init_random()
        eng.set_thermostat(0.7)
        eng.sweeps(200, measure=False)
        s = eng.get_state()
    assert np.abs(np.linalg.norm(s, axis=1) - 1.0).max() < 1e-6


def test_reference_known_answers_on_gpu(V):
    """The reference's energy unit tests (src/energy.rs:300-375) through the GPU totals."""
    import json
    import os

    gold = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_known_answers.json")))
    lat = V.Lattice.sc(10, 1, 1, pbc=(True, False, False))
    for case in gold["energy"]:
        terms = []
        for t in case["terms"]:
            if t[0] == "gauge":
                terms.append(V.Gauge(t[1]))
            elif t[0] == "anisotropy":
                terms.append(V.UniaxialAnisotropy(t[1], t[2]))
            elif t[0] == "zeeman":
                terms.append(V.Zeeman())
        H = V.hamiltonian(*terms)
        s = np.zeros((10, 3))
        s[:, 2] = 1.0 if case["state"] == "up" else -1.0
        with V.Engine(lat, H, spin=V.SPIN_HEISENBERG, seed=0, precision=V.FP64) as eng:
            eng.set_state(s)
            f = case["field"]
            eng.set_thermostat(1.0, f[:3], f[3])
            assert eng.total_energy() == pytest.approx(case["exact"], abs=1e-12), case["test"]
