"""Physics parity: the exact 2D result (Onsager; Kaufman on the finite torus),
and the reference CPU Metropolis (ref_cpu restatement) against the GPU
colour-class chain, within 3 combined binning standard errors."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def onsager_energy_per_spin(T, J=1.0):
    """Exact bond energy per spin of the infinite 2D square-lattice Ising model."""
    from scipy.special import ellipk

    b = J / T
    k = 2.0 * np.sinh(2 * b) / np.cosh(2 * b) ** 2
    return -J / np.tanh(2 * b) * (1.0 + (2.0 / np.pi) * (2.0 * np.tanh(2 * b) ** 2 - 1.0) * ellipk(k * k))


def binned(x, nbins=40):
    x = np.asarray(x, dtype=np.float64)
    b = x[: len(x) // nbins * nbins].reshape(nbins, -1).mean(1)
    return b.mean(), b.std(ddof=1) / np.sqrt(nbins)


def jackknife_var(x, nbins=40, scale=1.0):
    x = np.asarray(x, dtype=np.float64)
    x = x[: len(x) // nbins * nbins].reshape(nbins, -1)
    tot_s, tot_s2, m = x.sum(), (x * x).sum(), x.size
    vals = []
    for i in range(nbins):
        s = tot_s - x[i].sum()
        s2 = tot_s2 - (x[i] * x[i]).sum()
        k = m - x.shape[1]
        vals.append((s2 / k - (s / k) ** 2) * scale)
    vals = np.array(vals)
    full = (tot_s2 / m - (tot_s / m) ** 2) * scale
    return full, np.sqrt((nbins - 1) / nbins * ((vals - vals.mean()) ** 2).sum())


@pytest.mark.parametrize("T", [2.0, 2.3, 3.0])
def test_onsager_energy_finite_torus(V, T):
    """Energy per spin of the 2D Ising model against the exact value on the
    same finite torus (Kaufman's partition function, exact_ising2d.py): 64 x 64
    sites, 32 independent chains (5000 sweeps to equilibrate, 20000 measured),
    error = standard error over chains, limit 3 standard errors.  Near T_c
    (T = 2.3) the finite-size shift of the energy against the infinite lattice
    (1.3e-2 at L = 64, 7e-5 at L = 256) is in the exact value, not in the
    tolerance."""
    import exact_ising2d as X

    L, R, therm, meas = 64, 32, 5000, 20000
    H = V.hamiltonian(V.Exchange(1.0))
    engines = [V.Engine(V.Lattice.sc(L, L, 1, pbc=(True, True, False)), H, seed=17 + r, replica=r) for r in range(R)]
    try:
        for e in engines:
            e.init_random()
            e.set_thermostat(T)
            e.sweeps_async(therm, measure=False)
            e.sweeps_async(meas, measure=True)
        u = np.array([-e.read_sums(meas)[:, 0].mean() / (L * L) for e in engines])  # Exchange total: -J bond
    finally:
        for e in engines:
            e.close()
    mean, err = u.mean(), u.std(ddof=1) / np.sqrt(R)
    exact = X.energy_per_spin(T, L, L)
    assert abs(mean - exact) < 3 * err, (T, mean, err, exact)
    # the infinite-lattice value (Onsager) agrees away from T_c, where the
    # finite-size shift is far below the error
    if T != 2.3:
        assert abs(exact - onsager_energy_per_spin(T)) < 1e-9


def _ref_vs_gpu_ising(V, O, T, L=32, sweeps=30000, therm=2000):
    H = V.hamiltonian(V.Exchange(1.0), V.Zeeman())  # the CLI's hamiltonian (src/input.rs:271)
    lat = V.Lattice.sc(L, L, 1, pbc=(True, True, False))
    with V.Engine(lat, H, seed=int(T * 1000)) as eng:
        eng.init_random()
        eng.set_thermostat(T)
        eng.sweeps(therm, measure=False)
        Eg, Mg = eng.sweeps(sweeps)
    g = O.Graph(O.lattice("sc", L, L, 1, (1, 1, 0)))
    Hr = O.Hamiltonian(has_exchange=1, J=1.0, has_zeeman=1, zeeman_sign=1.0, compound=1)
    s = g.ising_init(3)
    _, obs = g.ref_sweeps(0, s, Hr, T, therm + sweeps, O.pcg64(int(T * 77)), proposal=O.PROPOSE_FLIP)
    return (Eg, Mg), (obs[therm:, 0], obs[therm:, 1])


@pytest.mark.parametrize("T", [1.8, 2.4, 3.5])
def test_ising_matches_reference_cpu(V, O, T):
    L = 32
    N = L * L
    (Eg, Mg), (Er, Mr) = _ref_vs_gpu_ising(V, O, T, L)
    for a, b in ((Eg / N, Er / N), (Mg / N, Mr / N)):
        (m1, e1), (m2, e2) = binned(a), binned(b)
        assert abs(m1 - m2) < 3 * np.hypot(e1, e2), (T, m1, e1, m2, e2)
    # specific heat Var(E)/(N T^2) (src/instrument.rs:119-122), jackknife errors
    c1, d1 = jackknife_var(Eg, scale=1.0 / (N * T * T))
    c2, d2 = jackknife_var(Er, scale=1.0 / (N * T * T))
    assert abs(c1 - c2) < 3 * np.hypot(d1, d2), (T, c1, d1, c2, d2)
    # susceptibility Var(|M|)/(N T) (src/instrument.rs:123-126)
    x1, f1 = jackknife_var(Mg, scale=1.0 / (N * T))
    x2, f2 = jackknife_var(Mr, scale=1.0 / (N * T))
    assert abs(x1 - x2) < 3 * np.hypot(f1, f2), (T, x1, f1, x2, f2)


def test_ising_3d_matches_reference_cpu(V, O):
    """sc 16^3, full PBC, T = 4.0 (ordered side of the transition)."""
    T, L, therm, sweeps = 4.0, 16, 2000, 20000
    N = L ** 3
    H = V.hamiltonian(V.Exchange(1.0), V.Zeeman())
    with V.Engine(V.Lattice.sc(L, L, L), H, seed=23) as eng:
        eng.init_random()
        eng.set_thermostat(T)
        eng.sweeps(therm, measure=False)
        Eg, Mg = eng.sweeps(sweeps)
    g = O.Graph(O.lattice("sc", L, L, L))
    Hr = O.Hamiltonian(has_exchange=1, J=1.0, has_zeeman=1, zeeman_sign=1.0, compound=1)
    _, obs = g.ref_sweeps(0, g.ising_init(4), Hr, T, therm + sweeps, O.pcg64(99), proposal=O.PROPOSE_FLIP)
    Er, Mr = obs[therm:, 0], obs[therm:, 1]
    for a, b in ((Eg / N, Er / N), (Mg / N, Mr / N)):
        (m1, e1), (m2, e2) = binned(a), binned(b)
        assert abs(m1 - m2) < 3 * np.hypot(e1, e2), (m1, e1, m2, e2)
    c1, d1 = jackknife_var(Eg, scale=1.0 / (N * T * T))
    c2, d2 = jackknife_var(Er, scale=1.0 / (N * T * T))
    assert abs(c1 - c2) < 3 * np.hypot(d1, d2), (c1, d1, c2, d2)


def test_heisenberg_matches_reference_cpu(V, O):
    """Heisenberg sc 8^3 with Exchange + Anisotropy + Zeeman (config-3 terms), FP32 GPU vs FP64 CPU."""
    T, mag, K = 1.0, 0.05, 0.1
    H = V.hamiltonian(V.Exchange(1.0), V.UniaxialAnisotropy((0, 0, 1), K), V.Zeeman())
    lat = V.Lattice.sc(8, 8, 8)
    with V.Engine(lat, H, spin=V.SPIN_HEISENBERG, seed=5) as eng:
        eng.init_random()
        eng.set_thermostat(T, (0, 0, 1), mag)
        eng.sweeps(1000, measure=False)
        Eg, Mg = eng.sweeps(20000)
    g = O.Graph(O.lattice("sc", 8, 8, 8))
    Hr = O.Hamiltonian(has_exchange=1, J=1.0, has_anisotropy=1, K=K, has_zeeman=1, zeeman_sign=1.0, compound=1)
    Hr.axis[:] = (0, 0, 1)
    s = g.heis_init(8)
    _, obs = g.ref_sweeps(1, s, Hr, T, 21000, O.pcg64(9), b=(0, 0, 1), bmag=mag, proposal=O.PROPOSE_RANDOM)
    N = lat.n_sites
    for a, b in ((Eg / N, obs[1000:, 0] / N), (Mg / N, obs[1000:, 1] / N)):
        (m1, e1), (m2, e2) = binned(a), binned(b)
        assert abs(m1 - m2) < 3 * np.hypot(e1, e2), (m1, e1, m2, e2)
    c1, d1 = jackknife_var(Eg, scale=1.0 / (N * T * T))
    c2, d2 = jackknife_var(obs[1000:, 0], scale=1.0 / (N * T * T))
    assert abs(c1 - c2) < 3 * np.hypot(d1, d2), (c1, d1, c2, d2)
    x1, f1 = jackknife_var(Mg, scale=1.0 / (N * T))
    x2, f2 = jackknife_var(obs[1000:, 1], scale=1.0 / (N * T))
    assert abs(x1 - x2) < 3 * np.hypot(f1, f2), (x1, f1, x2, f2)
