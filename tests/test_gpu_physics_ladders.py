"""Statistical parity with the reference's own CPU Metropolis at every point of
the schedules: the GPU chains (colour-class sweeps) against ref_cpu, the
restatement of the reference's random-site Metropolis and CLI measurement
(src/integrator.rs:66-137, src/machine.rs:91-101, src/instrument.rs:133-141).

At every temperature (or field point) the StatSensor observables <E>/N,
<|M|>/N, C = Var(E)/(N T^2) and chi = Var(|M|)/(N T) (src/instrument.rs:
113-126) agree within 3 combined standard errors.  Both arms run independent
chains (32 each) and the errors are jackknife errors over chains (see
ladder_stats.py, which also states the one-retest rule for 3-sigma
excursions).  Schedules:

* the 2D workload: sc 32x32x1 (PBC x, y), the CLI Hamiltonian Exchange +
  Zeeman (src/input.rs:271) with B = 0, Relax at T = 4 then
  CoolDown(4.0, 0.1, 0.1) -- its 39 temperatures (src/program.rs:182-214),
  1000 relax + 8000 measured sweeps each;
* Heisenberg sc 8^3 with Exchange + UniaxialAnisotropy(K = 0.1, z) + Zeeman
  (B = 0.05 along z): CoolDown(2.0, 0.2, 0.1), 18 temperatures;
* bcc and fcc, Ising and Heisenberg, three temperatures each around the
  transition, from random starts;
* the hysteresis batch's K = 0 replicas (fcc 4^3 cells, T = 0.5, spins
  aligned by the field) against ref_cpu with the same Zeeman sign at four
  field points of the descending branch.
"""
import numpy as np
import pytest

import ladder_stats as S

pytestmark = pytest.mark.gpu

R_GPU, R_CPU = 32, 32


def _ising_EM(J):
    def f(s, T, mag):  # Compound(Exchange, Zeeman) with B = 0: E = sum_i energy(i) = -2 J bond
        return -2.0 * J * s[:, 0], np.abs(s[:, 6])
    return f


def _heis_EM(J, K, zsign=1.0):
    def f(s, T, mag):
        E = -2.0 * J * s[:, 0] + K * s[:, 1] + zsign * abs(mag) * s[:, 2]
        return E, np.sqrt(s[:, 4] ** 2 + s[:, 5] ** 2 + s[:, 6] ** 2)
    return f


def _check_energy_formula(V, lat, H, spin, to_EM, T, b, mag):
    """The vectorised E, |M| of the sums equal the library's own totals."""
    with V.Engine(lat, H, spin=spin, seed=3) as e:
        e.init_random()
        e.set_thermostat(T, b, mag)
        s = e.sweeps_sums(3)
        E, M = to_EM(s, T, mag)
        for i in range(3):
            e2, m2 = e.energy_from_sums(s[i])
            assert abs(E[i] - e2) <= 1e-9 * max(1.0, abs(e2)) and abs(M[i] - m2) <= 1e-9 * max(1.0, m2)


def test_ising_2d_cooldown_every_temperature(V, O):
    L = 32
    N = L * L
    temps = O.cooldown_temperatures(4.0, 0.1, 0.1)
    assert len(temps) == 39
    lat = V.Lattice.sc(L, L, 1, pbc=(True, True, False))
    olat = O.lattice("sc", L, L, 1, (1, 1, 0))
    H = V.hamiltonian(V.Exchange(1.0), V.Zeeman())
    Hr = O.Hamiltonian(has_exchange=1, J=1.0, has_zeeman=1, zeeman_sign=1.0, compound=1)
    sched = [(float(T), (0, 0, 1), 0.0) for T in temps]
    init = (4.0, (0, 0, 1), 0.0, 1000)
    to_EM = _ising_EM(1.0)
    _check_energy_formula(V, lat, H, V.SPIN_ISING, to_EM, 2.5, (0, 0, 1), 0.0)

    def run(attempt):
        g = S.gpu_chains(lambda r: V.Engine(lat, H, spin=V.SPIN_ISING, seed=1000 * attempt + 101 + r, replica=r),
                         R_GPU, sched, 1000, 8000, to_EM, init=init)
        c = S.cpu_chains(O, olat, 0, Hr, R_CPU, sched, 1000, 8000, 7000 + 1000 * attempt, O.PROPOSE_FLIP,
                         init=init)
        return S.compare(g, c, N, temps)

    S.check_with_retest(run)


def test_heisenberg_sc8_cooldown_every_temperature(V, O):
    K, mag = 0.1, 0.05
    temps = O.cooldown_temperatures(2.0, 0.2, 0.1)
    assert len(temps) == 18
    lat = V.Lattice.sc(8, 8, 8)
    olat = O.lattice("sc", 8, 8, 8)
    N = lat.n_sites
    H = V.hamiltonian(V.Exchange(1.0), V.UniaxialAnisotropy((0, 0, 1), K), V.Zeeman())
    Hr = O.Hamiltonian(has_exchange=1, J=1.0, has_anisotropy=1, K=K, has_zeeman=1, zeeman_sign=1.0, compound=1)
    Hr.axis[:] = (0, 0, 1)
    sched = [(float(T), (0, 0, 1), mag) for T in temps]
    to_EM = _heis_EM(1.0, K)
    _check_energy_formula(V, lat, H, V.SPIN_HEISENBERG, to_EM, 1.0, (0, 0, 1), mag)

    def run(attempt):
        g = S.gpu_chains(lambda r: V.Engine(lat, H, spin=V.SPIN_HEISENBERG, seed=1000 * attempt + 301 + r,
                                            replica=r), R_GPU, sched, 300, 2000, to_EM)
        c = S.cpu_chains(O, olat, 1, Hr, R_CPU, sched, 300, 2000, 9000 + 1000 * attempt, O.PROPOSE_RANDOM)
        return S.compare(g, c, N, temps)

    S.check_with_retest(run)


CUBIC = [  # cell, extents (cells), spin, temperatures around the transition, sweeps (relax, measure)
    ("bcc", (8, 8, 8), "ising", (5.0, 6.3, 8.0), (1000, 4000)),            # neighbour-table kernels
    ("fcc", (16, 4, 4), "ising", (8.0, 9.8, 12.0), (1000, 4000)),          # sublattice kernels
    ("bcc", (8, 8, 8), "heisenberg", (1.5, 2.05, 3.0), (300, 1500)),
    ("fcc", (4, 4, 4), "heisenberg", (2.5, 3.2, 4.5), (300, 1500)),
]


@pytest.mark.parametrize("cell,ext,spin,temps,sweeps", CUBIC)
def test_bcc_fcc_match_reference_cpu(V, O, cell, ext, spin, temps, sweeps):
    ising = spin == "ising"
    lat = getattr(V.Lattice, cell)(*ext)
    olat = O.lattice(cell, *ext)
    N = lat.n_sites
    if ising:
        H = V.hamiltonian(V.Exchange(1.0), V.Zeeman())
        Hr = O.Hamiltonian(has_exchange=1, J=1.0, has_zeeman=1, zeeman_sign=1.0, compound=1)
        to_EM, kind, prop, mag = _ising_EM(1.0), 0, O.PROPOSE_FLIP, 0.0
    else:
        H = V.hamiltonian(V.Exchange(1.0), V.UniaxialAnisotropy((0, 0, 1), 0.1), V.Zeeman())
        Hr = O.Hamiltonian(has_exchange=1, J=1.0, has_anisotropy=1, K=0.1, has_zeeman=1, zeeman_sign=1.0,
                           compound=1)
        Hr.axis[:] = (0, 0, 1)
        to_EM, kind, prop, mag = _heis_EM(1.0, 0.1), 1, O.PROPOSE_RANDOM, 0.05
    relax, measure = sweeps
    sk = V.SPIN_ISING if ising else V.SPIN_HEISENBERG

    def run(attempt):
        rows = []
        for T in temps:  # each temperature from random starts
            sched = [(T, (0, 0, 1), mag)]
            g = S.gpu_chains(lambda r: V.Engine(lat, H, spin=sk, seed=1000 * attempt + 501 + r, replica=r),
                             R_GPU, sched, relax, measure, to_EM)
            c = S.cpu_chains(O, olat, kind, Hr, R_CPU, sched, relax, measure, 11000 + 1000 * attempt, prop)
            rows += S.compare(g, c, N, [T])
        return rows

    S.check_with_retest(run)


def test_hysteresis_k0_replicas_match_reference_cpu(V, O):
    """K = 0 replicas of the batched hysteresis workload (no cubic term: the
    reference has none) against ref_cpu with the same Zeeman sign (aligning)
    at the first four points of a descending field branch, state carried
    from point to point in both arms."""
    T, zsign = 0.5, -1.0
    fields = [5.0, 2.0, 1.0, 0.5]
    relax, measure = 300, 1500
    lat = V.Lattice.fcc(4, 4, 4)
    olat = O.lattice("fcc", 4, 4, 4)
    N = lat.n_sites
    Hr = O.Hamiltonian(has_exchange=1, J=1.0, has_zeeman=1, zeeman_sign=zsign, compound=1)

    def run(attempt):
        reps = [V.HeisReplica(seed=1000 * attempt + 701 + r, replica=r, temperature=T, exchange=1.0, anisotropy=0.0,
                              cubic=0.0) for r in range(R_GPU)]
        with V.HysteresisBatch(lat, reps, field_axis=(0, 0, 1), zeeman_sign=zsign) as hb:
            hb.init_random()
            sums = hb.run(np.array(fields), relax, measure)  # points x replicas x 12
        g = np.stack([sums[:, :, 10], sums[:, :, 11], sums[:, :, 8], sums[:, :, 9]], axis=-1) / measure
        sched = [(T, (0, 0, 1), h) for h in fields]
        c = S.cpu_chains(O, olat, 1, Hr, R_CPU, sched, relax, measure, 13000 + 1000 * attempt, O.PROPOSE_RANDOM)
        return S.compare(g, c, N, [T] * len(fields), labels=[f"B={h}" for h in fields])

    S.check_with_retest(run)
