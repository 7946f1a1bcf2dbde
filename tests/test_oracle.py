"""The oracle pinned against the reference's own known answers (CPU only)."""
import json
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "reference_known_answers.json")


@pytest.fixture(scope="module")
def gold():
    with open(GOLDEN) as f:
        return json.load(f)


def test_philox_known_answers(O, gold):
    for case in gold["philox4x32_10"]:
        ctr = [int(x, 16) for x in case["ctr"]]
        key = [int(x, 16) for x in case["key"]]
        assert O.philox(ctr, key) == [int(x, 16) for x in case["out"]]


def _ham(O, terms, compound):
    H = O.Hamiltonian()
    H.zeeman_sign = 1.0
    H.compound = int(compound)
    for t in terms:
        if t[0] == "gauge":
            H.has_gauge, H.gauge = 1, t[1]
        elif t[0] == "anisotropy":
            H.has_anisotropy, H.K = 1, t[2]
            H.axis[:] = t[1]
        elif t[0] == "zeeman":
            H.has_zeeman = 1
        elif t[0] == "exchange":
            H.has_exchange, H.J = 1, t[1]
    return H


def test_reference_energy_known_answers(O, gold):
    # a 10-site chain stands in for the tests' bare 10-spin states (no exchange term)
    g = O.Graph(O.lattice("sc", 10, 1, 1, (True, False, False)))
    for case in gold["energy"]:
        sz = 1.0 if case["state"] == "up" else -1.0
        spins = np.zeros((10, 3))
        spins[:, 2] = sz
        H = _ham(O, case["terms"], case["compound"])
        b = case["field"]
        e = g.ref_total_energy(1, spins, H, b=b[:3], bmag=b[3])
        assert e == case["exact"], case["test"]
        kind, bound = case["assert"]
        if kind == "lt":
            assert e - bound < 1e-12, case["test"]
        else:
            assert e - bound < 1e-12 and e + (-bound) < 1e-12 + 2 * abs(bound), case["test"]


def test_reference_state_known_answers(O, gold):
    g = O.Graph(O.lattice("sc", 10, 1, 1, (True, False, False)))
    up = np.ones(10, dtype=np.int8)
    assert O.lib().vo_ref_magnetization(10, 0, up.ctypes.data_as(O.C.POINTER(O.C.c_int8)), None) == 10.0
    del g


def test_schedules_replay_reference_fp_loops(O, gold):
    t = O.cooldown_temperatures(4.0, 0.1, 0.1)
    assert t.size == 39 and t[0] == 4.0 and abs(t[-1] - 0.2) < 1e-9
    t = O.cooldown_temperatures(5.5, 3.5, 0.1)
    assert t.size == 21 and abs(t[-1] - 3.5) < 1e-9
    t = O.cooldown_temperatures(2.0, 0.2, 0.1)
    assert t.size == 18 and abs(t[-1] - 0.3) < 1e-9
    f = O.hysteresis_fields(5.0, 0.1)
    assert f.size == 255
    assert f.max() > 5.0 and f.min() < -5.0  # the loop overshoots both ends


def test_accumulator_formulas(O):
    x = np.array([1.0, 2.0, 3.0, 4.0])
    mean, var, binder = O.accumulate(x)
    assert mean == 2.5
    assert var == np.mean(x * x) - 2.5 ** 2
    assert binder == 1.0 - np.mean(x ** 4) / (3.0 * np.mean(x * x) ** 2)


@pytest.mark.parametrize("cell,z", [("sc", 6), ("bcc", 8), ("fcc", 12)])
def test_lattice_coordination_and_symmetry(O, cell, z):
    g = O.Graph(O.lattice(cell, 4, 4, 4))
    nb = g.neighbours()
    assert nb.shape == (g.n, z) and (nb >= 0).all()
    pairs = {}
    for i in range(g.n):
        for j in nb[i]:
            pairs[(i, int(j))] = pairs.get((i, int(j)), 0) + 1
    assert all(pairs[(i, j)] == pairs[(j, i)] for (i, j) in pairs)
    # ground state: bond energy -z N J / 2
    H = _ham(O, [("exchange", 1.0)], False)
    assert g.ref_total_energy(0, np.ones(g.n, dtype=np.int8), H) == -z * g.n / 2


@pytest.mark.parametrize("cell,ext,pbc,ncol", [
    ("sc", (4, 4, 4), (1, 1, 1), 2), ("sc", (5, 4, 4), (1, 1, 1), None), ("sc", (5, 4, 4), (0, 1, 1), 2),
    ("bcc", (3, 3, 3), (1, 1, 1), 2), ("fcc", (4, 4, 4), (1, 1, 1), 4), ("sc", (32, 32, 1), (1, 1, 0), 2)])
def test_greedy_colouring_is_proper(O, cell, ext, pbc, ncol):
    g = O.Graph(O.lattice(cell, *ext, pbc))
    assert g.colouring_valid()
    if ncol is None:  # an odd periodic cycle: greedy needs more than two colours
        assert 3 <= g.ncolours <= 7
    else:
        assert g.ncolours == ncol


def test_checkerboard_is_the_greedy_colouring(O):
    g = O.Graph(O.lattice("sc", 6, 4, 2))
    x = np.arange(g.n) % 6
    y = (np.arange(g.n) // 6) % 4
    z = np.arange(g.n) // 24
    assert np.array_equal(g.colour, (x + y + z) % 2)


def test_ising_threshold_rule(O):
    # dE <= 0 always accepts; otherwise ceil(exp(-dE/T) 2^32)
    assert O.ising_threshold(1.0, 0.0, 2.0, 1, -2) == 1 << 32
    assert O.ising_threshold(1.0, 0.0, 2.0, 1, 0) == 1 << 32
    thr = O.ising_threshold(1.0, 0.0, 2.0, 1, 2)  # dE = 4
    assert thr == int(np.ceil(np.exp(-2.0) * 2 ** 32))
    assert O.ising_threshold(1.0, 0.0, 2.220446049250313e-16, 1, 6) == 0


def test_colour_oracle_is_deterministic_and_conserves_sums(O):
    g = O.Graph(O.lattice("sc", 8, 8, 8))
    s0 = g.ising_init(5)
    s1, obs1 = g.ising_sweeps(s0, 1.0, 0.0, 4.0, 5, 0, 4)
    s2, obs2 = g.ising_sweeps(s0, 1.0, 0.0, 4.0, 5, 0, 4)
    assert np.array_equal(s1, s2) and np.array_equal(obs1, obs2)
    nb = g.neighbours()
    bond = int(sum(int(s1[i]) * int(s1[j]) for i in range(g.n) for j in nb[i])) // 2
    assert obs1[-1, 0] == bond and obs1[-1, 1] == int(s1.sum())


def test_heisenberg_oracle_sums_and_unit_norm(O):
    g = O.Graph(O.lattice("fcc", 3, 3, 3))
    s0 = g.heis_init(9)
    assert np.allclose(np.linalg.norm(s0, axis=1), 1.0, atol=1e-15)
    P = O.HeisParams(J=1.0, K=0.1, hz=0.2, Kc=0.05, T=0.7)
    P.axis[:] = (0, 0, 1)
    P.b[:] = (0, 0, 1)
    s1, obs = g.heis_sweeps(s0, P, 9, 0, 3)
    assert np.allclose(np.linalg.norm(s1, axis=1), 1.0, atol=1e-14)
    nb = g.neighbours()
    bond = sum(float(s1[i] @ s1[j]) for i in range(g.n) for j in nb[i]) / 2
    assert abs(obs[-1, 0] - bond) < 1e-9
    assert np.allclose(obs[-1, 4:7], s1.sum(0))


def test_proposal_is_uniform_on_sphere(O):
    rng = np.random.default_rng(0)
    w = rng.integers(0, 2 ** 32, size=(20000, 2), dtype=np.uint64)
    p = np.array([O.heis_proposal(int(a), int(b)) for a, b in w])
    assert np.allclose(np.linalg.norm(p, axis=1), 1.0, atol=1e-14)
    assert np.all(np.abs(p.mean(0)) < 0.02)
    assert np.allclose((p ** 2).mean(0), 1 / 3, atol=0.02)


def test_ref_cpu_limits(O):
    g = O.Graph(O.lattice("sc", 8, 8, 1, (1, 1, 0)))
    H = _ham(O, [("exchange", 1.0)], False)
    rng = O.pcg64(3)
    s = g.ising_init(1)
    _, obs = g.ref_sweeps(0, s, H, 0.3, 200, rng)
    assert obs[-1, 0] == -2 * g.n  # frozen into the ground state (E_bond = -2N)
    _, obs = g.ref_sweeps(0, s, H, 1e6, 200, rng)
    assert abs(obs[100:, 0].mean()) < 0.1 * 2 * g.n


def test_ref_cpu_matches_colour_oracle_statistically(O):
    """Both chains sample the same Boltzmann distribution (2D 8x8, T = 3)."""
    g = O.Graph(O.lattice("sc", 8, 8, 1, (1, 1, 0)))
    H = _ham(O, [("exchange", 1.0)], False)
    s = g.ising_init(2)
    _, ref = g.ref_sweeps(0, s, H, 3.0, 20000, O.pcg64(11))
    _, col = g.ising_sweeps(s, 1.0, 0.0, 3.0, 2, 0, 20000)
    e_ref = ref[1000:, 0]
    e_col = -col[1000:, 0].astype(float)

    def binned(x, nb=50):
        b = x[: len(x) // nb * nb].reshape(nb, -1).mean(1)
        return b.mean(), b.std(ddof=1) / np.sqrt(nb)

    (m1, s1), (m2, s2) = binned(e_ref), binned(e_col)
    assert abs(m1 - m2) < 3 * np.hypot(s1, s2)


def test_msc_oracle_matches_plane_by_plane_definition(O):
    """The batched oracle draws each 32-replica word's threshold planes once
    and compares them most significant first; a direct restatement of the
    draw definition (replica lane l's uniform U has bit 31-p equal to bit l of
    plane p = word p & 3 of Philox4x32-7(entry, sweep, 6 << 24 | colour << 8 |
    p >> 2, word)) gives the same spins after two sweeps."""
    seed, J = 77, 1.0
    lat = O.lattice("sc", 8, 6, 1, (1, 1, 0))
    temps = np.geomspace(1.5, 3.0, 32)
    ref = O.MscBatch([(lat, temps)])
    ref.init(seed)
    g = ref.groups[0]
    spins = g["spins"].copy()
    ref.run(J, seed, 0, 0, 2, 1, exchange=False)
    graph = O.Graph(lat)
    nb, col = graph.neighbours(), graph.colour
    rank = np.zeros(graph.n, dtype=np.int64)
    for c in range(graph.ncolours):
        idx = np.nonzero(col == c)[0]
        rank[idx] = np.arange(idx.size)
    z = 4
    for sweep in range(2):
        for c in range(2):
            for i in np.nonzero(col == c)[0]:
                planes = []
                for r in range(32):
                    s = spins[r]
                    na = sum(1 for q in nb[i] if q >= 0 and s[q] != s[i])
                    th = O.ising_threshold(J, 0.0, max(temps[r], 2.220446049250313e-16), 1, z - 2 * na)
                    if th >= 1 << 32:
                        acc = True
                    else:
                        if not planes:
                            planes = sum((O.philox([int(rank[i]), sweep, (6 << 24) | (c << 8) | b, 0], [seed, 0],
                                                   rounds=O.MSC_ROUNDS) for b in range(8)), [])
                        u = 0
                        for p in range(32):
                            u |= ((planes[p] >> r) & 1) << (31 - p)
                        acc = u < th
                    if acc:
                        s[i] = -s[i]
    assert np.array_equal(spins, g["spins"])


def test_exact_finite_torus_energy_matches_enumeration():
    """Kaufman's finite-torus partition function (used by the Onsager checks)
    against brute-force sums over every state of small tori."""
    import itertools

    import exact_ising2d as X

    for m, n in ((3, 3), (2, 4), (4, 4)):
        for T in (1.5, 2.269, 4.0):
            e = np.array(list(itertools.product((-1, 1), repeat=m * n)), dtype=np.int64).reshape(-1, m, n)
            bond = (e * np.roll(e, 1, axis=1)).sum(axis=(1, 2)) + (e * np.roll(e, 1, axis=2)).sum(axis=(1, 2))
            w = np.exp((bond - bond.max()) / T)
            u = -(bond * w).sum() / w.sum() / (m * n)
            assert abs(X.energy_per_spin(T, m, n) - u) < 1e-10, (m, n, T)


def test_philox_round_count(O):
    """The reduced-round function is the 10-round one cut short: 10 rounds
    reproduce vo_philox4x32_10, fewer rounds give other words."""
    ctr, key = [1, 2, 3, 4], [5, 6]
    assert O.philox(ctr, key, rounds=10) == O.philox(ctr, key)
    lib = O.lib()
    import ctypes as C

    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib.vo_philox4x32_r(c, k, 10, o)
    assert list(o) == O.philox(ctr, key)
    assert O.philox(ctr, key, rounds=7) != O.philox(ctr, key)


def test_heisenberg_draws_use_the_reduced_round_function(O):
    """One oracle Heisenberg sweep at a temperature where every move accepts
    sets each site to the proposal built from its Philox4x32-HEIS_ROUNDS block
    (counter: class entry, sweep, tag 3 << 24 | colour << 8, replica)."""
    seed = 5
    g = O.Graph(O.lattice("sc", 4, 4, 4, (1, 1, 1)))
    s0 = g.heis_init(seed)
    P = O.HeisParams(J=1.0, K=0.0, hz=0.0, Kc=0.0, T=1e12)
    s1, _ = g.heis_sweeps(s0, P, seed, 0, 1, proposal=O.PROPOSE_RANDOM)
    assert O.HEIS_ROUNDS == 7
    for c in range(g.ncolours):
        for j, i in enumerate(np.nonzero(g.colour == c)[0]):
            w = O.philox([int(j), 0, (3 << 24) | (c << 8), 0], [seed, 0], rounds=O.HEIS_ROUNDS)
            np.testing.assert_array_equal(s1[i], O.heis_proposal(w[0], w[1]))
