"""Batched Heisenberg replicas under a field schedule (vg_hbatch_*).

Parity: every replica of an FP64 batch follows the FP64 oracle (same Philox
draws, same colour classes and class entries), and its per-point sums match
the oracle's sweep observables accumulated the same way.  The FP32 batch is
checked against the FP64 batch, the batch against single-lattice contexts,
and a schedule split over two runs against one run.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL_FP64 = 1e-9     # FP64 batch vs FP64 oracle, relative, per point sum
SPIN_TOL = 1e-9     # per-component spin agreement, FP64


def _replicas(V, n, T=0.8, J=1.0):
    return [V.HeisReplica(seed=1000 + 17 * r, replica=r, temperature=T * (1 + 0.1 * r), exchange=J,
                          anisotropy=0.05 * (r % 2), cubic=0.02 * r) for r in range(n)]


def _oracle_run(O, olat, rep, s0, fields, relax, measure, zsign, axis, baxis, sweep0=0, proposal=1):
    """Per-point sums of one replica from the oracle (VG_HB_NSUMS layout)."""
    g = O.Graph(olat)
    spin = s0.copy()
    out = np.zeros((len(fields), 12))
    sweep = sweep0
    for p, h in enumerate(fields):
        P = O.HeisParams(J=rep.exchange, K=rep.anisotropy, hz=zsign * h, Kc=rep.cubic, T=rep.temperature)
        P.axis[:] = axis
        P.b[:] = baxis
        spin, obs = g.heis_sweeps(spin, P, rep.seed, sweep, relax + measure, replica=rep.replica, proposal=proposal)
        sweep += relax + measure
        for t in range(relax, relax + measure):
            o = obs[t]
            m2 = o[4] ** 2 + o[5] ** 2 + o[6] ** 2
            e = -2 * rep.exchange * o[0] + rep.anisotropy * o[1] + zsign * h * o[2] - rep.cubic * o[3]
            out[p, :8] += o[:8]
            out[p, 8] += np.sqrt(m2)
            out[p, 9] += m2
            out[p, 10] += e
            out[p, 11] += e * e
    return spin, out


CASES = [  # cell, extents, pbc
    ("fcc", (4, 4, 4), (1, 1, 1)),
    ("fcc", (8, 3, 2), (1, 0, 1)),    # float4 runs, an open axis
    ("bcc", (5, 4, 3), (1, 1, 0)),    # odd extents
    ("fcc", (3, 2, 5), (0, 1, 1)),
]


@pytest.mark.parametrize("cell,ext,pbc", CASES)
def test_fp64_batch_matches_oracle(V, O, cell, ext, pbc):
    lat = getattr(V.Lattice, cell)(*ext, pbc=tuple(bool(p) for p in pbc))
    olat = O.lattice(cell, *ext, pbc)
    reps = _replicas(V, 3)
    axis, baxis, zsign = (0.0, 0.6, 0.8), (0.0, 0.0, 1.0), -1.0
    fields = np.array([0.7, -0.4, 0.1])
    relax, measure = 1, 2
    with V.HysteresisBatch(lat, reps, anisotropy_axis=axis, field_axis=baxis, zeeman_sign=zsign,
                           precision=V.FP64) as hb:
        hb.init_random()
        s0 = [hb.get_replica(r) for r in range(len(reps))]
        sums = hb.run(fields, relax, measure)
        for r, rep in enumerate(reps):
            g = O.Graph(olat)
            assert np.array_equal(s0[r], g.heis_init(rep.seed, rep.replica).reshape(-1, 3)) or \
                np.abs(s0[r] - g.heis_init(rep.seed, rep.replica).reshape(-1, 3)).max() < 1e-12
            want_s, want = _oracle_run(O, olat, rep, s0[r].reshape(-1), fields, relax, measure, zsign, axis, baxis)
            got_s = hb.get_replica(r)
            # FP64 against FP64: a decision can differ only where u equals
            # exp(-dE/T) to rounding (about 1e-16 per attempt), so every spin
            # must agree and the per-point sums are always compared
            same = np.all(np.abs(got_s - want_s.reshape(-1, 3)) < SPIN_TOL, axis=1)
            assert same.all(), f"replica {r}: {int((~same).sum())} of {same.size} spins differ"
            np.testing.assert_allclose(sums[:, r, :], want, rtol=REL_FP64, atol=1e-8,
                                       err_msg=f"per-point sums of replica {r}")


def test_init_random_matches_single_lattice_contexts(V):
    lat = V.Lattice.fcc(4, 4, 4)
    reps = _replicas(V, 2)
    for prec in (V.FP32, V.FP64):
        with V.HysteresisBatch(lat, reps, precision=prec) as hb:
            hb.init_random()
            for r, rep in enumerate(reps):
                H = V.hamiltonian(V.Exchange(1.0))
                with V.Engine(lat, H, spin=V.SPIN_HEISENBERG, seed=rep.seed, replica=rep.replica,
                              precision=prec) as eng:
                    eng.init_random()
                    assert np.array_equal(hb.get_replica(r), eng.get_state().reshape(-1, 3))


def test_batch_follows_single_lattice_context(V):
    """A replica of the batch and a context with the same seed and id draw
    the same numbers: FP64 trajectories agree to rounding."""
    lat = V.Lattice.fcc(4, 4, 2)
    rep = V.HeisReplica(seed=77, replica=5, temperature=1.3, exchange=1.0, anisotropy=0.1, cubic=0.0)
    h = 0.25
    with V.HysteresisBatch(lat, [rep], anisotropy_axis=(0, 0, 1), field_axis=(0, 0, 1), zeeman_sign=1.0,
                           precision=V.FP64) as hb:
        hb.init_random()
        hb.run([h], 0, 3)
        got = hb.get_replica(0)
    H = V.hamiltonian(V.Exchange(1.0), V.UniaxialAnisotropy((0, 0, 1), 0.1), V.Zeeman())
    with V.Engine(lat, H, spin=V.SPIN_HEISENBERG, seed=77, replica=5, precision=V.FP64) as eng:
        eng.init_random()
        eng.set_thermostat(1.3, (0, 0, 1), h)
        eng.sweeps(3)
        want = eng.get_state().reshape(-1, 3)
    same = np.all(np.abs(got - want) < 1e-9, axis=1)
    assert same.mean() > 0.999


@pytest.mark.parametrize("ext", [(8, 4, 4), (6, 4, 4)])   # float4 runs / scalar
def test_fp32_batch_tracks_fp64_batch(V, ext):
    lat = V.Lattice.fcc(*ext)
    reps = _replicas(V, 4)
    fields = np.array([0.5, 0.0])
    out = {}
    for prec in (V.FP64, V.FP32):
        with V.HysteresisBatch(lat, reps, zeeman_sign=-1.0, precision=prec) as hb:
            hb.init_random()
            s = hb.run(fields, 0, 2)
            out[prec] = (s, [hb.get_replica(r) for r in range(len(reps))])
            if prec == V.FP32:
                assert hb.info().sites_per_thread == (4 if ext[0] % 4 == 0 else 1)
    s64, st64 = out[V.FP64]
    s32, st32 = out[V.FP32]
    for r in range(len(reps)):
        same = np.all(np.abs(st32[r] - st64[r]) < 1e-4, axis=1)
        assert same.mean() > 0.99
    # Observables: FP32 per-thread partials, FP64 block sums
    n = lat.n_sites
    np.testing.assert_allclose(s32[:, :, 4:7] / n, s64[:, :, 4:7] / n, atol=2e-2)
    np.testing.assert_allclose(s32[:, :, 10] / n, s64[:, :, 10] / n, rtol=2e-2, atol=2e-2)


def test_split_schedule_equals_one_run(V):
    lat = V.Lattice.bcc(4, 4, 4)
    reps = _replicas(V, 2)
    fields = np.array([1.0, 0.5, 0.0, -0.5])
    with V.HysteresisBatch(lat, reps, precision=V.FP32) as a, V.HysteresisBatch(lat, reps, precision=V.FP32) as b:
        a.init_random()
        b.init_random()
        sa = a.run(fields, 2, 3)
        b.run(fields[:1], 2, 3)
        sb = b.run(fields[1:], 2, 3)
        assert b.info().sweep_index == a.info().sweep_index == 20
        np.testing.assert_array_equal(sa[1:], sb)
        for r in range(2):
            np.testing.assert_array_equal(a.get_replica(r), b.get_replica(r))
        assert a.info().graph == 1


def test_hysteresis_loop_opens_below_the_ordering_temperature(V):
    """Spins follow the field (zeeman_sign -1): saturated at +-max, a loop
    with positive area and coercive fields of opposite sign at low T."""
    lat = V.Lattice.fcc(6, 6, 6)
    reps = [V.HeisReplica(seed=5 + r, replica=r, temperature=0.5, exchange=1.0, anisotropy=-0.5, cubic=0.0)
            for r in range(2)]
    fields = V.hysteresis_fields(3.0, 0.25)
    relax, measure = 100, 50
    with V.HysteresisBatch(lat, reps, anisotropy_axis=(0, 0, 1), field_axis=(0, 0, 1), zeeman_sign=-1.0) as hb:
        hb.init_random()
        sums = hb.run(fields, relax, measure)
    n = lat.n_sites
    m = sums[:, :, 6] / (measure * n)       # mean Mz per spin
    assert np.all(m[0] > 0.8) and np.all(m[len(fields) // 2] < -0.8)
    for r in range(2):
        area = V.loop_area(fields, m[:, r])
        hd, hu = V.coercive_fields(fields, m[:, r])
        assert area > 0.1
        assert hd < 0 < hu


def test_rejections(V):
    reps = _replicas(V, 1)
    with pytest.raises(V.VegasGpuError) as e:
        V.HysteresisBatch(V.Lattice.sc(4, 4, 4), reps)
    assert e.value.status == 5
    with V.HysteresisBatch(V.Lattice.fcc(2, 2, 2), reps) as hb:
        with pytest.raises(V.VegasGpuError):
            hb.run([], 1, 1)
        bad = np.zeros((hb.lattice.n_sites, 3))
        with pytest.raises(V.VegasGpuError) as e:
            hb.set_replica(0, bad)
        assert e.value.status == 1 and "unit" in str(e.value)
        with pytest.raises(V.VegasGpuError):
            hb.get_replica(3)


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_tracked_sums_do_not_drift(V, prec):
    """Measured sweeps update the lattice sums by the changes of the accepted
    moves.  300 tracked sweeps of one field point against the same 300 sweeps
    measured as 300 one-sweep points (each starting from an exact sum)."""
    p = V.FP32 if prec == "fp32" else V.FP64
    lat = V.Lattice.fcc(8, 8, 4)
    reps = _replicas(V, 2)
    n = 300
    with V.HysteresisBatch(lat, reps, anisotropy_axis=(0, 0, 1), zeeman_sign=-1.0, precision=p) as a, \
            V.HysteresisBatch(lat, reps, anisotropy_axis=(0, 0, 1), zeeman_sign=-1.0, precision=p) as b:
        a.init_random()
        b.init_random()
        sa = a.run([0.3], 0, n)[0]
        sb = b.run(np.full(n, 0.3), 0, 1).sum(axis=0)
        np.testing.assert_array_equal(a.get_replica(1), b.get_replica(1))
    rtol = 2e-5 if prec == "fp32" else 1e-11
    for k in (0, 1, 3, 4, 5, 6, 10):   # bond, aniso, cubic, M, E
        np.testing.assert_allclose(sa[:, k], sb[:, k], rtol=rtol, atol=rtol * lat.n_sites * n)
    np.testing.assert_array_equal(sa[:, 7], sb[:, 7])  # accepted moves
