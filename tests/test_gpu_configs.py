"""Parity at the benchmarked configurations themselves, against the CPU oracle.

Each case runs the exact lattice, Hamiltonian and kernel path that bench.py
times, for a few sweeps (the oracle's share is bounded to tens of seconds):

* plain Ising sc 256^3, full PBC, J = 1, h = 0 (the two-pass checkerboard
  kernels the bench times, and the one-launch-per-sweep tiled kernel):
  spins and per-sweep bond / magnetisation sums bit-exact against the
  colour-order oracle (same Philox draws);
* Heisenberg sc 128^3, J = 1, K = 0.1 along z, B = 0.05 along z: one sweep in
  FP64 to 1e-12 per component, and in FP32 to 2e-6 per component with at
  most 0.1 % of decisions differing;
* the 256-replica multi-spin-coded batch (64 x 2D 64^2, 64 x 2D 512^2 on
  T 2.0-2.6, 64 x 3D 32^3, 64 x 3D 128^3 on T 4.2-4.8, geometric ladders,
  exchange every 10 sweeps) for two rounds: the per-round anti-aligned bond and
  up-spin counts of every replica, the ladders and swap counts bit-exact, and
  the full spin arrays of lanes 0, 17 and 31 of every word;
* the hysteresis batch, fcc 64^3 cells x 64 replicas (8 seeds x 8 cubic
  constants), T = 0.5, one field point (B_z = +5) in FP64: three replicas'
  spins to 1e-9 and their per-point sums to 1e-9 relative.

Reference update rules: src/integrator.rs:66-137, energies src/energy.rs:82-213.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SEED = 20261203


@pytest.mark.parametrize("path", ["structured", "tiled"])
def test_ising_sc256_bit_exact(V, O, path):
    """The bench's default path (the two-pass checkerboard kernels, AUTO)
    and the one-launch-per-sweep kernel on shared-memory tiles; five sweeps,
    so that the tiled run also ends with one two-pass sweep."""
    L, T, n = 256, 4.5, 5
    want = V.PATH_TILED if path == "tiled" else V.PATH_STRUCTURED
    with V.Engine(V.Lattice.sc(L, L, L), V.hamiltonian(V.Exchange(1.0)), spin=V.SPIN_ISING, seed=SEED,
                  path=V.PATH_AUTO if path == "structured" else want) as eng:
        assert eng.info().path == want
        eng.init_random()
        s0 = eng.get_state()
        g = O.Graph(O.lattice("sc", L, L, L))
        assert np.array_equal(s0, g.ising_init(SEED))
        eng.set_thermostat(T)
        E, M = eng.sweeps(n)
        ref, obs = g.ising_sweeps(s0, 1.0, 0.0, T, SEED, 0, n)
        got = eng.get_state()
        assert np.array_equal(got, ref), f"{int((got != ref).sum())} of {ref.size} spins differ"
        np.testing.assert_array_equal(E, -obs[:, 0].astype(float))
        np.testing.assert_array_equal(M, np.abs(obs[:, 1]).astype(float))
        assert (got != s0).mean() > 0.1  # the sweeps did flip spins


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_heisenberg_sc128_follows_oracle(V, O, precision):
    L, T, K, mag = 128, 1.0, 0.1, 0.05
    fp64 = precision == "fp64"
    H = V.hamiltonian(V.Exchange(1.0), V.UniaxialAnisotropy((0, 0, 1), K), V.Zeeman())
    with V.Engine(V.Lattice.sc(L, L, L), H, spin=V.SPIN_HEISENBERG, seed=SEED,
                  precision=V.FP64 if fp64 else V.FP32) as eng:
        assert eng.info().path == V.PATH_STRUCTURED
        eng.init_random()
        s0 = eng.get_state()
        eng.set_thermostat(T, (0, 0, 1), mag)
        sums = eng.sweeps_sums(1)
        s1 = eng.get_state()
    g = O.Graph(O.lattice("sc", L, L, L))
    r0 = g.heis_init(SEED)
    assert np.abs(s0 - r0).max() < (1e-12 if fp64 else 1e-6)
    P = O.HeisParams(J=1.0, K=K, hz=mag, Kc=0.0, T=T)
    P.axis[:] = (0, 0, 1)
    P.b[:] = (0, 0, 1)
    ref, obs = g.heis_sweeps(s0, P, SEED, 0, 1)
    tol = 1e-12 if fp64 else 2e-6
    same = np.all(np.abs(s1 - ref) < tol, axis=1)
    moved = np.any(np.abs(s1 - s0) > 1e-3, axis=1).mean()
    assert moved > 0.05
    if fp64:
        assert same.all(), f"{int((~same).sum())} of {same.size} spins differ"
        np.testing.assert_allclose(sums[0, :7], obs[0, :7], rtol=1e-12, atol=1e-8)
    else:
        assert same.mean() >= 0.999, same.mean()
        n = L ** 3
        scale = np.array([3 * n, n, n, n, n, n, n])
        assert np.all(np.abs(sums[0, :7] - obs[0, :7]) <= 1e-5 * scale)


def test_msc_batch_256_replicas_bit_exact(V, O):
    """The full c4 batch under three launch shapes (the default, the shape the
    bench's autotuner picks on a GB300 and two words in flight at two words per
    thread) against one oracle run: the round's last pass tallies the
    per-replica observables, so every shape must reproduce them exactly."""
    every, rounds = 10, 2
    t2 = np.geomspace(2.0, 2.6, 64)
    t3 = np.geomspace(4.2, 4.8, 64)
    shapes = [((64, 64, 1), (1, 1, 0), t2), ((512, 512, 1), (1, 1, 0), t2), ((32, 32, 32), (1, 1, 1), t3),
              ((128, 128, 128), (1, 1, 1), t3)]
    gpu = [(V.Lattice.sc(*e, pbc=tuple(bool(p) for p in pb)), t) for e, pb, t in shapes]
    cpu = [(O.lattice("sc", *e, pb), t) for e, pb, t in shapes]
    ref = O.MscBatch(cpu)
    ref.init(SEED)
    obs_ref, acc_ref = ref.run(1.0, SEED, 0, 0, every, rounds, True)
    assert acc_ref.sum() > 0
    for tuning in (None, (128, 8, 2), (256, 2, 2)):
        with V.Batch(gpu, J=1.0, seed=SEED, sweeps_per_round=every, exchange=True) as b:
            assert b.info().total_replicas == 256
            if tuning:
                b.set_tuning(*tuning)
            b.init_random()
            b.run(rounds)
            for rd in range(rounds):
                counts, _ = b.observables(rd)
                assert np.array_equal(counts, obs_ref[rd]), f"{tuning}, round {rd}: per-replica counts differ"
            off = 0
            for gi, g in enumerate(ref.groups):
                assert np.array_equal(b.ladder(gi), g["tau"]), f"{tuning}, group {gi}: ladder differs"
                acc, _ = b.swap_stats(gi)
                n = g["temps"].size
                assert np.array_equal(acc, acc_ref[off:off + n]), f"{tuning}, group {gi}: swap counts differ"
                off += n
                for w in range(n // 32):
                    for lane in (0, 17, 31):
                        r = 32 * w + lane
                        assert np.array_equal(b.get_replica(gi, r), g["spins"][r]), (tuning, gi, r)


def test_hysteresis_fcc64_x64_fp64_follows_oracle(V, O):
    from test_gpu_hbatch import _oracle_run

    L, T = 64, 0.5
    reps = [V.HeisReplica(seed=SEED + 7919 * (r // 8), replica=r, temperature=T, exchange=1.0, anisotropy=0.0,
                          cubic=0.1 * (r % 8) / 7) for r in range(64)]
    fields = np.array([5.0])
    relax, measure = 1, 1
    zsign = -1.0
    with V.HysteresisBatch(V.Lattice.fcc(L, L, L), reps, field_axis=(0, 0, 1), zeeman_sign=zsign,
                           precision=V.FP64) as hb:
        hb.init_random()
        picks = (0, 27, 63)
        s0 = {r: hb.get_replica(r) for r in picks}
        sums = hb.run(fields, relax, measure)
        got = {r: hb.get_replica(r) for r in picks}
    olat = O.lattice("fcc", L, L, L)
    for r in picks:
        want_s, want = _oracle_run(O, olat, reps[r], s0[r].reshape(-1), fields, relax, measure, zsign,
                                   (0.0, 0.0, 1.0), (0.0, 0.0, 1.0))
        same = np.all(np.abs(got[r] - want_s.reshape(-1, 3)) < 1e-9, axis=1)
        assert same.all(), f"replica {r}: {int((~same).sum())} of {same.size} spins differ"
        np.testing.assert_allclose(sums[:, r, :], want, rtol=1e-9, atol=1e-8, err_msg=f"replica {r}")
