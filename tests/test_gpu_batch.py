"""Batched multi-spin-coded Ising (32 replicas per word) with replica exchange,
bit-exact against the single-replica oracle of the same draws."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _groups(V, O):
    t2 = np.geomspace(2.0, 2.6, 32)
    t3 = np.geomspace(4.2, 4.8, 64)
    gpu = [(V.Lattice.sc(16, 16, 1, pbc=(True, True, False)), t2), (V.Lattice.sc(8, 6, 4), t3)]
    cpu = [(O.lattice("sc", 16, 16, 1, (1, 1, 0)), t2), (O.lattice("sc", 8, 6, 4), t3)]
    return gpu, cpu


@pytest.mark.parametrize("exchange", [True, False])
def test_batch_matches_oracle(V, O, exchange):
    seed, every, rounds = 31, 3, 4
    gpu, cpu = _groups(V, O)
    ref = O.MscBatch(cpu)
    ref.init(seed)
    with V.Batch(gpu, J=1.0, seed=seed, sweeps_per_round=every, exchange=exchange) as b:
        b.init_random()
        for gi, g in enumerate(ref.groups):
            for r in (0, 5, 31):
                assert np.array_equal(b.get_replica(gi, r), g["spins"][r])
        b.run(rounds)
        obs_ref, acc_ref = ref.run(1.0, seed, 0, 0, every, rounds, exchange)
        for gi, g in enumerate(ref.groups):
            for r in range(g["temps"].size):
                assert np.array_equal(b.get_replica(gi, r), g["spins"][r]), (gi, r)
            assert np.array_equal(b.ladder(gi), g["tau"])
        off = 0
        for gi, g in enumerate(ref.groups):
            acc, att = b.swap_stats(gi)
            n = g["temps"].size
            assert np.array_equal(acc, acc_ref[off:off + n])
            off += n
        for rd in range(rounds):
            counts, tau = b.observables(rd)
            assert np.array_equal(counts, obs_ref[rd])
        if exchange:
            assert acc_ref.sum() > 0


def test_batch_resumes_across_runs(V, O):
    seed = 5
    gpu, cpu = _groups(V, O)
    ref = O.MscBatch(cpu)
    ref.init(seed)
    with V.Batch(gpu, J=1.0, seed=seed, sweeps_per_round=2) as b:
        b.init_random()
        b.run(2)
        b.run(3)
        ref.run(1.0, seed, 0, 0, 2, 5)
        for gi, g in enumerate(ref.groups):
            assert np.array_equal(b.ladder(gi), g["tau"])
            assert np.array_equal(b.get_replica(gi, 7), g["spins"][7])
        assert b.info().round_index == 5 and b.info().sweep_index == 10


def test_batch_physics_matches_single_lattice_engine(V):
    """At one temperature the packed replicas sample what the single-lattice engine samples."""
    T, L = 2.4, 32
    temps = np.full(32, T)
    with V.Batch([(V.Lattice.sc(L, L, 1, pbc=(True, True, False)), temps)], seed=3, sweeps_per_round=10,
                 exchange=False) as b:
        b.init_random()
        b.run(50)
        b.run(200)
        e = []
        for rd in range(200):
            counts, _ = b.observables(rd)
            e.append(-(2 * L * L - 2 * counts[:, 0]) / (L * L))
        e = np.array(e)  # rounds x replicas
    H = V.hamiltonian(V.Exchange(1.0))
    with V.Engine(V.Lattice.sc(L, L, 1, pbc=(True, True, False)), H, seed=9) as eng:
        eng.init_random()
        eng.set_thermostat(T)
        eng.sweeps(500, measure=False)
        E, _ = eng.sweeps(20000)
    u_batch = e.mean()
    err_batch = e.mean(axis=0).std(ddof=1) / np.sqrt(e.shape[1])
    blocks = (E / (L * L)).reshape(40, -1).mean(axis=1)
    u_eng, err_eng = blocks.mean(), blocks.std(ddof=1) / np.sqrt(40)
    assert abs(u_batch - u_eng) < 4 * np.hypot(err_batch, err_eng), (u_batch, err_batch, u_eng, err_eng)


def test_batch_rejects_bad_groups(V):
    with pytest.raises(V.VegasGpuError):
        V.Batch([(V.Lattice.sc(16, 16, 1, pbc=(True, True, False)), np.ones(20))])
    with pytest.raises(V.VegasGpuError):
        V.Batch([(V.Lattice.bcc(4, 4, 4), np.ones(32))])


def _snapshot(b, groups):
    spins = [[b.get_replica(gi, r) for r in range(t.size)] for gi, (_, t) in enumerate(groups)]
    ladders = [b.ladder(gi) for gi in range(len(groups))]
    stats = [b.swap_stats(gi) for gi in range(len(groups))]
    return spins, ladders, stats


@pytest.mark.parametrize("shape", [(128, 2, 1), (128, 8, 2), (256, 2, 2), (256, 8, 1)])
def test_every_launch_shape_gives_the_oracle_result(V, O, shape):
    seed, every, rounds = 17, 2, 3
    gpu, cpu = _groups(V, O)
    ref = O.MscBatch(cpu)
    ref.init(seed)
    with V.Batch(gpu, J=1.0, seed=seed, sweeps_per_round=every, exchange=True) as b:
        b.set_tuning(*shape)
        assert b.tuning() == shape
        b.init_random()
        b.run(rounds)
        obs_ref, _ = ref.run(1.0, seed, 0, 0, every, rounds, True)
        for gi, g in enumerate(ref.groups):
            for r in (0, 13, g["temps"].size - 1):
                assert np.array_equal(b.get_replica(gi, r), g["spins"][r]), (shape, gi, r)
            assert np.array_equal(b.ladder(gi), g["tau"])
        for rd in range(rounds):
            assert np.array_equal(b.observables(rd)[0], obs_ref[rd])


def test_autotune_leaves_the_trajectory_unchanged(V, O, tmp_path):
    seed, every = 23, 2
    gpu, _ = _groups(V, O)
    with V.Batch(gpu, J=1.0, seed=seed, sweeps_per_round=every) as a, \
            V.Batch(gpu, J=1.0, seed=seed, sweeps_per_round=every) as c:
        a.init_random()
        c.init_random()
        a.run(3)
        c.run(3)
        obs_before = [a.observables(rd)[0] for rd in range(3)]
        cache = str(tmp_path / "tune.json")
        shape, ms = a.autotune(rounds=1, cache=cache)
        assert ms is not None and ms > 0 and a.tuning() == shape
        # the last run's observables and the counters survive the tuning rounds
        assert [np.array_equal(a.observables(rd)[0], o) for rd, o in enumerate(obs_before)] == [True] * 3
        assert a.info().sweep_index == c.info().sweep_index and a.info().round_index == c.info().round_index
        a.run(2)
        c.run(2)
        sa, sc = _snapshot(a, gpu), _snapshot(c, gpu)
        for x, y in zip(sa[0], sc[0]):
            for u, v in zip(x, y):
                assert np.array_equal(u, v)
        for x, y in zip(sa[1], sc[1]):
            assert np.array_equal(x, y)
        for (x1, x2), (y1, y2) in zip(sa[2], sc[2]):
            assert np.array_equal(x1, y1) and np.array_equal(x2, y2)
        # a second batch of the same shape takes the cached shape without timing
        with V.Batch(gpu, J=1.0, seed=1, sweeps_per_round=every) as d:
            shape2, ms2 = d.autotune(cache=cache)
            assert shape2 == shape and ms2 is None and d.tuning() == shape


def test_unsupported_tuning_is_rejected(V, O):
    gpu, _ = _groups(V, O)
    with V.Batch(gpu, J=1.0, seed=1) as b:
        with pytest.raises(V.VegasGpuError) as e:
            b.set_tuning(512, 4, 1)
        assert e.value.status == 5
