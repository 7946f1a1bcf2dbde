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
