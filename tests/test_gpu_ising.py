"""Ising colour-class sweeps on the GPU, bit-exact against the CPU oracle (same Philox draws)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = [
    # cell, extents, pbc, expected path (AUTO: small checkerboard lattices run resident)
    ("sc", (32, 4, 4), (1, 1, 1), "resident"),
    ("sc", (32, 32, 1), (1, 1, 0), "resident"),     # 2D square lattice, open z
    ("sc", (64, 6, 5), (1, 1, 0), "resident"),
    ("sc", (32, 5, 4), (0, 0, 1), "resident"),      # open x and y boundaries
    ("sc", (64, 16, 10), (1, 1, 1), "structured"),
    ("sc", (96, 18, 6), (1, 0, 1), "structured"),
    ("sc", (128, 8, 10), (1, 1, 1), "structured"),  # pairs of groups per thread
    ("sc", (256, 64, 1), (1, 1, 0), "structured"),  # pairs, 2D (open z of extent 1)
    ("sc", (16, 4, 4), (1, 1, 1), "generic"),       # x/2 not a multiple of 16
    ("sc", (33, 4, 4), (1, 1, 1), "generic"),       # odd periodic cycle: greedy colouring
    ("bcc", (4, 4, 4), (1, 1, 1), "generic"),
    ("bcc", (3, 5, 2), (1, 0, 1), "generic"),
    ("fcc", (4, 4, 4), (1, 1, 1), "generic"),
    ("fcc", (3, 3, 3), (1, 1, 0), "generic"),
    # bcc / fcc with x a multiple of 16: one array per sublattice, 16-cell runs
    ("bcc", (16, 4, 4), (1, 1, 1), "structured"),
    ("bcc", (16, 3, 2), (1, 0, 1), "structured"),   # open y
    ("bcc", (32, 2, 1), (0, 1, 1), "structured"),   # open x; z of extent 1 (doubled bonds)
    ("fcc", (16, 4, 4), (1, 1, 1), "structured"),
    ("fcc", (16, 3, 3), (1, 1, 0), "structured"),   # open z
    ("fcc", (32, 2, 5), (0, 1, 1), "structured"),   # open x
]
SUB = CASES[14:]


def _engine(V, cell, ext, pbc, ham, seed, **kw):
    lat = getattr(V.Lattice, cell)(*ext, pbc=tuple(bool(p) for p in pbc))
    return V.Engine(lat, ham, spin=V.SPIN_ISING, seed=seed, **kw)


@pytest.mark.parametrize("cell,ext,pbc,path", CASES)
def test_flip_sweeps_bit_exact(V, O, cell, ext, pbc, path):
    seed, J, T, n = 1234, 1.0, 3.2, 6
    with _engine(V, cell, ext, pbc, V.hamiltonian(V.Exchange(J)), seed) as eng:
        want = {"structured": V.PATH_STRUCTURED, "generic": V.PATH_GENERIC, "resident": V.PATH_RESIDENT}[path]
        assert eng.info().path == want
        eng.init_random()
        g = O.Graph(O.lattice(cell, *ext, pbc))
        s0 = g.ising_init(seed)
        assert np.array_equal(eng.get_state(), s0)
        eng.set_thermostat(T)
        E, M = eng.sweeps(n)
        ref, obs = g.ising_sweeps(s0, J, 0.0, T, seed, 0, n)
        assert np.array_equal(eng.get_state(), ref)
        np.testing.assert_array_equal(E, -J * obs[:, 0].astype(float))   # Exchange::total_energy = bond energy
        np.testing.assert_array_equal(M, np.abs(obs[:, 1]).astype(float))


@pytest.mark.parametrize("cell,ext,pbc,path", CASES[:2] + CASES[4:9] + SUB)
def test_random_proposal_and_field_bit_exact(V, O, cell, ext, pbc, path):
    """MetropolisIntegrator (random +-1 proposal) with Exchange + Zeeman, field Down."""
    seed, J, T, mag, n = 99, 0.7, 2.1, 0.35, 5
    H = V.hamiltonian(V.Exchange(J), V.Zeeman())
    with _engine(V, cell, ext, pbc, H, seed, proposal=V.PROPOSE_RANDOM) as eng:
        eng.init_random()
        g = O.Graph(O.lattice(cell, *ext, pbc))
        s0 = g.ising_init(seed)
        eng.set_thermostat(T, (0.0, 0.0, -1.0), mag)
        E, M = eng.sweeps(n)
        hz = 1.0 * mag * -1.0
        ref, obs = g.ising_sweeps(s0, J, hz, T, seed, 0, n, proposal=O.PROPOSE_RANDOM)
        assert np.array_equal(eng.get_state(), ref)
        bond, m = obs[:, 0].astype(float), obs[:, 1].astype(float)
        # Compound total: sum_i energy(i) = -2 J bond + |B| (s . b) summed
        np.testing.assert_allclose(E, -2 * J * bond + mag * (-m), rtol=0, atol=1e-9)
        np.testing.assert_array_equal(M, np.abs(m))


@pytest.mark.parametrize("proposal", [0, 1])
@pytest.mark.parametrize("ext,pbc", [((64, 8, 6), (1, 1, 1)), ((32, 32, 1), (1, 1, 0)), ((32, 6, 5), (0, 1, 0))])
def test_all_paths_agree(V, ext, pbc, proposal):
    """Grid checkerboard, generic ELL and resident shared-memory kernels draw identical numbers."""
    H = V.hamiltonian(V.Exchange(1.0), V.Zeeman())
    out = []
    for path in (V.PATH_STRUCTURED, V.PATH_GENERIC, V.PATH_RESIDENT):
        with _engine(V, "sc", ext, pbc, H, 5, path=path, proposal=proposal) as eng:
            assert eng.info().path == path
            eng.init_random()
            eng.set_thermostat(2.9, (0, 0, 1), 0.2)
            E, M = eng.sweeps(20)
            out.append((eng.get_state(), E, M))
    for o in out[1:]:
        assert np.array_equal(out[0][0], o[0])
        assert np.array_equal(out[0][1], o[1]) and np.array_equal(out[0][2], o[2])


@pytest.mark.parametrize("proposal", [0, 1])
@pytest.mark.parametrize("cell,ext,pbc", [(c, e, p) for c, e, p, _ in SUB])
def test_sublattice_and_generic_paths_agree(V, cell, ext, pbc, proposal):
    """bcc / fcc: the sublattice kernel and the ELL kernel give the same
    states and per-sweep sums, including the measurement-only pass."""
    H = V.hamiltonian(V.Exchange(0.8), V.Zeeman(), V.Gauge(0.1))
    out = []
    for path in (V.PATH_STRUCTURED, V.PATH_GENERIC):
        with _engine(V, cell, ext, pbc, H, 21, path=path, proposal=proposal) as eng:
            assert eng.info().path == path
            eng.init_random()
            eng.set_thermostat(3.7, (0, 0, -1), 0.3)
            sums = eng.sweeps_sums(70)
            out.append((eng.get_state(), sums, eng.total_energy(), eng.magnetization()[1]))
    assert np.array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])
    assert out[0][2] == out[1][2] and out[0][3] == out[1][3]


def test_sublattice_tie_queue_overflow_matches_generic(V):
    """A block keeps at most 512 tied entries for after its runs and decides
    the rest in line: with one warp per SM walking ~320 runs per thread
    (~650 ties per block) both happen; the result equals the ELL kernel's."""
    ext = (1024, 192, 128)
    H = V.hamiltonian(V.Exchange(1.0), V.Zeeman())
    out = []
    for path, opts in ((V.PATH_STRUCTURED, dict(threads_per_block=32, blocks_per_sm=1)), (V.PATH_GENERIC, {})):
        with _engine(V, "bcc", ext, (1, 1, 1), H, 31, path=path, **opts) as eng:
            assert eng.info().path == path
            if path == V.PATH_STRUCTURED:
                groups = ext[0] * ext[1] * ext[2] // 16
                assert groups // (eng.info().grid_blocks * 32) * 32 // 16 > 512
            eng.init_random()
            eng.set_thermostat(3.0, (0, 0, 1), 0.1)
            sums = eng.sweeps_sums(2)
            out.append((eng.get_state(), sums))
    assert np.array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])


def test_sublattice_needs_x_multiple_of_16(V):
    H = V.hamiltonian(V.Exchange(1.0))
    with pytest.raises(V.VegasGpuError) as e:
        _engine(V, "fcc", (24, 4, 4), (1, 1, 1), H, 1, path=V.PATH_STRUCTURED)
    assert e.value.status == 5
    with _engine(V, "fcc", (24, 4, 4), (1, 1, 1), H, 1) as eng:
        assert eng.info().path == V.PATH_GENERIC


@pytest.mark.parametrize("proposal", [0, 1])
@pytest.mark.parametrize("ext,pbc", [((128, 64, 20), (1, 1, 1)), ((512, 512, 1), (1, 1, 0))])
def test_pair_rounds_bit_exact(V, O, ext, pbc, proposal):
    """More 16-site groups than grid threads: the pass runs two groups per
    thread per round (a one-warp-per-SM grid)."""
    seed, J, T, mag, n = 77, 1.0, 4.4, 0.2, 3
    H = V.hamiltonian(V.Exchange(J), V.Zeeman())
    with _engine(V, "sc", ext, pbc, H, seed, path=V.PATH_STRUCTURED, proposal=proposal, threads_per_block=32,
                 blocks_per_sm=1) as eng:
        assert eng.info().grid_blocks * 32 < ext[0] * ext[1] * ext[2] // 32
        eng.init_random()
        g = O.Graph(O.lattice("sc", *ext, pbc))
        s0 = g.ising_init(seed)
        eng.set_thermostat(T, (0.0, 0.0, 1.0), mag)
        E, M = eng.sweeps(n)
        ref, obs = g.ising_sweeps(s0, J, mag, T, seed, 0, n, proposal=proposal)
        assert np.array_equal(eng.get_state(), ref)
        np.testing.assert_allclose(E, -2 * J * obs[:, 0] + mag * obs[:, 1], rtol=0, atol=1e-9)
        np.testing.assert_array_equal(M, np.abs(obs[:, 1]).astype(float))


def test_resume_from_sweep_index(V):
    """(seed, sweep index) is the whole RNG state: splitting a run changes nothing."""
    H = V.hamiltonian(V.Exchange(1.0))
    with _engine(V, "sc", (32, 8, 8), (1, 1, 1), H, 8) as a, _engine(V, "sc", (32, 8, 8), (1, 1, 1), H, 8) as b:
        for e in (a, b):
            e.init_random()
            e.set_thermostat(4.5)
        a.sweeps(10, measure=False)
        b.sweeps(4, measure=False)
        s = b.get_state()
        b.set_state(s)
        b.sweeps(6, measure=False)
        assert a.sweep_index == b.sweep_index == 10
        assert np.array_equal(a.get_state(), b.get_state())


def test_sweep_index_stays_32_bit(V, O):
    """The sweep index is the 32-bit Philox counter word: the last index a run
    may use is 2^32 - 1 and runs that would pass it are refused (the state
    and the index stay as they were)."""
    H = V.hamiltonian(V.Exchange(1.0))
    with _engine(V, "sc", (32, 8, 8), (1, 1, 1), H, 8) as eng:
        eng.init_random()
        eng.set_thermostat(4.5)
        with pytest.raises(V.VegasGpuError) as e:
            eng.sweep_index = 1 << 32
        assert e.value.status == 1
        last = (1 << 32) - 2
        eng.sweep_index = last
        s0 = eng.get_state()
        with pytest.raises(V.VegasGpuError) as e:
            eng.sweeps(3)
        assert e.value.status == 1 and "2^32" in str(e.value)
        assert eng.sweep_index == last and np.array_equal(eng.get_state(), s0)
        eng.sweeps(2, measure=False)  # sweeps 2^32 - 2 and 2^32 - 1
        g = O.Graph(O.lattice("sc", 32, 8, 8))
        ref, _ = g.ising_sweeps(s0, 1.0, 0.0, 4.5, 8, last, 2)
        assert np.array_equal(eng.get_state(), ref)
        assert eng.sweep_index == 1 << 32
        with pytest.raises(V.VegasGpuError):
            eng.sweeps(1)


def test_set_get_roundtrip_and_observables(V, O):
    lat = ("sc", (32, 6, 4), (1, 1, 1))
    rng = np.random.default_rng(1)
    s = rng.choice(np.array([-1, 1], dtype=np.int8), size=32 * 6 * 4)
    H = V.hamiltonian(V.Exchange(1.0), V.Zeeman(), V.Gauge(0.25))
    with _engine(V, *lat, H, 3) as eng:
        eng.set_state(s)
        assert np.array_equal(eng.get_state(), s)
        eng.set_thermostat(2.0, (0, 0, 1), 0.5)
        g = O.Graph(O.lattice(lat[0], *lat[1], lat[2]))
        Href = O.Hamiltonian(has_exchange=1, J=1.0, has_zeeman=1, zeeman_sign=1.0, has_gauge=1, gauge=0.25,
                             compound=1)
        e_ref = g.ref_total_energy(0, s, Href, b=(0, 0, 1), bmag=0.5)
        assert eng.total_energy() == pytest.approx(e_ref, abs=1e-9)
        m, mag = eng.magnetization()
        assert mag == abs(int(s.sum())) and m[2] == int(s.sum())


def test_low_and_high_temperature_limits(V):
    H = V.hamiltonian(V.Exchange(1.0))
    with _engine(V, "sc", (32, 16, 16), (1, 1, 1), H, 2) as eng:
        eng.set_state(np.ones(32 * 16 * 16, dtype=np.int8))
        eng.set_thermostat(0.0)  # clamped to f64::EPSILON: nothing can flip upward in energy
        E, M = eng.sweeps(3)
        assert np.all(E == -3 * 32 * 16 * 16) and np.all(M == 32 * 16 * 16)
        # (at T -> infinity every proposal is accepted and checkerboard passes
        # flip whole sublattices deterministically, as the oracle does too; a
        # large finite T disorders the lattice)
        eng.set_thermostat(50.0)
        E, M = eng.sweeps(300)
        n = 32 * 16 * 16
        assert abs(E[100:].mean()) < 0.1 * 3 * n and M[100:].mean() < 0.1 * n


def test_invalid_spins_rejected(V):
    H = V.hamiltonian(V.Exchange(1.0))
    with _engine(V, "sc", (32, 4, 4), (1, 1, 1), H, 2) as eng:
        bad = np.ones(512, dtype=np.int8)
        bad[7] = 0
        with pytest.raises(V.VegasGpuError) as e:
            eng.set_state(bad)
        assert e.value.status == 1
        with pytest.raises(V.VegasGpuError):
            eng.set_state(np.ones(100, dtype=np.int8))
        with pytest.raises(V.VegasGpuError):
            eng.set_thermostat(float("nan"))
        eng.set_thermostat(2.0)
        eng.sweeps(1)  # the context stays usable after rejected calls


def test_acceptance_counts(V):
    H = V.hamiltonian(V.Exchange(1.0))
    with _engine(V, "sc", (32, 8, 8), (1, 1, 1), H, 4) as eng:
        eng.init_random()
        eng.set_thermostat(1e9)
        sums = eng.sweeps_sums(5)
        n = 32 * 8 * 8
        # at T -> infinity every flip with dE > 0 is accepted with probability ~1
        assert np.all(sums[:, 7] > 0.99 * n)


def test_device_memory_cap_reports_oom(V):
    """Out-of-memory is reported as a status, without exhausting the device."""
    H = V.hamiltonian(V.Exchange(1.0))
    with pytest.raises(V.VegasGpuError) as e:
        V.Engine(V.Lattice.sc(256, 256, 256), H, max_device_bytes=1 << 20)
    assert e.value.status == 4  # VG_ERR_OOM
    with _engine(V, "sc", (64, 16, 16), (1, 1, 1), H, 1, max_device_bytes=1 << 26) as eng:
        eng.init_random()
        eng.sweeps(2)  # within the cap the context works


@pytest.mark.parametrize("ext,pbc,proposal", [((128, 8, 10), (1, 1, 1), 0), ((128, 8, 10), (1, 1, 1), 1),
                                              ((256, 64, 1), (1, 1, 0), 0)])
def test_one_call_equals_single_sweep_calls(V, ext, pbc, proposal):
    """70 sweeps in one call (two reduction chunks) give the state and the
    per-sweep sums of 70 one-sweep calls."""
    H = V.hamiltonian(V.Exchange(1.0), V.Zeeman())
    out = []
    for split in (False, True):
        with _engine(V, "sc", ext, pbc, H, 99, path=V.PATH_STRUCTURED, proposal=proposal) as eng:
            eng.init_random()
            eng.set_thermostat(3.1, (0, 0, 1), 0.2)
            if split:
                sums = np.concatenate([eng.sweeps_sums(1) for _ in range(70)])
            else:
                sums = eng.sweeps_sums(70)   # one chunk of 64 sweeps and one of 6
            out.append((eng.get_state(), sums))
    assert np.array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])


TILED = [  # extents (all periodic), proposal, sweeps (odd counts end with one two-pass sweep)
    ((64, 4, 4), 0, 6),       # tile boxes wrap onto themselves in y and z
    ((64, 8, 6), 1, 5),
    ((192, 18, 6), 0, 7),     # 6 groups (3 pairs) per row
    ((128, 10, 12), 1, 4),
    ((1024, 40, 36), 0, 3),   # 512-byte rows: several tiles per SM (more than one wave)
]


@pytest.mark.parametrize("ext,proposal,n", TILED)
def test_tiled_sweeps_bit_exact(V, O, ext, proposal, n):
    """One launch per sweep over shared-memory tiles with halos: the same
    spins and per-sweep sums as the colour-order oracle and as the two-pass
    checkerboard kernels, with a field Down and both proposals."""
    seed, J, T, mag = 4321, 1.0, 3.7, 0.3
    H = V.hamiltonian(V.Exchange(J), V.Zeeman())
    out = {}
    for path in (V.PATH_TILED, V.PATH_STRUCTURED):
        with _engine(V, "sc", ext, (1, 1, 1), H, seed, path=path, proposal=proposal) as eng:
            assert eng.info().path == path
            eng.init_random()
            s0 = eng.get_state()
            eng.set_thermostat(T, (0.0, 0.0, -1.0), mag)
            sums = eng.sweeps_sums(n)
            E, M = eng.sweeps(2)
            out[path] = (eng.get_state(), sums, E, M, eng.sweep_index)
    a, b = out[V.PATH_TILED], out[V.PATH_STRUCTURED]
    assert np.array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])
    np.testing.assert_array_equal(a[2], b[2])
    np.testing.assert_array_equal(a[3], b[3])
    assert a[4] == b[4] == n + 2
    g = O.Graph(O.lattice("sc", *ext))
    ref, obs = g.ising_sweeps(s0, J, -mag, T, seed, 0, n + 2, proposal=proposal)
    assert np.array_equal(a[0], ref)
    np.testing.assert_array_equal(a[1][:, 0], obs[:n, 0].astype(float))
    np.testing.assert_array_equal(a[1][:, 6], obs[:n, 1].astype(float))


def test_tiled_path_selection(V):
    H = V.hamiltonian(V.Exchange(1.0))
    with _engine(V, "sc", (256, 128, 128), (1, 1, 1), H, 1) as eng:
        assert eng.info().path == V.PATH_STRUCTURED  # AUTO keeps the two-pass kernels
    with _engine(V, "sc", (256, 128, 128), (1, 1, 1), H, 1, path=V.PATH_TILED) as eng:
        assert eng.info().path == V.PATH_TILED
    for ext, pbc in (((64, 8, 6), (1, 1, 0)), ((32, 8, 8), (1, 1, 1)), ((96, 8, 8), (1, 1, 1)),
                     ((64, 2, 8), (1, 1, 1))):
        with pytest.raises(V.VegasGpuError) as e:
            _engine(V, "sc", ext, pbc, H, 1, path=V.PATH_TILED)
        assert e.value.status == 5


# Generic path with a grid narrower than the class (152 blocks of 64 threads
# = 9,728 threads per pass): the kernel takes 4 entries per thread at a time
# (2 with twelve neighbours), the last batch of each thread partly past the
# class's end.
BATCHED = [
    ("sc", (33, 24, 30), (1, 1, 1)),   # odd x: greedy colouring, classes ~11.9 k (1.2 batches)
    ("bcc", (9, 30, 30), (1, 0, 1)),   # classes 8.1 k, fewer than the threads: one entry each
    ("bcc", (9, 60, 60), (1, 1, 1)),   # classes 32.4 k: 3.3 batches
    ("fcc", (9, 40, 40), (1, 1, 0)),   # twelve neighbours, classes ~14.4 k
]


@pytest.mark.parametrize("cell,ext,pbc", BATCHED)
@pytest.mark.parametrize("proposal", [0, 1])
def test_generic_entry_batches_bit_exact(V, O, cell, ext, pbc, proposal):
    seed, J, T, mag, n = 2024, 1.0, 3.7, 0.2, 4
    H = V.hamiltonian(V.Exchange(J), V.Zeeman()) if proposal else V.hamiltonian(V.Exchange(J))
    with _engine(V, cell, ext, pbc, H, seed, proposal=proposal, path=V.PATH_GENERIC, threads_per_block=64,
                 blocks_per_sm=1) as eng:
        assert eng.info().path == V.PATH_GENERIC
        g = O.Graph(O.lattice(cell, *ext, pbc))
        eng.init_random()
        s0 = eng.get_state()
        assert np.array_equal(s0, g.ising_init(seed))
        if proposal:
            eng.set_thermostat(T, (0, 0, 1), mag)
            sums = eng.sweeps_sums(n)
            ref, obs = g.ising_sweeps(s0, J, mag, T, seed, 0, n, proposal=1)
        else:
            eng.set_thermostat(T)
            sums = eng.sweeps_sums(n)
            ref, obs = g.ising_sweeps(s0, J, 0.0, T, seed, 0, n)
        assert np.array_equal(eng.get_state(), ref)
        np.testing.assert_array_equal(sums[:, 0], obs[:, 0])
        np.testing.assert_array_equal(sums[:, 6], obs[:, 1])


# Periodic axes of extent 1 (bcc / fcc) and 2: the neighbour lists repeat a
# site (a bcc cell's eight neighbours are one site), odd rings and doubled
# bonds give greedy colourings of three or four classes.
TINY = [
    ("sc", (2, 2, 2), (1, 1, 1)),
    ("sc", (3, 2, 1), (1, 1, 0)),
    ("sc", (2, 3, 4), (1, 1, 1)),
    ("bcc", (1, 1, 1), (1, 1, 1)),
    ("bcc", (2, 1, 3), (1, 1, 1)),
    ("fcc", (1, 1, 1), (1, 1, 1)),
    ("fcc", (1, 2, 1), (1, 0, 1)),
]


@pytest.mark.parametrize("cell,ext,pbc", TINY)
@pytest.mark.parametrize("proposal", [0, 1])
def test_tiny_periodic_lattices_bit_exact(V, O, cell, ext, pbc, proposal):
    seed, J, T, mag, n = 314, 1.0, 2.5, 0.4, 8
    H = V.hamiltonian(V.Exchange(J), V.Zeeman()) if proposal else V.hamiltonian(V.Exchange(J))
    with _engine(V, cell, ext, pbc, H, seed, proposal=proposal) as eng:
        g = O.Graph(O.lattice(cell, *ext, pbc))
        eng.init_random()
        s0 = eng.get_state()
        assert np.array_equal(s0, g.ising_init(seed))
        if proposal:
            eng.set_thermostat(T, (0, 0, -1), mag)
            sums = eng.sweeps_sums(n)
            ref, obs = g.ising_sweeps(s0, J, -mag, T, seed, 0, n, proposal=1)
        else:
            eng.set_thermostat(T)
            sums = eng.sweeps_sums(n)
            ref, obs = g.ising_sweeps(s0, J, 0.0, T, seed, 0, n)
        assert np.array_equal(eng.get_state(), ref)
        np.testing.assert_array_equal(sums[:, 0], obs[:, 0])
        np.testing.assert_array_equal(sums[:, 6], obs[:, 1])


def test_largest_power_of_two_sc_lattice(V):
    """sc 1024^3: 2^30 int8 spins, 2^29 bytes per checkerboard class (the
    class offsets are 32-bit).  The sums the passes accumulate over two
    measured sweeps equal a recount of the final state on the device."""
    lat = V.Lattice.sc(1024, 1024, 1024)
    with V.Engine(lat, V.hamiltonian(V.Exchange(1.0)), seed=3) as eng:
        assert eng.info().path == V.PATH_STRUCTURED
        eng.init_random()
        eng.set_thermostat(4.5)
        sums = eng.sweeps_sums(2)
        cur = eng.current_sums()
        assert sums[-1, 0] == cur[0] and sums[-1, 6] == cur[6]
        assert abs(cur[6]) < 0.01 * lat.n_sites          # a random start stays unmagnetised
        assert 0.3 * lat.n_sites < sums[-1, 7] < lat.n_sites  # accepted moves of the sweep


def test_lattices_beyond_the_site_limit_are_rejected(V):
    with pytest.raises(V.VegasGpuError, match="2\\^31-1 sites"):
        V.Engine(V.Lattice.sc(2048, 1024, 1024), V.hamiltonian(V.Exchange(1.0)), seed=1)
