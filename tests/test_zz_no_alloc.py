"""vg_ising_sc_sweeps_noalloc: the Ising sweep entry point for callers that cannot
allocate device memory (a host framework owns the memory pool, the stream is being
captured by someone else, or an allocation could stall a real-time loop).

The caller supplies the two checkerboard class arrays and the sums buffer (here
from PyTorch's allocator, standing in for such a host); the library adds no
allocation of its own.  Two calls in a row must reproduce the context API
(vg_sweeps_sums) exactly: the same spins and the same integer lattice sums in
every column (the zeeman column is mz, which the context reports times the
field's orientation).  The shapes cover one thread block per pass with all axes
periodic, an open axis (per-site neighbour counts differ: the scalar threshold
path), a 2D lattice, and a lattice of many blocks per pass whose calls cross
two reductions of 8 sweeps and end in a partial one.  This file is collected
last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [  # nx, ny, nz, pbc, sweeps of the two calls
    ((64, 8, 6), (1, 1, 1), (5, 7)),
    ((64, 8, 6), (1, 1, 0), (5, 7)),       # z open: non-uniform coordination
    ((64, 32, 1), (1, 1, 0), (6, 3)),      # 2D
    ((256, 64, 64), (1, 1, 1), (19, 9)),   # 128 blocks per pass; chunks of 8 + 8 + 3
]


def to_classes(spins, shape):
    nx, ny, nz = shape
    s = (spins.reshape(nz, ny, nx) > 0).astype(np.uint8)
    parity = (np.arange(nx)[None, None, :] + np.arange(ny)[None, :, None] + np.arange(nz)[:, None, None]) & 1
    return [np.ascontiguousarray(s[parity == c]) for c in (0, 1)]


def from_classes(c0, c1, shape):
    nx, ny, nz = shape
    parity = (np.arange(nx)[None, None, :] + np.arange(ny)[None, :, None] + np.arange(nz)[:, None, None]) & 1
    s = np.empty((nz, ny, nx), dtype=np.int8)
    s[parity == 0] = np.where(c0 > 0, 1, -1)
    s[parity == 1] = np.where(c1 > 0, 1, -1)
    return s.reshape(-1)


@pytest.mark.parametrize("shape,pbc,calls", SHAPES)
def test_noalloc_matches_context_api_on_two_calls(V, shape, pbc, calls):
    torch = pytest.importorskip("torch")
    L = V.lib()
    lat = V.Lattice.sc(*shape, pbc=tuple(bool(p) for p in pbc))
    desc = lat.desc()
    seed = 11
    H = V.hamiltonian(V.Exchange(1.0), V.Zeeman())
    with V.Engine(lat, H, spin=V.SPIN_ISING, seed=seed, path=V.PATH_STRUCTURED) as eng:
        assert eng.info().path == V.PATH_STRUCTURED
        eng.init_random()
        s0 = eng.get_state()
        c0, c1 = (torch.from_numpy(c).cuda() for c in to_classes(s0, shape))
        stream = torch.cuda.current_stream().cuda_stream
        sweep0 = 0
        # call 1: no field; call 2: field Down with |B| = 0.3 (per-site Zeeman -0.3)
        for (T, b, mag), n in zip(((4.0, (0, 0, 1), 0.0), (3.0, (0, 0, -1), 0.3)), calls):
            out = torch.full((n * 8,), float("nan"), dtype=torch.float64, device="cuda")
            orient = 1.0 if b[2] >= 0 else -1.0
            hz = 1.0 * mag * orient
            rc = L.vg_ising_sc_sweeps_noalloc(C.byref(desc), 1.0, hz, T, seed, 0, sweep0, n, c0.data_ptr(),
                                              c1.data_ptr(), out.data_ptr(), C.c_void_p(stream))
            assert rc == 0, L.vg_last_error(None)
            torch.cuda.synchronize()
            eng.set_thermostat(T, b, mag)
            ref = eng.sweeps_sums(n)
            sweep0 += n
            got = out.cpu().numpy().reshape(n, 8)
            assert np.array_equal(from_classes(c0.cpu().numpy(), c1.cpu().numpy(), shape), eng.get_state())
            want = ref.copy()
            want[:, 2] *= orient  # the context's zeeman member carries the field orientation
            np.testing.assert_array_equal(got, want)


def test_noalloc_rejects_lattices_it_cannot_run(V):
    L = V.lib()
    desc = V.Lattice.sc(16, 4, 4).desc()
    rc = L.vg_ising_sc_sweeps_noalloc(C.byref(desc), 1.0, 0.0, 2.0, 1, 0, 0, 1, C.c_void_p(1), C.c_void_p(1), None,
                                      None)
    assert rc == 5 and b"multiple of 32" in L.vg_last_error(None)
    desc = V.Lattice.sc(64, 8, 6).desc()
    rc = L.vg_ising_sc_sweeps_noalloc(C.byref(desc), 1.0, 0.0, 2.0, 1, 0, (1 << 32) - 2, 3, C.c_void_p(1),
                                      C.c_void_p(1), None, None)
    assert rc == 1 and b"2^32" in L.vg_last_error(None)
