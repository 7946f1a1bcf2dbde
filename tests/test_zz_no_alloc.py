"""vg_ising_sc_sweeps_noalloc: the Ising sweep entry point for callers that cannot
allocate device memory (a host framework owns the memory pool, the stream is being
captured by someone else, or an allocation could stall a real-time loop).

The caller supplies the two checkerboard class arrays and the sums buffer (here
from PyTorch's allocator, standing in for such a host); the library adds no
allocation of its own.  Two calls in a row must reproduce the context API
(vg_sweeps_sums) exactly: the same spins and the same integer lattice sums.
This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPE = (64, 8, 6)  # nx, ny, nz; periodic


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


def test_noalloc_matches_context_api_on_two_calls(V):
    torch = pytest.importorskip("torch")
    L = V.lib()
    lat = V.Lattice.sc(*SHAPE)
    desc = lat.desc()
    seed = 11
    H = V.hamiltonian(V.Exchange(1.0), V.Zeeman())
    with V.Engine(lat, H, spin=V.SPIN_ISING, seed=seed, path=V.PATH_STRUCTURED) as eng:
        assert eng.info().path == V.PATH_STRUCTURED
        eng.init_random()
        s0 = eng.get_state()
        c0, c1 = (torch.from_numpy(c).cuda() for c in to_classes(s0, SHAPE))
        stream = torch.cuda.current_stream().cuda_stream
        sweep0 = 0
        # call 1: no field; call 2: field Down with |B| = 0.3 (per-site Zeeman -0.3)
        for T, b, mag, n in ((4.0, (0, 0, 1), 0.0, 5), (3.0, (0, 0, -1), 0.3, 7)):
            out = torch.zeros(n * 8, dtype=torch.float64, device="cuda")
            hz = 1.0 * mag * (1.0 if b[2] >= 0 else -1.0)
            rc = L.vg_ising_sc_sweeps_noalloc(C.byref(desc), 1.0, hz, T, seed, 0, sweep0, n, c0.data_ptr(),
                                              c1.data_ptr(), out.data_ptr(), C.c_void_p(stream))
            assert rc == 0, L.vg_last_error(None)
            torch.cuda.synchronize()
            eng.set_thermostat(T, b, mag)
            ref = eng.sweeps_sums(n)
            sweep0 += n
            got = out.cpu().numpy().reshape(n, 8)
            assert np.array_equal(from_classes(c0.cpu().numpy(), c1.cpu().numpy(), SHAPE), eng.get_state())
            np.testing.assert_array_equal(got[:, 0], ref[:, 0])   # bond sums
            np.testing.assert_array_equal(got[:, 6], ref[:, 6])   # magnetisation
            np.testing.assert_array_equal(got[:, 7], ref[:, 7])   # accepted moves


def test_noalloc_rejects_lattices_it_cannot_run(V):
    L = V.lib()
    desc = V.Lattice.sc(16, 4, 4).desc()
    rc = L.vg_ising_sc_sweeps_noalloc(C.byref(desc), 1.0, 0.0, 2.0, 1, 0, 0, 1, C.c_void_p(1), C.c_void_p(1), None,
                                      None)
    assert rc == 5 and b"multiple of 32" in L.vg_last_error(None)
