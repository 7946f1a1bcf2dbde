"""The C-ABI library loads and exports the header's symbols; host-side utilities (CPU only)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(REPO, "include", "vegas_gpu.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(vg_[a-z_0-9]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(V):
    syms = declared_symbols()
    assert len(syms) >= 30
    lib = V.lib()
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


def test_binding_covers_the_header(V):
    from vegas_gb300 import _abi

    assert set(declared_symbols()) == set(_abi.SIGNATURES)
    assert V.lib().vg_abi_version() == 1


@pytest.mark.parametrize("cell,ext,pbc", [
    ("sc", (4, 4, 4), (1, 1, 1)), ("sc", (32, 32, 1), (1, 1, 0)), ("sc", (5, 3, 2), (0, 1, 1)),
    ("bcc", (3, 4, 2), (1, 1, 1)), ("bcc", (3, 3, 3), (1, 0, 1)), ("fcc", (3, 3, 3), (1, 1, 1)),
    ("fcc", (2, 3, 4), (0, 1, 0))])
def test_lattice_tables_match_oracle(V, O, cell, ext, pbc):
    lat = getattr(V.Lattice, cell)(*ext, pbc=tuple(bool(p) for p in pbc))
    g = O.Graph(O.lattice(cell, *ext, pbc))
    nb = lat.neighbours()
    assert nb.shape == (g.n, g.zmax)
    assert np.array_equal(np.sort(nb, axis=1), np.sort(g.neighbours(), axis=1))
    col, nc = lat.colouring()
    assert nc == g.ncolours and np.array_equal(col, g.colour)


@pytest.mark.parametrize("cell,nb", [("bcc", 2), ("fcc", 4)])
def test_bcc_fcc_colour_classes_are_the_sublattices(V, O, cell, nb):
    """The sublattice kernels take class q = basis sublattice q and class
    entry = cell index; that is the greedy colouring's assignment (and so
    the generic path's draws) for any extents and boundaries, including
    extents 1 and 2 where periodic images repeat a neighbour."""
    rng = np.random.default_rng(11)
    shapes = [(16, 1, 1), (16, 2, 1), (2, 2, 2), (1, 3, 5)] + [tuple(int(v) for v in rng.integers(1, 7, size=3))
                                                               for _ in range(12)]
    for k, ext in enumerate(shapes):
        pbc = tuple(bool((k >> a) & 1) for a in range(3))
        lat = getattr(V.Lattice, cell)(*ext, pbc=pbc)
        col, nc = lat.colouring()
        assert nc == nb, (ext, pbc)
        assert np.array_equal(col, np.arange(lat.n_sites) % nb), (ext, pbc)
        g = O.Graph(O.lattice(cell, *ext, tuple(int(p) for p in pbc)))
        assert np.array_equal(g.colour, col), (ext, pbc)


def _half(cell, b, a):
    """Whether basis site b sits at the half-cell position on axis a."""
    if cell == "bcc":
        return b == 1
    return (b == 1 and a != 2) or (b == 2 and a != 1) or (b == 3 and a != 0)


@pytest.mark.parametrize("cell,nb", [("bcc", 2), ("fcc", 4)])
def test_sublattice_stencil_equals_neighbour_table(O, cell, nb):
    """The sublattice kernels' stencil: the neighbours of basis b on basis q
    are the cells c + sum over the axes where the two basis positions differ
    of {0, d_b} e_a (d_b = +1 if b sits at the half position, else -1),
    wrapped on periodic axes and dropped across open ones; as multisets it
    equals the oracle's neighbour table."""
    rng = np.random.default_rng(5)
    for k in range(10):
        ext = tuple(int(v) for v in rng.integers(1, 6, size=3))
        pbc = tuple((k >> a) & 1 for a in range(3))
        g = O.Graph(O.lattice(cell, *ext, pbc))
        table = g.nbr.reshape(g.n, g.zmax)
        nx, ny, nz = ext
        for i in range(g.n):
            b, c = i % nb, i // nb
            x, y, z = c % nx, (c // nx) % ny, c // (nx * ny)
            got = []
            for q in range(nb):
                if q == b:
                    continue
                axes = [a for a in range(3) if _half(cell, q, a) != _half(cell, b, a)]
                for m in range(1 << len(axes)):
                    pos, ok = [x, y, z], True
                    for t, a in enumerate(axes):
                        if (m >> t) & 1:
                            pos[a] += 1 if _half(cell, b, a) else -1
                            if not 0 <= pos[a] < ext[a]:
                                ok = ok and bool(pbc[a])
                                pos[a] %= ext[a]
                    if ok:
                        got.append(((pos[2] * ny + pos[1]) * nx + pos[0]) * nb + q)
            want = [int(j) for j in table[i] if j >= 0]
            assert sorted(got) == sorted(want), (ext, pbc, i)


def test_periodic_extent_one_is_rejected(V):
    with pytest.raises(V.VegasGpuError) as e:
        V.Lattice.sc(4, 4, 1, pbc=(True, True, True)).neighbours()
    assert e.value.status == 5  # VG_ERR_UNSUPPORTED


def test_status_strings(V):
    L = V.lib()
    assert L.vg_status_string(0) == b"ok"
    assert L.vg_status_string(6) == b"no CUDA device"


def test_hamiltonian_builder_mirrors_macro(V):
    h1 = V.hamiltonian(V.Exchange(1.0))
    assert h1.compound == 0 and h1.has_exchange == 1
    h3 = V.hamiltonian(V.Exchange(1.0), V.UniaxialAnisotropy((0, 0, 1), 0.1), V.Zeeman())
    assert h3.compound == 1 and h3.has_anisotropy and h3.has_zeeman and h3.zeeman_sign == 1.0
    h = V.hamiltonian(V.Gauge(1.0), V.Gauge(2.0))
    assert h.gauge == 3.0 and h.compound == 1


def test_no_cpu_fallback_without_device(V):
    """Without a GPU the engine refuses loudly instead of computing on the CPU."""
    if V.device_count() > 0:
        pytest.skip("a GPU is visible")
    with pytest.raises(V.VegasGpuError) as e:
        V.Engine(V.Lattice.sc(32, 4, 4), V.hamiltonian(V.Exchange(1.0)))
    assert e.value.status == 6  # VG_ERR_NO_DEVICE


def test_invalid_descriptors_rejected_before_device_use(V):
    L = V.lib()
    d = V.Lattice.sc(0, 4, 4).desc()
    h = V.hamiltonian(V.Exchange(1.0))
    out = C.c_void_p()
    assert L.vg_ctx_create(C.byref(d), C.byref(h), 0, 1, C.byref(out)) == 1
    d = V.Lattice.sc(32, 4, 4).desc()
    bad = V.hamiltonian(V.Exchange(1.0), V.Gauge(1.0))
    bad.compound = 0
    assert L.vg_ctx_create(C.byref(d), C.byref(bad), 0, 1, C.byref(out)) == 1
    assert b"exactly one term" in L.vg_last_error(None)
