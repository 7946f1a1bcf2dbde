"""The C++ host mirror (Machine, programs, instruments, TOML input, CLI) over the C ABI."""
import os
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BIN = os.path.join(REPO, "vegas-rs_gb300", "_build", "bin")


def _bin(name):
    path = os.path.join(BIN, name)
    if not os.path.exists(path):
        import build_ext

        build_ext.build()
    return path


def test_host_selftest_cpu():
    r = subprocess.run([_bin("host_selftest"), "--cpu"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert "checks passed" in r.stdout


def test_cli_prints_default_input_and_fails_loudly_without_args():
    r = subprocess.run([_bin("vegas_gpu_cli"), "input"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "[[stages]]" in r.stdout and 'program = "CoolDown"' in r.stdout
    r = subprocess.run([_bin("vegas_gpu_cli"), "run", "/nonexistent.toml"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and r.stderr.startswith("Error:")


def test_parquet_writer_is_read_by_arrow(tmp_path):
    """The host's Parquet files (the reference's ObservableParquetOutput
    schema, src/output.rs:37-46) read back with an independent reader."""
    pq = pytest.importorskip("pyarrow.parquet")
    import pyarrow as pa

    r = subprocess.run([_bin("host_selftest"), "--parquet-demo", str(tmp_path)], capture_output=True, text=True,
                       timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr
    assert not (tmp_path / "demo.parquet.tmp").exists()
    f = pq.ParquetFile(str(tmp_path / "demo.parquet"))
    assert f.metadata.num_rows == 2500 and f.metadata.num_row_groups == 3
    # pages compressed with SNAPPY, as the reference writes them (src/output.rs:48)
    for g in range(3):
        for k in range(8):
            assert f.metadata.row_group(g).column(k).compression == "SNAPPY"
    t = f.read()
    assert t.schema.names == ["relax", "stage", "step", "n", "temperature", "field", "energy", "magnetization"]
    assert [t.schema.field(k).type for k in range(8)] == [pa.bool_(), pa.uint64(), pa.uint64(), pa.uint64(),
                                                          pa.float64(), pa.float64(), pa.float64(), pa.float64()]
    assert all(not t.schema.field(k).nullable for k in range(8))
    i = list(range(2500))
    assert t.column("relax").to_pylist() == [k % 3 == 0 for k in i]
    assert t.column("stage").to_pylist() == [k // 100 for k in i]
    assert t.column("step").to_pylist() == [k % 100 for k in i]
    assert t.column("n").to_pylist() == [100] * 2500
    assert t.column("temperature").to_pylist() == [1.0 + k / 1000.0 for k in i]
    assert t.column("energy").to_pylist() == [-k / 7.0 for k in i]
    assert t.column("magnetization").to_pylist() == [k * 1e-3 for k in i]


@pytest.mark.gpu
def test_host_selftest_gpu(tmp_path):
    r = subprocess.run([_bin("host_selftest"), "--gpu", str(tmp_path)], capture_output=True, text=True, timeout=600,
                       cwd=tmp_path)
    assert r.returncode == 0, r.stdout + r.stderr
    try:
        import pyarrow.parquet as pq
    except ImportError:  # the GPU host has no pyarrow: the C++ side checked the file structure
        return
    obs = pq.read_table(str(tmp_path / "host_obs.parquet"))
    assert obs.num_rows == 20 + 7 * 40
    assert obs.column("relax").to_pylist()[:20] == [True] * 20
    assert obs.column("stage").to_pylist()[-1] == 14
    st = pq.read_table(str(tmp_path / "host_state.parquet"))
    assert st.num_rows == 1024 * (3 + 7 * (2 + 5))


@pytest.mark.gpu
def test_cli_run_and_bench(tmp_path):
    toml = tmp_path / "in.toml"
    toml.write_text(
        'model = "Ising"\nalgorithm = "Metropolis"\n[sample.unitcell]\nname = "sc"\n'
        "[sample.size]\nx = 32\ny = 32\nz = 1\n[sample.pbc]\nx = true\ny = true\nz = false\n"
        '[[stages]]\nprogram = "Relax"\nsteps = 100\ntemperature = 4.0\n'
        '[[stages]]\nprogram = "CoolDown"\nmax_temperature = 4.0\nmin_temperature = 0.1\ncool_rate = 0.1\n'
        "relax = 20\nsteps = 100\n"
        f'[output]\nobservables = "{tmp_path}/obs.parquet"\n')
    r = subprocess.run([_bin("vegas_gpu_cli"), "run", str(toml), "-s", "1"], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.strip().splitlines()
    assert len(lines) == 39  # CoolDown(4.0, 0.1, 0.1) visits 39 temperatures
    cols = [list(map(float, ln.split())) for ln in lines]
    assert all(len(c) == 7 for c in cols)
    # energy per spin at the lowest temperature is near the ground state -2 (bond) x 2 (Compound total)
    assert cols[-1][2] / 1024 < -3.9
    assert (tmp_path / "obs.parquet").exists() and not (tmp_path / "obs.parquet.tmp").exists()
    r = subprocess.run([_bin("vegas_gpu_cli"), "bench", "potts", "8"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "unknown model" in r.stderr


@pytest.mark.gpu
def test_cli_run_matches_reference_cpu_statistically(tmp_path, O):
    """`vegas_gpu_cli run` (src/main.rs:61-75: Input::run with the GPU
    integrator, src/input.rs:347-367) against the reference restatement
    ref_cpu at one CoolDown temperature: sc 32x32x1 (PBC x, y), Relax 500 at
    T = 2.5, then CoolDown(2.5, 2.5, 0.1) -- the single temperature 2.5 --
    with 100 relax + 2000 measured sweeps.  16 CLI runs (seeds 1..16) against
    16 ref_cpu chains of the same schedule; the StatSensor line's <E>, C,
    <|M|> and chi (src/instrument.rs:113-126) agree within 3 combined
    standard errors of the run-to-run means."""
    import numpy as np

    toml = tmp_path / "in.toml"
    toml.write_text(
        'model = "Ising"\nalgorithm = "Metropolis"\n[sample.unitcell]\nname = "sc"\n'
        "[sample.size]\nx = 32\ny = 32\nz = 1\n[sample.pbc]\nx = true\ny = true\nz = false\n"
        '[[stages]]\nprogram = "Relax"\nsteps = 500\ntemperature = 2.5\n'
        '[[stages]]\nprogram = "CoolDown"\nmax_temperature = 2.5\nmin_temperature = 2.5\ncool_rate = 0.1\n'
        "relax = 100\nsteps = 2000\n")
    runs = 16
    gpu = []
    for s in range(1, runs + 1):
        r = subprocess.run([_bin("vegas_gpu_cli"), "run", str(toml), "-s", str(s)], capture_output=True, text=True,
                           timeout=120)
        assert r.returncode == 0, r.stderr
        lines = r.stdout.strip().splitlines()
        assert len(lines) == 1
        gpu.append([float(x) for x in lines[0].split()])
    gpu = np.array(gpu)
    assert np.all(gpu[:, 0] == 2.5)
    N, T = 1024, 2.5
    g = O.Graph(O.lattice("sc", 32, 32, 1, (1, 1, 0)))
    Hr = O.Hamiltonian(has_exchange=1, J=1.0, has_zeeman=1, zeeman_sign=1.0, compound=1)
    cpu = []
    for s in range(runs):
        rng = O.pcg64(500 + s)
        st, _ = g.ref_sweeps(0, g.ising_init(900 + s), Hr, T, 600, rng, measure=False, clone=False)
        _, obs = g.ref_sweeps(0, st, Hr, T, 2000, rng, clone=False)
        E, M = obs[:, 0], obs[:, 1]
        # the StatSensor columns: T, |B|, <E>, Var(E)/(N T^2), <|M|>, Var(|M|)/(N T), U4
        cpu.append([E.mean(), E.var() / (N * T * T), M.mean(), M.var() / (N * T)])
    cpu = np.array(cpu)
    for col, k in ((2, 0), (3, 1), (4, 2), (5, 3)):
        a, b = gpu[:, col], cpu[:, k]
        se = np.hypot(a.std(ddof=1), b.std(ddof=1)) / np.sqrt(runs)
        assert abs(a.mean() - b.mean()) < 3 * se, (col, a.mean(), b.mean(), se)


def test_gpu_produced_observables_file_reads_back():
    """A GPU-produced ObservableSensor file (the CLI on a GB300, made by
    tests/golden/make_cli_observables.py) read with an independent reader:
    the reference's schema (src/output.rs:37-46), SNAPPY pages, one row per
    sweep of the schedule, and energy / magnetization columns equal to the
    per-sweep E and |M| the Python engine produced for the same seed and
    schedule through the same C ABI."""
    pq = pytest.importorskip("pyarrow.parquet")
    import numpy as np

    golden = os.path.join(REPO, "tests", "golden")
    f = pq.ParquetFile(os.path.join(golden, "cli_observables.parquet"))
    ref = np.load(os.path.join(golden, "cli_observables_engine.npz"))
    t = f.read()
    assert t.schema.names == ["relax", "stage", "step", "n", "temperature", "field", "energy", "magnetization"]
    assert all(f.metadata.row_group(0).column(k).compression == "SNAPPY" for k in range(8))
    # Relax 50 at T = 3, then CoolDown(3.0, 2.0, 0.5): 3 x (20 relax + 40 measured)
    assert t.num_rows == 50 + 3 * 60
    assert t.column("relax").to_pylist() == [True] * 50 + ([True] * 20 + [False] * 40) * 3
    assert t.column("stage").to_pylist() == [0] * 50 + sum(([1 + 2 * k] * 20 + [2 + 2 * k] * 40 for k in range(3)), [])
    assert t.column("temperature").to_pylist() == [3.0] * 50 + [3.0] * 60 + [2.5] * 60 + [2.0] * 60
    assert t.column("n").to_pylist() == [1024] * t.num_rows
    np.testing.assert_array_equal(np.array(t.column("energy").to_pylist()), ref["energy"])
    np.testing.assert_array_equal(np.array(t.column("magnetization").to_pylist()), ref["magnetization"])
