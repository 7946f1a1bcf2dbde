"""Generates the GPU-produced Parquet fixture of tests/test_host_cpp.py (run on
a machine with a GPU, from the repository root):

    python tests/golden/make_cli_observables.py

1. `vegas_gpu_cli run` of a small Ising input (sc 32x32x1, PBC x, y; Relax 50
   sweeps at T = 3.0, then CoolDown(3.0, 2.0, 0.5) with 20 relax + 40
   measured sweeps per temperature), seed 7, writes the ObservableSensor file
   cli_observables.parquet (the reference's schema, src/output.rs:37-46);
2. the Python engine runs the same schedule from the same seed through the
   same C ABI and saves its per-sweep E and |M| to cli_observables_engine.npz.
The CPU test reads the Parquet file with an independent reader (pyarrow) and
compares its energy and magnetization columns with the engine's values.
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "vegas-rs_gb300"))

import build_ext  # noqa: E402
import vegas_gb300 as V  # noqa: E402

SEED = 7
TOML = ('model = "Ising"\nalgorithm = "Metropolis"\n[sample.unitcell]\nname = "sc"\n'
        "[sample.size]\nx = 32\ny = 32\nz = 1\n[sample.pbc]\nx = true\ny = true\nz = false\n"
        '[[stages]]\nprogram = "Relax"\nsteps = 50\ntemperature = 3.0\n'
        '[[stages]]\nprogram = "CoolDown"\nmax_temperature = 3.0\nmin_temperature = 2.0\ncool_rate = 0.5\n'
        "relax = 20\nsteps = 40\n"
        '[output]\nobservables = "{out}"\n')


def main():
    build_ext.build()
    cli = os.path.join(REPO, "vegas-rs_gb300", "_build", "bin", "vegas_gpu_cli")
    out = os.path.join(HERE, "cli_observables.parquet")
    with tempfile.TemporaryDirectory() as d:
        toml = os.path.join(d, "in.toml")
        with open(toml, "w") as f:
            f.write(TOML.format(out=out))
        r = subprocess.run([cli, "run", toml, "-s", str(SEED)], capture_output=True, text=True)
        if r.returncode != 0:
            raise SystemExit(r.stderr)
    lat = V.Lattice.sc(32, 32, 1, pbc=(True, True, False))
    H = V.hamiltonian(V.Exchange(1.0), V.Zeeman())  # the CLI's Hamiltonian (src/input.rs:271)
    E, M = [], []
    with V.Engine(lat, H, spin=V.SPIN_ISING, seed=SEED) as eng:
        eng.init_random()
        schedule = [(3.0, 50)] + [(T, n) for T in (3.0, 2.5, 2.0) for n in (20, 40)]
        for T, n in schedule:
            eng.set_thermostat(T)
            e, m = eng.sweeps(n)
            E.append(e)
            M.append(m)
    np.savez(os.path.join(HERE, "cli_observables_engine.npz"), energy=np.concatenate(E),
             magnetization=np.concatenate(M), seed=SEED)
    print("wrote", out)


if __name__ == "__main__":
    main()
