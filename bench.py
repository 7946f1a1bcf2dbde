"""Benchmark: attempted spin flips/ns of the GPU Metropolis hot path.

Workload (N=1 line): plain 3D Ising Metropolis on an sc 256x256x256 lattice
(16,777,216 spins, int8 payload, full PBC, J=1, h=0, random +-1 start from a
seed) -- the single-lattice configuration the headline metric is quoted on.
One step = 200 measured sweeps (per-sweep E and |M| reduced on the device,
as the reference's instruments do after every sweep) at the next temperature
of the 21-point ladder 5.5 -> 3.5 (CoolDown(5.5, 3.5, 0.1), replayed with the
reference's FP loop).  Synthetic data: the lattice and its initial state are
generated from a seed; no external dataset exists for this workload.

Timing: CUDA events on the engine's stream around every step; L2 is flushed
(a 256 MiB write) between steps outside the events; the lattice itself
(16.8 MB) is L2-resident within a step.  `value` = total attempted flips /
summed step time (device-resident state); `e2e` = the same metric through the
C ABI with host buffers: host->device copy of the state from pinned memory,
the sweeps, device->host copy of the per-sweep E/|M| and of the final state.

--impl reference times the reference algorithm on the host cores (the C
restatement in oracle/ -- Rust is absent, so the crate cannot be built):
independent random-site Metropolis chains on the same lattice, one per core.

Multi-GPU: the path does not need a collective; --gpus N runs N independent
replicas (one per rank/GPU, torchrun) and reports the aggregate.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

REPO = os.path.dirname(os.path.abspath(__file__))
for p in (os.path.join(REPO, "vegas-rs_gb300"), REPO):
    if p not in sys.path:
        sys.path.insert(0, p)

L = 256
SWEEPS_PER_STEP = 200
SEED = 20261203
BYTES_PER_FLIP = 3.0  # int8 sc checkerboard: (C + 1) x 1 byte, C = 2 colour passes
METRIC = "attempted spin flips/ns on 1 GB300 (batched vs plain GPU path), % HBM roofline"


def ladder():
    out, t = [], 5.5
    while True:  # CoolDown::run (src/program.rs:202-211)
        out.append(t)
        t -= 0.1
        if t < 3.5:
            break
    return out


def aggregate_value(flips_per_rank, world, max_ms):
    """Whole-job flips/ns: every rank runs its own replica (same work per rank),
    timed by the slowest rank."""
    return flips_per_rank * world / (max_ms * 1e6)


def peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def read_profile_traffic(name):
    """Per-launch DRAM bytes of the dominant kernel from its committed ncu summary."""
    path = os.path.join(REPO, "profiles", name)
    try:
        for line in open(path):
            if line.startswith("traffic_bytes_per_launch:"):
                return float(line.split(":", 1)[1].strip())
    except OSError:
        pass
    return None


class Clocks:
    """nvidia-smi sampling (every 20 ms) around the timed region; the summary
    uses the samples taken while it ran (mark_start / mark_stop)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap,timestamp")

    def __init__(self, device_index):
        self.dev = device_index
        self.proc = None
        self.path = None
        self.t0 = self.t1 = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "20"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
            time.sleep(0.5)  # the sampler is running before the timed region starts
        except OSError:
            self.proc = None
        return self

    def mark_start(self):
        self.t0 = time.time()

    def mark_stop(self):
        self.t1 = time.time()

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        import datetime

        rows, inside = [], []
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 10:
                rows.append(parts)
                try:
                    ts = datetime.datetime.strptime(parts[9], "%Y/%m/%d %H:%M:%S.%f").timestamp()
                except ValueError:
                    ts = None
                if ts is not None and self.t0 is not None and self.t0 - 0.05 <= ts <= self.t1 + 0.05:
                    inside.append(parts)
        os.unlink(self.path)
        if inside:
            rows = inside
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        load = [s for s in sm if s > 0.5 * max(sm)] if sm else []
        return {"sm_mhz": statistics.median(load) if load else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows), "window": "timed region" if inside else "whole run"}


def cpu_baseline_sample(threads=1, sweeps=2):
    """ref_cpu (C restatement of the reference's Metropolis) on the same 256^3 lattice."""
    import oracle as O

    H = O.Hamiltonian(has_exchange=1, J=1.0, compound=0)
    lat = O.lattice("sc", L, L, L)
    flips, dt = O.ref_parallel(lat, 0, H, 4.5, sweeps, threads, seed=SEED, measure=True)
    return flips / (dt * 1e9), dt


def run_reference(args, rank):
    """--impl reference: the reference algorithm on all host cores."""
    if rank != 0:
        return
    import oracle as O

    oracle_lib = O.lib()
    del oracle_lib
    threads = os.cpu_count() or 1
    H = O.Hamiltonian(has_exchange=1, J=1.0, compound=0)
    lat = O.lattice("sc", L, L, L)
    # each step is one measured reference sweep of a 256^3 lattice on every
    # host core (about five seconds) at the temperature the GPU arm's step of
    # the same index runs: the CoolDown(5.5, 3.5, 0.1) ladder, one
    # temperature per step, the chains carrying their state along it; the
    # warm-up sweeps run untimed first
    steps = max(1, args.steps)
    warm = max(0, args.warmup)
    temps = ladder()
    sched = [temps[(warm + k) % len(temps)] for k in range(steps)]
    flips, dt = O.ref_parallel_ladder(lat, 0, H, sched, 1, threads, seed=SEED, measure=True, warmup=warm)
    v = flips / (dt * 1e9)
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "flips/ns", "n_gpus": args.gpus,
        "steps": steps, "warmup": warm, "ms_per_step": dt * 1e3 / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "ising-sc-256^3-pbc-J1-h0 (reference random-site Metropolis, CLI measurement)",
                   "lattice": [L, L, L], "threads": threads,
                   "temperatures": "CoolDown(5.5, 3.5, 0.1) ladder, one per step (the GPU arm's steps)",
                   "step_temperatures": sched},
        "cpu_baseline": {"value": v, "unit": "flips/ns", "cores": threads, "kind": "port",
                         "sample": f"{steps} measured sweeps per core, one 256^3 lattice per core"},
        "e2e": {"value": v, "unit": "flips/ns", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "gpu_launches": 0,
    }
    print(json.dumps(line), flush=True)


def run_tiled(V, torch, args, n_l, flush):
    """The same workload on the one-launch-per-sweep kernel (both colour
    passes on shared-memory tiles with halos, staged by bulk asynchronous
    copies), timed with the same step protocol for comparison; its launch
    is a whole sweep, 3 N algorithmic bytes."""
    N = n_l ** 3
    temps = ladder()
    with V.Engine(V.Lattice.sc(n_l, n_l, n_l), V.hamiltonian(V.Exchange(1.0)), spin=V.SPIN_ISING, seed=SEED,
                  path=V.PATH_TILED) as eng:
        eng.init_random()
        s = torch.cuda.ExternalStream(eng.stream())
        for k in range(3):
            eng.set_thermostat(temps[k])
            eng.sweeps_async(SWEEPS_PER_STEP, measure=True)
        eng.synchronize()
        steps = 5
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        for k, (a, c) in enumerate(ev):
            with torch.cuda.stream(s):
                flush.fill_(1.0)
            eng.set_thermostat(temps[(3 + k) % len(temps)])
            a.record(s)
            eng.sweeps_async(SWEEPS_PER_STEP, measure=True)
            c.record(s)
        eng.synchronize()
        ms = sum(a.elapsed_time(c) for a, c in ev)
        launch_ms, _ = eng.time_passes(50, measure=True)
    v = float(N) * SWEEPS_PER_STEP * steps / (ms * 1e6)
    peak, _ = peaks()
    return {"value": v, "unit": "flips/ns", "steps": steps,
            "kernel": "ising_tile_sweep_kernel (one launch per sweep)", "roofline_frac": v * BYTES_PER_FLIP / peak,
            "launch_ms": ms / (steps * SWEEPS_PER_STEP), "launch_ms_isolated_events": launch_ms,
            "traffic": read_profile_traffic("ising_tile_sweep_256cubed.md")}


def run_batched(V, torch, args):
    """The batched form: 256 replicas in four size groups, multi-spin coded 32 per
    word, replica exchange every 10 sweeps, each round one CUDA graph launch."""
    import numpy as np

    t2 = np.geomspace(2.0, 2.6, 64)
    t3 = np.geomspace(4.2, 4.8, 64)
    groups = [(V.Lattice.sc(64, 64, 1, pbc=(True, True, False)), t2),
              (V.Lattice.sc(512, 512, 1, pbc=(True, True, False)), t2),
              (V.Lattice.sc(32, 32, 32), t3), (V.Lattice.sc(128, 128, 128), t3)]
    rounds = 20  # 200 sweeps per step, as the plain path
    with V.Batch(groups, J=1.0, seed=SEED, sweeps_per_round=10, exchange=True) as b:
        b.init_random()
        shape, tune_ms = b.autotune(rounds=3)  # times every launch shape, restores the state
        for _ in range(max(args.warmup, 1)):
            b.run(rounds)
        s = torch.cuda.ExternalStream(b.stream())
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        for a, c in ev:
            a.record(s)
            b.run_async(rounds)
            c.record(s)
        b.synchronize()
        ms = sum(a.elapsed_time(c) for a, c in ev)
        info = b.info()
        flips = float(info.replica_sites) * 10 * rounds * args.steps
        acc, att = b.swap_stats(3)
    cpu = None
    if not args.no_cpu_baseline:
        import oracle as O

        cores = os.cpu_count() or 1
        fl, dt = O.ref_parallel(O.lattice("sc", 128, 128, 128), 0, O.Hamiltonian(has_exchange=1, J=1.0, compound=0),
                                4.5, 1, cores, seed=SEED, measure=True)
        cpu = {"value": fl / (dt * 1e9), "unit": "flips/ns", "cores": cores, "kind": "port",
               "sample": f"one measured reference sweep of an independent 128^3 replica on each of {cores} cores"}
    return {"value": flips / (ms * 1e6), "unit": "flips/ns", "ms_per_step": ms / args.steps, "cpu_baseline": cpu,
            "replicas": int(info.total_replicas), "replica_sites": int(info.replica_sites),
            "sweeps_per_step": 10 * rounds, "graph": bool(info.graph),
            "workload": "256 replicas: 64 x 2D 64^2, 64 x 2D 512^2 (T 2.0-2.6), 64 x 3D 32^3, 64 x 3D 128^3 "
                        "(T 4.2-4.8), geometric ladders, multi-spin coded 32 per word, exchange every 10 sweeps",
            "bytes_per_flip": 0.375,
            "tuning": {"threads_per_block": shape[0], "words_per_thread": shape[1], "words_in_flight": shape[2],
                       "ms_per_round_when_tuned": tune_ms},
            "swap_acceptance_3d128": float(acc[:-1].sum() / max(att[:-1].sum(), 1))}


def run_cooldown_2d(V, torch, args):
    """The reference's own CPU-sized case: sc 32x32x1 (PBC x, y; open z),
    J=1, random start, Relax 1000 sweeps at T=4 then CoolDown(4.0, 0.1, 0.1)
    with 1000 relax + 20000 measured sweeps per temperature (39 temperatures
    by the reference's loop).  Timed on a bounded sample: the relax and the
    first 5 temperatures (106,000 sweeps), on the resident kernel (all sweeps
    of a call in one launch); the reference restatement runs 20,000 measured
    sweeps of the same lattice on one host core beside it."""
    import oracle as O

    lat = V.Lattice.sc(32, 32, 1, pbc=(True, True, False))
    H = V.hamiltonian(V.Exchange(1.0))
    temps, t = [], 4.0
    while True:  # CoolDown::run (src/program.rs:202-211)
        temps.append(t)
        t -= 0.1
        if t < 0.1:
            break
    k = 5
    with V.Engine(lat, H, spin=V.SPIN_ISING, seed=1) as eng:
        eng.init_random()
        path = eng.info().path
        s = torch.cuda.ExternalStream(eng.stream())
        a, c = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        eng.set_thermostat(4.0)
        eng.sweeps(100)  # warm-up
        a.record(s)
        eng.set_thermostat(4.0)
        eng.sweeps_async(1000, measure=False)
        for T in temps[:k]:
            eng.set_thermostat(T)
            eng.sweeps_async(1000, measure=False)
            eng.sweeps_async(20000, measure=True)
        c.record(s)
        eng.synchronize()
        ms = a.elapsed_time(c)
    sweeps = 1000 + k * 21000
    full = 1000 + len(temps) * 21000
    n = lat.n_sites
    cpu = None
    if not args.no_cpu_baseline:
        olat = O.lattice("sc", 32, 32, 1, (1, 1, 0))
        flips, dt = O.ref_parallel(olat, 0, O.Hamiltonian(has_exchange=1, J=1.0, compound=0), 2.0, 20000, 1,
                                   seed=1, measure=True)
        cpu = {"value": flips / (dt * 1e9), "unit": "flips/ns", "cores": 1, "kind": "port",
               "sample": "20,000 measured reference sweeps of the 32x32x1 lattice at T=2.0 on one core"}
    return {"workload": "sc 32x32x1 (open z) Ising, Relax 1000 @ T=4 + CoolDown(4.0, 0.1, 0.1) x (1000 + 20000)",
            "value": n * sweeps / (ms * 1e6), "unit": "flips/ns", "sample_sweeps": sweeps,
            "sample_ms": ms, "full_schedule_s_projected": ms * full / sweeps / 1e3, "temperatures": len(temps),
            "path": {1: "generic", 2: "structured", 3: "resident"}.get(path, "?"), "cpu_baseline": cpu}


def run_sublattice(V, torch, args):
    """bcc 128^3 cells (4,194,304 sites), full PBC, J=1: Ising (T = 3.0,
    flip proposals) and Heisenberg (K = 0.1 along z, B = 0.05 along z, T = 1.0,
    sphere proposals, FP32) through the sublattice kernels, each beside the
    same sweeps on the neighbour-table (ELL) kernels; 20 measured sweeps per
    timing, after 5 warm-up sweeps."""
    out = {}
    cases = (("ising", V.SPIN_ISING, V.hamiltonian(V.Exchange(1.0)), 3.0),
             ("heisenberg", V.SPIN_HEISENBERG,
              V.hamiltonian(V.Exchange(1.0), V.UniaxialAnisotropy((0, 0, 1), 0.1), V.Zeeman()), 1.0))
    lat = V.Lattice.bcc(128, 128, 128)
    n = 20
    for name, spin, H, T in cases:
        row = {}
        for key, path in (("sublattice", V.PATH_STRUCTURED), ("ell", V.PATH_GENERIC)):
            with V.Engine(lat, H, spin=spin, seed=SEED, path=path,
                          proposal=V.PROPOSE_RANDOM if spin == V.SPIN_HEISENBERG else V.PROPOSE_FLIP) as eng:
                eng.init_random()
                eng.set_thermostat(T, (0, 0, 1), 0.05 if spin == V.SPIN_HEISENBERG else 0.0)
                eng.sweeps(5)
                s = torch.cuda.ExternalStream(eng.stream())
                a, c = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(s)
                eng.sweeps_async(n, measure=True)
                c.record(s)
                eng.synchronize()
                row[key] = lat.n_sites * n / (a.elapsed_time(c) * 1e6)
        out[name] = {"value": row["sublattice"], "ell_value": row["ell"], "unit": "flips/ns",
                     "kernel": "ising_sub_kernel" if spin == V.SPIN_ISING else "heis_sub_kernel"}
    return {"workload": "bcc 128^3 cells (4,194,304 sites) PBC J=1, Ising T=3.0 and Heisenberg T=1.0 K=0.1 B=0.05, "
                        "20 measured sweeps, sublattice kernels beside the neighbour-table kernels",
            **out}


def run_wolff(V, torch, args):
    """docs/wolff.toml's workload shape: sc 10x10x10 Ising, Wolff cluster
    steps; a bounded sample of 20,000 steps at T = 4.5 (near the critical
    point, where clusters are largest in spread) on the single-block kernel,
    beside the same steps of the oracle's cluster algorithm on one core; and
    sc 64^3 and 128^3 near T_c on the bit-packed one-block and the
    multi-block kernels."""
    import oracle as O

    lat = V.Lattice.sc(10, 10, 10)
    n = 20000
    with V.Engine(lat, V.hamiltonian(V.Exchange(1.0)), seed=SEED) as eng:
        eng.init_random()
        eng.set_thermostat(4.5)
        eng.wolff_steps(2000)
        s = torch.cuda.ExternalStream(eng.stream())
        a, c = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(s)
        lib = V.lib()
        import ctypes as C

        V._check(lib.vg_wolff_steps(eng._h, C.c_uint64(n), 0, None, None), eng._h)
        c.record(s)
        eng.synchronize()
        ms = a.elapsed_time(c)
        state = eng.get_state()
    cpu = None
    if not args.no_cpu_baseline:
        g = O.Graph(O.lattice("sc", 10, 10, 10))
        t0 = time.perf_counter()
        _, obs = g.wolff_steps(state, 1.0, 4.5, SEED, 0, n)
        dt = time.perf_counter() - t0
        cpu = {"value": n / dt, "unit": "cluster steps/s", "cores": 1, "kind": "port",
               "sample": f"{n} cluster steps of the oracle's Wolff algorithm at T = 4.5 on one core",
               "mean_cluster": float(obs[:, 2].mean())}
    # larger lattices near T_c: 64^3 (spins and marks as bits in one block)
    # and 128^3 (the multi-block kernel), equilibrated first
    larger = {}
    for L, kind in ((64, "one-block bit-packed kernel"), (128, "multi-block kernel")):
        ng = 300
        with V.Engine(V.Lattice.sc(L, L, L), V.hamiltonian(V.Exchange(1.0)), seed=SEED) as eng:
            eng.init_random()
            eng.set_thermostat(4.5)
            eng.sweeps(300, measure=False)
            eng.wolff_steps(300, measure=False)
            state_g = eng.get_state()
            step0 = eng.info().sweep_index
            s = torch.cuda.ExternalStream(eng.stream())
            a, c = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(s)
            _, Mg = eng.wolff_steps(ng)
            c.record(s)
            eng.synchronize()
            ms_g = a.elapsed_time(c)
        entry = {"workload": f"sc {L}^3 Ising, Wolff cluster steps at T = 4.5 after 300 Metropolis sweeps and 300 "
                             f"cluster steps ({kind}, measured steps)",
                 "value": ng / (ms_g * 1e-3), "unit": "cluster steps/s", "ms": ms_g, "steps": ng,
                 "mean_abs_m_per_spin": float(Mg.mean() / L ** 3)}
        if not args.no_cpu_baseline:
            g = O.Graph(O.lattice("sc", L, L, L))
            m = 20
            t0 = time.perf_counter()
            _, obs = g.wolff_steps(state_g, 1.0, 4.5, SEED, step0, m)
            dt = time.perf_counter() - t0
            entry["cpu_baseline"] = {"value": m / dt, "unit": "cluster steps/s", "cores": 1, "kind": "port",
                                     "sample": f"{m} cluster steps of the oracle's Wolff algorithm from the same state",
                                     "mean_cluster": float(obs[:, 2].mean())}
        larger[f"sc{L}"] = entry
    return {"workload": "sc 10x10x10 Ising, Wolff cluster steps (docs/wolff.toml lattice), T = 4.5",
            "value": n / (ms * 1e-3), "unit": "cluster steps/s", "ms": ms, "steps": n, "cpu_baseline": cpu,
            "larger": larger}


def run_heisenberg(V, torch, args):
    """Heisenberg sc 128^3, J=1, K=0.1 along z, B=0.05 along z, uniform-on-sphere
    proposals, FP32 updates with FP64 sums; a step is 100 measured sweeps at the
    next temperature of the 0.2-2.0 ladder.  Beside the throughput: the error of
    the device sums (FP32 partials, FP64 combination) against an FP64
    recomputation from the exported state, and an all-FP64 run's throughput."""
    import numpy as np

    n_l, sweeps = 128, 100
    lat = V.Lattice.sc(n_l, n_l, n_l)
    H = V.hamiltonian(V.Exchange(1.0), V.UniaxialAnisotropy((0, 0, 1), 0.1), V.Zeeman())
    temps = [0.2 + 0.1 * k for k in range(19)]
    out = {}
    for prec, steps in ((V.FP32, args.steps), (V.FP64, 1)):
        with V.Engine(lat, H, spin=V.SPIN_HEISENBERG, seed=SEED, precision=prec) as eng:
            eng.init_random()
            eng.set_thermostat(temps[0], (0, 0, 1), 0.05)
            eng.sweeps(sweeps)
            s = torch.cuda.ExternalStream(eng.stream())
            ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
            for k, (a, c) in enumerate(ev):
                eng.set_thermostat(temps[(k + 1) % len(temps)], (0, 0, 1), 0.05)
                a.record(s)
                eng.sweeps_async(sweeps, measure=True)
                c.record(s)
            eng.synchronize()
            ms = sum(a.elapsed_time(c) for a, c in ev)
            pass_ms, _ = eng.time_passes(20, measure=False)
            key = "fp32" if prec == V.FP32 else "fp64"
            # average pass over the timed sweeps (as the headline), and one pass timed alone
            out[key] = {"value": lat.n_sites * sweeps * steps / (ms * 1e6), "pass_ms": ms / (steps * sweeps * 2),
                        "pass_ms_isolated": pass_ms}
            if prec == V.FP32:
                st = eng.get_state().reshape(n_l, n_l, n_l, 3)
                got = eng.current_sums()
                bond = sum(float(np.sum(st * np.roll(st, 1, axis=a))) for a in range(3))
                ref = {"bond": (0, bond), "anisotropy": (1, float(np.sum(st[..., 2] ** 2))),
                       "mz": (6, float(st[..., 2].sum()))}
                out["sum_rel_err"] = {k: abs(float(got[i]) - v) / abs(v) for k, (i, v) in ref.items()}
    alg = 18.0 * lat.n_sites  # per pass: read both classes (12 B each), write one class
    peak, _ = peaks()
    ach = alg / (out["fp32"]["pass_ms"] * 1e-3) / 1e9
    cpu = None
    if not args.no_cpu_baseline:
        import oracle as O

        OH = O.Hamiltonian(has_exchange=1, J=1.0, has_anisotropy=1, K=0.1, has_zeeman=1, zeeman_sign=1.0, compound=1)
        OH.axis[:] = (0.0, 0.0, 1.0)
        flips, dt = O.ref_parallel(O.lattice("sc", n_l, n_l, n_l), 1, OH, 1.0, 2, 1, seed=SEED,
                                   proposal=O.PROPOSE_RANDOM, measure=True, bmag=0.05)
        cpu = {"value": flips / (dt * 1e9), "unit": "flips/ns", "cores": 1, "kind": "port",
               "sample": f"2 measured reference sweeps of the {n_l}^3 Heisenberg lattice on one core"}
    return {"cpu_baseline": cpu,
            "workload": "heisenberg-sc-128^3-pbc J=1 K=0.1 z B=0.05 z, random proposals, FP32 update / FP64 sums",
            "value": out["fp32"]["value"], "unit": "flips/ns", "sweeps_per_step": sweeps,
            "fp64_value": out["fp64"]["value"], "bytes_per_flip": 36.0,
            "roofline": {"achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                         "pass_ms": out["fp32"]["pass_ms"], "pass_ms_isolated": out["fp32"]["pass_ms_isolated"],
                         "kernel": "heis_sc4_kernel (one colour pass, measured sweeps)"},
            "sum_rel_err_vs_fp64_recompute": out["sum_rel_err"]}


def run_hysteresis(V, torch, args):
    """Batched Heisenberg hysteresis: fcc 64^3 cells (1,048,576 spins), 64
    replicas (8 seeds x 8 cubic constants 0-0.1), T=0.5, J=1, field along z
    from +5 to -5 and back in steps of 0.1 (201 points).  Throughput on a
    bounded sample of the schedule (a step = 4 field points x (10 relax + 40
    measured sweeps) of all 64 replicas); loop area and coercive fields of a
    full loop on fcc 8^3 cells in FP32 and FP64 (same seeds)."""
    import numpy as np

    def replicas():
        return [V.HeisReplica(seed=SEED + 7919 * (r // 8), replica=r, temperature=0.5, exchange=1.0,
                              anisotropy=0.0, cubic=0.1 * (r % 8) / 7) for r in range(64)]

    fields = V.hysteresis_fields(5.0, 0.1)
    lat = V.Lattice.fcc(64, 64, 64)
    relax, measure, pts = 10, 40, 4
    with V.HysteresisBatch(lat, replicas(), field_axis=(0, 0, 1), zeeman_sign=-1.0) as hb:
        hb.init_random()
        hb.run(fields[:pts], relax, measure)  # warm-up (graph capture)
        s = torch.cuda.ExternalStream(hb.stream())
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        for k, (a, c) in enumerate(ev):
            a.record(s)
            hb.run_async(fields[(k * pts) % 200:(k * pts) % 200 + pts], relax, measure)
            c.record(s)
        hb.synchronize()
        ms = sum(a.elapsed_time(c) for a, c in ev)
        sweep_ms = hb.time_passes(10)
        info = hb.info()
    n_total = float(lat.n_sites) * 64
    value = n_total * pts * (relax + measure) * args.steps / (ms * 1e6)
    alg = 15.0 * n_total  # per colour pass (4 classes, 12 B payload): read all, write one class
    peak, _ = peaks()
    ach = alg / (sweep_ms / 4 * 1e-3) / 1e9
    # full loop, small lattice, FP32 against FP64
    small = V.Lattice.fcc(8, 8, 8)
    loops = {}
    for prec in (V.FP32, V.FP64):
        with V.HysteresisBatch(small, replicas(), field_axis=(0, 0, 1), zeeman_sign=-1.0, precision=prec) as hb:
            hb.init_random()
            sums = hb.run(fields, 20, 30)
        m = sums[:, :, 6] / (30 * small.n_sites)
        loops[prec] = ([V.loop_area(fields, m[:, r]) for r in range(64)],
                       [V.coercive_fields(fields, m[:, r]) for r in range(64)])
    cpu = None
    if not args.no_cpu_baseline:
        import oracle as O

        cores = os.cpu_count() or 1
        OH = O.Hamiltonian(has_exchange=1, J=1.0, has_zeeman=1, zeeman_sign=-1.0, compound=1)
        fl, dt = O.ref_parallel(O.lattice("fcc", 64, 64, 64), 1, OH, 0.5, 1, cores, seed=SEED,
                                proposal=O.PROPOSE_RANDOM, measure=True, bmag=1.0)
        cpu = {"value": fl / (dt * 1e9), "unit": "flips/ns", "cores": cores, "kind": "port",
               "sample": f"one measured reference sweep of an independent fcc 64^3-cell replica on each of {cores} "
                         "cores (exchange + Zeeman: the reference has no cubic term)"}
    a32, a64 = np.array(loops[V.FP32][0]), np.array(loops[V.FP64][0])
    h32, h64 = np.array(loops[V.FP32][1]), np.array(loops[V.FP64][1])
    return {"workload": "fcc 64^3 cells x 64 replicas (8 seeds x 8 Kc in 0-0.1), T=0.5, B_z +5 -> -5 -> +5 "
                        "step 0.1, FP32 updates, FP64 sums",
            "value": value, "unit": "flips/ns", "ms_per_step": ms / args.steps, "cpu_baseline": cpu,
            "sample": f"{pts} field points x ({relax} relax + {measure} measured sweeps) per step",
            "graph": bool(info.graph), "sites_per_thread": int(info.sites_per_thread), "bytes_per_flip": 60.0,
            "roofline": {"achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                         "sweep_ms": sweep_ms, "kernel": "hb_pass (one colour pass, all replicas)"},
            "loop_fcc8": {"area_fp64_mean": float(a64.mean()), "area_fp32_mean": float(a32.mean()),
                          "area_rel_diff_mean": float(np.mean(np.abs(a32 - a64) / np.abs(a64))),
                          "hc_fp64_mean": [float(np.nanmean(h64[:, 0])), float(np.nanmean(h64[:, 1]))],
                          "hc_abs_diff_mean": float(np.nanmean(np.abs(h32 - h64))),
                          "schedule": "201 points x (20 relax + 30 measured sweeps)"}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--lattice", type=int, default=L)
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-heisenberg", action="store_true")
    args = ap.parse_args()

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        run_reference(args, rank)
        return

    import numpy as np
    import torch

    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))

    import vegas_gb300 as V

    n_l = args.lattice
    lat = V.Lattice.sc(n_l, n_l, n_l)
    H = V.hamiltonian(V.Exchange(1.0))
    eng = V.Engine(lat, H, spin=V.SPIN_ISING, seed=SEED, replica=rank, device=local_rank)
    eng.init_random()
    info = eng.info()
    N = lat.n_sites
    stream = torch.cuda.ExternalStream(eng.stream())
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    temps = ladder()

    def flush_l2():
        with torch.cuda.stream(stream):
            flush.fill_(1.0)

    def step(k):
        eng.set_thermostat(temps[k % len(temps)])
        eng.sweeps_async(SWEEPS_PER_STEP, measure=True)

    for k in range(args.warmup):
        step(k)
    eng.synchronize()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    stops = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    tiled = info.path == V.PATH_TILED
    # one launch per sweep (tiled) or per colour pass, plus the sum reductions
    launches_per_step = SWEEPS_PER_STEP * (1 if tiled else info.n_colours) + (SWEEPS_PER_STEP + 63) // 64
    with Clocks(local_rank) as clk:
        clk.mark_start()
        wall0 = time.perf_counter()
        for k in range(args.steps):
            flush_l2()
            starts[k].record(stream)
            step(args.warmup + k)
            stops[k].record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - wall0
        clk.mark_stop()
    eng.read_sums(SWEEPS_PER_STEP)  # results of the last step reach the host
    step_ms = [a.elapsed_time(b) for a, b in zip(starts, stops)]
    dev_ms = sum(step_ms)
    if dist:
        t = torch.tensor([dev_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dev_ms = float(t.item())
        dist.barrier()
    flips_rank = float(N) * SWEEPS_PER_STEP * args.steps
    value = aggregate_value(flips_rank, world, dev_ms)

    # dominant kernel: one colour pass.  Its average launch duration comes from
    # the timed region (CUDA events on the engine stream around each step; a
    # step is SWEEPS_PER_STEP x n_colours passes plus a few sum reductions,
    # which are charged to the passes); an isolated per-launch timing is
    # reported beside it.
    passes = SWEEPS_PER_STEP * (1 if tiled else info.n_colours) * args.steps
    pass_ms = dev_ms / passes
    iso_pass_ms, sweep_ms = eng.time_passes(50, measure=True)
    # algorithmic bytes: (C + 1) x 1 byte per site and sweep, C = 2 colour
    # passes -- a colour pass reads both classes (N) and writes one (N/2); a
    # tiled launch is one sweep (3 N), whatever its real traffic (the tiles
    # read each class once and write each once, 2 N plus halos)
    alg_bytes_per_launch = (3.0 if tiled else 1.5) * N
    achieved = alg_bytes_per_launch / (pass_ms * 1e-3) / 1e9
    peak, peak_kind = peaks()
    traffic = read_profile_traffic("ising_tile_sweep_256cubed.md" if tiled else "ising_sc_pass_256cubed.md")
    kernel = ("ising_tile_sweep_kernel (one sweep: both colour passes on shared-memory tiles)" if tiled
              else "ising_sc2_kernel (one colour pass)")

    # end to end through the C ABI with host buffers
    import ctypes as C

    hbuf = C.c_void_p()
    V._check(V.lib().vg_host_alloc(C.byref(hbuf), N))
    obuf = C.c_void_p()
    V._check(V.lib().vg_host_alloc(C.byref(obuf), 16 * SWEEPS_PER_STEP))
    host_state = np.ctypeslib.as_array((C.c_int8 * N).from_address(hbuf.value))
    host_state[:] = eng.get_state()
    Eo = (C.c_double * SWEEPS_PER_STEP).from_address(obuf.value)
    Mo = (C.c_double * SWEEPS_PER_STEP).from_address(obuf.value + 8 * SWEEPS_PER_STEP)
    e2e_steps = max(3, min(args.steps, 10))
    lib = V.lib()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(e2e_steps):
        eng.set_thermostat(temps[k % len(temps)])
        V._check(lib.vg_set_state(eng._h, hbuf, C.c_int64(N)), eng._h)
        V._check(lib.vg_sweeps(eng._h, C.c_uint64(SWEEPS_PER_STEP), 1, Eo, Mo), eng._h)
        V._check(lib.vg_get_state(eng._h, hbuf, C.c_int64(N)), eng._h)
    e2e_s = time.perf_counter() - t0
    e2e_value = float(N) * SWEEPS_PER_STEP * e2e_steps * world / (e2e_s * 1e9)
    lib.vg_host_free(hbuf)
    lib.vg_host_free(obuf)

    tiled_cmp = run_tiled(V, torch, args, n_l, flush) if not tiled else None

    batched = None
    if not args.no_batched:
        batched = run_batched(V, torch, args)

    cool = run_cooldown_2d(V, torch, args) if not args.no_heisenberg else None
    wolff = run_wolff(V, torch, args) if not args.no_heisenberg else None
    sub = run_sublattice(V, torch, args) if not args.no_heisenberg else None
    heis = hyst = None
    if not args.no_heisenberg:
        heis = run_heisenberg(V, torch, args)
        hyst = run_hysteresis(V, torch, args)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        v, dt = cpu_baseline_sample(threads=1, sweeps=2)
        cpu = {"value": v, "unit": "flips/ns", "cores": 1, "kind": "port",
               "sample": f"2 measured reference sweeps of the 256^3 lattice on one core ({dt:.1f} s of sweeping)"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "flips/ns", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dev_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int8", "data": "synthetic",
            "config": {"workload": f"ising-sc-{n_l}^3-pbc-J1-h0 plain single lattice, checkerboard kernels",
                       "lattice": [n_l, n_l, n_l], "spins": N, "sweeps_per_step": SWEEPS_PER_STEP,
                       "temperatures": "CoolDown(5.5, 3.5, 0.1) ladder, one per step",
                       "measurement": "per-sweep E and |M| on device",
                       "l2": "flushed between steps (256 MiB write, outside the events); the 16.8 MB lattice is "
                             "L2-resident within a step",
                       "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                       "path": {1: "generic", 2: "structured", 4: "tiled"}.get(info.path, "?")},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "kernel": kernel, "launch_ms": pass_ms,
                         "launch_ms_isolated_events": iso_pass_ms,
                         "alg_bytes_per_launch": alg_bytes_per_launch, "peak_kind": peak_kind,
                         "note": "frac > 1 means the lattice is served from L2"},
            "e2e": {"value": e2e_value, "unit": "flips/ns", "h2d_bytes_per_step": N,
                    "d2h_bytes_per_step": N + 16 * SWEEPS_PER_STEP},
            "gpu_launches": launches_per_step * args.steps,
            "cpu_baseline": cpu,
            "tiled": tiled_cmp,
            "batched": batched,
            "batched_vs_plain": (batched["value"] / value) if batched else None,
            "cooldown_2d": cool,
            "wolff": wolff,
            "sublattice": sub,
            "heisenberg": heis,
            "hysteresis_batch": hyst,
            "clocks": clk.summary(),
            "wall_s": wall,
            "sweep_ms": sweep_ms,
        }
        print(json.dumps(line), flush=True)
    eng.close()
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
