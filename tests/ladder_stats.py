"""Helpers for the statistical parity tests: independent chains of the GPU
engine and of the reference restatement (ref_cpu) over a temperature or
field schedule, and the StatSensor observables compared between them.

Observables (src/instrument.rs:113-126, src/accumulator.rs:42-63): per point
of a schedule, <E>/N, <|M|>/N, C = (<E^2> - <E>^2) / (N T^2) and
chi = (<|M|^2> - <|M|>^2) / (N T), with E the Compound total energy and |M|
the magnetisation magnitude, both per sweep.  Each arm runs R independent
chains (own seeds and initial states); the moments are pooled over all
chains (equal weights) and their standard errors are jackknife errors over
chains, which need no assumption on autocorrelation times within a chain.
"""
from __future__ import annotations

import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np

OBS = ("E/N", "|M|/N", "C", "chi")


def moments(E, M):
    """Per-chain moments <E>, <E^2>, <|M|>, <|M|^2> of one measured stretch."""
    E = np.asarray(E, dtype=np.float64)
    M = np.asarray(M, dtype=np.float64)
    return np.array([E.mean(), (E * E).mean(), M.mean(), (M * M).mean()])


def observables(mom, N, T):
    """mom: (R, 4) per-chain moments -> ((4,) pooled observables, (4,) jackknife errors)."""
    mom = np.asarray(mom, dtype=np.float64)
    R = mom.shape[0]

    def obs(m):
        e, e2, a, a2 = m
        return np.array([e / N, a / N, (e2 - e * e) / (N * T * T), (a2 - a * a) / (N * T)])

    full = obs(mom.mean(axis=0))
    tot = mom.sum(axis=0)
    jk = np.array([obs((tot - mom[i]) / (R - 1)) for i in range(R)])
    err = np.sqrt((R - 1) / R * ((jk - jk.mean(axis=0)) ** 2).sum(axis=0))
    return full, err


def compare(gpu, cpu, N, points, labels=None):
    """gpu, cpu: (P, R, 4) moments per schedule point.  Returns rows
    (point label, observable, gpu value, gpu error, cpu value, cpu error, z)."""
    rows = []
    for k, T in enumerate(points):
        g, ge = observables(gpu[k], N, T)
        c, ce = observables(cpu[k], N, T)
        for i, name in enumerate(OBS):
            s = float(np.hypot(ge[i], ce[i]))
            d = float(g[i] - c[i])
            if s > 0:
                z = d / s
            else:  # both arms frozen (no fluctuation at all): the values must agree
                z = 0.0 if abs(d) <= 1e-12 * max(1.0, abs(g[i])) else np.inf
            rows.append(((labels[k] if labels else T), name, float(g[i]), float(ge[i]), float(c[i]), float(ce[i]), z))
    return rows


def failures(rows, limit=3.0):
    return [r for r in rows if not abs(r[6]) <= limit]


def table(rows):
    return "\n".join(f"{r[0]!s:>8} {r[1]:>6}  gpu {r[2]:+.6g} +- {r[3]:.3g}  cpu {r[4]:+.6g} +- {r[5]:.3g}  z {r[6]:+.2f}"
                     for r in rows)


def check_with_retest(run, limit=3.0):
    """run(attempt) -> comparison rows of one full measurement (attempt 0, and
    attempt 1 with new independent seeds for both arms).

    With a few hundred comparisons at 3 combined standard errors, about one
    excursion beyond 3 sigma is expected from chance alone (0.27 % each).  A
    point outside the limit is therefore measured once more, with new seeds
    for both arms, and must then lie within it; a real disagreement between
    the arms shows in both measurements."""
    rows = run(0)
    bad = failures(rows, limit)
    if not bad:
        return rows, None
    keys = {(r[0], r[1]) for r in bad}
    again = run(1)
    still = [r for r in again if (r[0], r[1]) in keys and not abs(r[6]) <= limit]
    assert not still, ("outside %.1f combined standard errors twice:\n" % limit) + table(still) + \
        "\nfirst measurement:\n" + table(bad)
    return rows, again


def gpu_chains(make_engine, R, schedule, relax, measure, to_EM, init=None):
    """R engines (make_engine(r)) run concurrently on their own streams over
    `schedule` (a list of (T, b, |B|)); returns (P, R, 4) moments.  init:
    optional (T, b, |B|, sweeps) relaxed before the schedule."""
    engines = [make_engine(r) for r in range(R)]
    try:
        for e in engines:
            e.init_random()
        if init is not None:
            T0, b0, m0, n0 = init
            for e in engines:
                e.set_thermostat(T0, b0, m0)
                e.sweeps_async(n0, measure=False)
        out = np.zeros((len(schedule), R, 4))
        for k, (T, b, mag) in enumerate(schedule):
            for e in engines:
                e.set_thermostat(T, b, mag)
                if relax:
                    e.sweeps_async(relax, measure=False)
                e.sweeps_async(measure, measure=True)
            for r, e in enumerate(engines):
                E, M = to_EM(e.read_sums(measure), T, mag)
                out[k, r] = moments(E, M)
        return out
    finally:
        for e in engines:
            e.close()


def cpu_chains(O, olat, kind, H, R, schedule, relax, measure, seed, proposal, init=None, threads=None):
    """R independent ref_cpu chains (the reference's random-site Metropolis
    with its CLI measurement) over the same schedule, run on host threads;
    returns (P, R, 4) moments."""
    g = O.Graph(olat)

    def chain(r):
        s = g.ising_init(seed + r) if kind == 0 else g.heis_init(seed + r)
        rng = O.pcg64(1000003 * seed + r)
        if init is not None:
            T0, b0, m0, n0 = init
            s, _ = g.ref_sweeps(kind, s, H, T0, n0, rng, b=b0, bmag=m0, proposal=proposal, measure=False,
                                clone=False)
        res = np.zeros((len(schedule), 4))
        for k, (T, b, mag) in enumerate(schedule):
            if relax:
                s, _ = g.ref_sweeps(kind, s, H, T, relax, rng, b=b, bmag=mag, proposal=proposal, measure=False,
                                    clone=False)
            s, obs = g.ref_sweeps(kind, s, H, T, measure, rng, b=b, bmag=mag, proposal=proposal, measure=True,
                                  clone=False)
            res[k] = moments(obs[:, 0], obs[:, 1])
        return res

    n = threads or min(R, os.cpu_count() or 1)
    with ThreadPoolExecutor(max_workers=n) as ex:
        res = list(ex.map(chain, range(R)))
    return np.stack(res, axis=1)
