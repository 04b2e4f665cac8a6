"""Randomised parity sweep: many small random models against the oracle.

Each case draws a model kind (Ising cached / plain, PUBO counter / plain,
MaxSAT), a size (1 to ~300 variables, so blocks end ragged), term orders,
integer or real weights, a solver (SA or PT), an RNG mode and, for two-body
Ising models, the kernel.  Every walker must match the oracle exactly.
"""
import numpy as np
import pytest

import qiotoolkit_gb300 as q
from qiotoolkit_gb300.instances import _pack
from oracle import oracle as O

pytestmark = pytest.mark.gpu

SA = "simulatedannealing.qiotoolkit"
PT = "paralleltempering.qiotoolkit"


def _random_model(rng):
    kind = rng.choice(["ising", "ising_plain", "pubo", "pubo_plain", "maxsat"])
    n = int(rng.choice([1, 2, 5, 31, 32, 33, 63, 64, 65, 100, 180, 300]))
    m = int(rng.integers(1, 4 * n + 2))
    integer = bool(rng.integers(0, 2))
    ids = []
    for _ in range(m):
        if kind == "maxsat":
            o = int(rng.integers(1, min(n, 4) + 1))
            vs = rng.choice(n, size=o, replace=False) + 1
            ids.append((vs * rng.choice([-1, 1], size=o)).tolist())
        else:
            o = int(rng.integers(1, min(n, 4 if kind.startswith("pubo") else 2) + 1))
            if kind.startswith("ising") and rng.random() < 0.7:
                o = min(2, n)
            ids.append(sorted(rng.choice(n, size=o, replace=False).tolist()))
    if kind == "maxsat":
        coef = rng.integers(1, 10, m).astype(float) if integer else rng.uniform(1, 10, m)
    else:
        coef = rng.integers(-4, 5, m).astype(float) if integer else rng.standard_normal(m)
    off, ids_f, c = _pack(ids, coef)
    return kind, off, ids_f, c


def _same(g, o):
    np.testing.assert_array_equal(g["cost"], o.cost)
    np.testing.assert_array_equal(g["lowest"], o.lowest)
    np.testing.assert_array_equal(g["attempts"], o.attempts)
    np.testing.assert_array_equal(g["accepts"], o.accepts)
    np.testing.assert_array_equal(g["lowest_states"], o.lowest_states)


@pytest.mark.parametrize("case", range(40))
def test_fuzz(case):
    rng = np.random.default_rng(1000 + case)
    kind, off, ids, coef = _random_model(rng)
    g = q.Model(kind, off=off, ids=ids, coef=coef)
    o = O.Model(kind, off=off, ids=ids, coef=coef)
    mode = str(rng.choice(["replay", "counter"]))
    sweeps = int(rng.integers(2, 40))
    seed = int(rng.integers(0, 2 ** 31))
    full = kind == "maxsat"
    if rng.random() < 0.7:
        restarts = int(rng.integers(1, 40))
        b0, b1 = float(rng.uniform(0, 0.5)), float(rng.uniform(0.6, 4.0))
        params = {"seed": seed, "sweeps": sweeps, "restarts": restarts, "beta_start": b0,
                  "beta_stop": b1, "rng_mode": mode, "maxsat_full_sweep": full}
        kernels = ["warp"]
        if kind == "ising" and q.Model(kind, off=off, ids=ids, coef=coef).info.max_locality <= 2:
            kernels.append("lanes")
        r = O.run(o, "sa", seed=seed, step_limit=sweeps, restarts=restarts, sched=("linear", b0, b1),
                  rng_mode=mode, threads=4, full_maxsat_sweep=full)
        for kern in kernels:
            s = q.Solver(g, SA, {"params": dict(params, kernel=kern)}).init().run()
            _same(s.replicas(), r)
    else:
        temps = sorted(set(np.round(rng.uniform(0.1, 4.0, int(rng.integers(2, 9))), 3).tolist()))
        params = {"seed": seed, "sweeps": sweeps, "all_betas": temps, "rng_mode": mode,
                  "maxsat_full_sweep": full}
        s = q.Solver(g, PT, {"params": params}).init().run()
        r = O.run(o, "pt", seed=seed, step_limit=sweeps, sched=("list", 0, 0), sched_values=temps,
                  rng_mode=mode, threads=4, full_maxsat_sweep=full)
        _same(s.replicas(), r)
