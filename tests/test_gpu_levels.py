"""Level-scheduled sweep kernel (params "kernel": "levels") against the oracle.

Integer Ising models whose terms have one or two members, counter streams:
one warp per walker runs the variables of each dependency level at once.
The bar is the same as for the other kernels: identical trajectories, costs
compared with ==, final and lowest states equal.
"""
import numpy as np
import pytest

import qiotoolkit_gb300 as q
from qiotoolkit_gb300 import instances as I
from oracle import oracle as O

pytestmark = pytest.mark.gpu

SA = "simulatedannealing.qiotoolkit"
PA = "populationannealing.cpu"


def _er_int(n, m, seed, big):
    off, ids, _ = I.er_ising(n, m, seed=seed)
    rng = np.random.default_rng(seed)
    coef = rng.integers(-big, big + 1, len(off) - 1).astype(float)
    return off, ids, coef


def _square_fields(L, seed):
    """+-J lattice with integer fields (one-member terms: the padding spin)."""
    off, ids, coef = I.square_pm_j(L, seed=seed)
    rng = np.random.default_rng(seed)
    n = L * L
    off2 = np.concatenate([off, off[-1] + 1 + np.arange(n)])
    ids2 = np.concatenate([ids, np.arange(n)])
    coef2 = np.concatenate([coef, rng.integers(-2, 3, n).astype(float)])
    return off2, ids2.astype(ids.dtype), coef2


def _square_big(L, seed):
    """+-3000 couplings: chunk sums beyond 16 bits (32-bit chunk sums)."""
    off, ids, coef = I.square_pm_j(L, seed=seed)
    return off, ids, coef * 3000.0


def _ring(n, seed):
    """+-J ring: two incidences per variable (4-word level entries)."""
    rng = np.random.default_rng(seed)
    off = np.arange(0, 2 * n + 1, 2)
    ids = np.stack([np.arange(n), (np.arange(n) + 1) % n], 1).ravel()
    return off, ids, rng.choice([-1.0, 1.0], n)


def _hub(n, seed):
    """ER couplings plus a hub joined to every fifth variable: more than 15
    incidences at the hub (level entries without records)."""
    off, ids, coef = _er_int(n, 2 * n, seed, 3)
    hub = np.arange(1, n, 5)
    off2 = np.concatenate([off, off[-1] + 2 * np.arange(1, len(hub) + 1)])
    ids2 = np.concatenate([ids, np.stack([np.zeros_like(hub), hub], 1).ravel()])
    rng = np.random.default_rng(seed + 1)
    return off2, ids2.astype(ids.dtype), np.concatenate([coef, rng.integers(-3, 4, len(hub)).astype(float)])


MODELS = {
    "ring": lambda: _ring(200, 30),
    "hub": lambda: _hub(150, 29),
    "square16": lambda: I.square_pm_j(16, seed=31),
    "square_fields": lambda: _square_fields(12, 32),
    "square_big": lambda: _square_big(10, 33),
    "cubic6": lambda: I.cubic_pm_j(6, seed=34),
    "cubic8": lambda: I.cubic_pm_j(8, seed=35),
    "er_int": lambda: _er_int(120, 300, 36, 5),
    "er_bigint": lambda: _er_int(80, 200, 37, 300),
}


def _both(gen):
    off, ids, coef = gen()
    return (q.Model("ising", off=off, ids=ids, coef=coef),
            O.Model("ising", off=off, ids=ids, coef=coef))


def _same(g, o):
    np.testing.assert_array_equal(g["cost"], o.cost)
    np.testing.assert_array_equal(g["lowest"], o.lowest)
    np.testing.assert_array_equal(g["attempts"], o.attempts)
    np.testing.assert_array_equal(g["accepts"], o.accepts)
    np.testing.assert_array_equal(g["states"], o.states)
    np.testing.assert_array_equal(g["lowest_states"], o.lowest_states)


@pytest.mark.parametrize("name", list(MODELS))
def test_levels_sa_matches_oracle(name):
    g, o = _both(MODELS[name])
    assert g.info.level_kernel == 1, name
    params = {"seed": 77, "sweeps": 60, "restarts": 40, "beta_start": 0.05,
              "beta_stop": 2.5, "rng_mode": "counter", "kernel": "levels"}
    s = q.Solver(g, SA, {"params": params}).init().run()
    assert s.stats().sweep_kernel == 3
    r = O.run(o, "sa", seed=77, step_limit=60, restarts=40, sched=("linear", 0.05, 2.5),
              rng_mode="counter", threads=4)
    _same(s.replicas(), r)
    c, _ = s.best()
    assert c == r.best_cost


LARGE = {
    # name: (model, sweeps, restarts, kernel param)
    "square64_auto": (lambda: I.square_pm_j(64, seed=38), 12, 30, None),      # auto choice
    "square128": (lambda: I.square_pm_j(128, seed=40), 6, 20, "levels"),
    "square256": (lambda: I.square_pm_j(256, seed=41), 3, 12, "levels"),
    "square256_big": (lambda: _square_big(256, 42), 3, 12, "levels"),         # int2 records
    "cubic20": (lambda: I.cubic_pm_j(20, seed=39), 6, 20, "levels"),
}


@pytest.mark.parametrize("name", list(LARGE))
def test_levels_sa_large_lattices_match_oracle(name):
    gen, sweeps, restarts, kern = LARGE[name]
    g, o = _both(gen)
    params = {"seed": 5, "sweeps": sweeps, "restarts": restarts, "beta_start": 0.3,
              "beta_stop": 3.0, "rng_mode": "counter"}
    if kern:
        params["kernel"] = kern
    s = q.Solver(g, SA, {"params": params}).init().run()
    assert s.stats().sweep_kernel == 3
    r = O.run(o, "sa", seed=5, step_limit=sweeps, restarts=restarts, sched=("linear", 0.3, 3.0),
              rng_mode="counter", threads=8)
    _same(s.replicas(), r)


@pytest.mark.parametrize("name", ["square16", "cubic6", "er_int"])
def test_levels_equal_other_kernels(name):
    g, _ = _both(MODELS[name])
    out = {}
    for kern in ("levels", "lanes", "warp"):
        p = {"seed": 9, "sweeps": 40, "restarts": 33, "beta_start": 0.2, "beta_stop": 4.0,
             "rng_mode": "counter", "kernel": kern}
        out[kern] = q.Solver(g, SA, {"params": p}).init().run().replicas()
    for kern in ("lanes", "warp"):
        for k in ("cost", "lowest", "attempts", "accepts", "states", "lowest_states"):
            np.testing.assert_array_equal(out["levels"][k], out[kern][k], err_msg=f"{kern} {k}")


def test_levels_single_walker_and_pieces():
    """One walker; a run split into pieces (the serving path) equals one run."""
    g, o = _both(MODELS["square16"])
    p = {"seed": 3, "sweeps": 25, "restarts": 1, "beta_start": 0.1, "beta_stop": 2.0,
         "rng_mode": "counter", "kernel": "levels"}
    s = q.Solver(g, SA, {"params": p}).init().run()
    r = O.run(o, "sa", seed=3, step_limit=25, restarts=1, sched=("linear", 0.1, 2.0), rng_mode="counter")
    _same(s.replicas(), r)
    srv = q.Server(max_active=4, sa_sweeps_per_piece=7)
    try:
        rid = srv.submit(g, SA, {"params": p})
        res = srv.wait(rid)
    finally:
        srv.close()
    assert res["solutions"] == s.result()["solutions"]


@pytest.mark.parametrize("name", ["square16", "cubic6", "square_fields"])
def test_levels_pa_multinomial_matches_oracle(name):
    g, o = _both(MODELS[name])
    params = {"seed": 21, "sweeps": 25, "population": 70, "beta_start": 0.0, "beta_stop": 2.5,
              "sweeps_per_replica": 3, "rng_mode": "counter", "resampling": "multinomial",
              "kernel": "levels"}
    s = q.Solver(g, PA, {"params": params}).init().run()
    assert s.stats().sweep_kernel == 3
    r = O.run(o, "pa", seed=21, step_limit=25, population=70, sched=("linear", 0.0, 2.5),
              sweeps_per_replica=3, rng_mode="counter", resampling="multinomial", threads=4)
    _same(s.replicas(), r)
    c, _ = s.best()
    assert c == r.best_cost
