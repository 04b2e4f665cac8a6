"""Parameter-free population annealing and SSMC (the Bayesian searches) on
the GPU against the oracle, with the reference's replayed streams and with
counter streams (each run keyed by one draw of the master stream).

The search's runs share one master stream.  The first four take the
adapter's initial parameter vectors, whose alpha or beta jitter is drawn from
that stream; later runs take the strategy's picks.  The oracle replays the
same sequence of runs from the seed: it computes the initial vectors itself
and takes the picks from the library's run list.  Every run the time limit
did not cut short must report the oracle's lowest cost for that run, and the
result must be the best of them by the reference's rule.  The strategy's picks themselves are
checked by range only; they are this library's own Gaussian-process model,
not a replay of the reference's.
"""
import numpy as np
import pytest

import qiotoolkit_gb300 as q
from qiotoolkit_gb300 import instances as I
from oracle import oracle as O

pytestmark = pytest.mark.gpu

PAPF = "populationannealing-parameterfree.cpu"
SSMCPF = "substochasticmontecarlo-parameterfree.cpu"

CASES = {
    "er_ising": ("ising", lambda: I.er_ising(48, 120, seed=61), 21),
    "pubo": ("pubo", lambda: I.random_pubo(32, 80, seed=62), 22),
}


def _terms(off, ids, coef):
    return [(float(coef[k]), [int(x) for x in ids[off[k]:off[k + 1]]]) for k in range(len(coef))]


def _check(res, ref, n_init=4):
    pf = res["benchmark"]["parameter_free"]
    runs = pf["runs"]
    assert len(runs) > n_init and any(r["recommended"] for r in runs)
    for k, (r, (v, sl, low, _)) in enumerate(zip(runs, ref)):
        if k < n_init:
            assert r["params"] == v
        assert r["step_limit"] == sl
        if r["steps"] < r["step_limit"]:
            break  # cut by the time limit: the master stream diverges from here
        assert r["lowest"] == low, (k, r, low)
    # improvements count only beyond 1e-11 (parameter_free_solver.h:123-151),
    # so the result is one of the runs' costs within that of the lowest
    cost = res["solutions"]["cost"]
    assert cost in [r["lowest"] for r in runs]
    assert abs(cost - min(r["lowest"] for r in runs)) <= 1e-11


@pytest.mark.parametrize("mode", ["replay", "counter", "multinomial"])
@pytest.mark.parametrize("name", list(CASES))
def test_pa_parameter_free_runs_match_oracle(name, mode):
    kind, gen, seed = CASES[name]
    off, ids, coef = gen()
    g = q.Model(kind, off=off, ids=ids, coef=coef)
    o = O.Model(kind, off=off, ids=ids, coef=coef)
    rng = "replay" if mode == "replay" else "counter"
    rs = "multinomial" if mode == "multinomial" else "reference"
    s = q.Solver(g, PAPF, {"params": {"seed": seed, "timeout": 20, "threads": 4, "rng_mode": rng,
                                      "resampling": rs}}).init().run()
    res = s.result()
    runs = res["benchmark"]["parameter_free"]["runs"]
    ref = O.pa_parameter_free_replay(o, kind, _terms(off, ids, coef), seed=seed, threads=4,
                                     runs=[r["params"] for r in runs], rng_mode=rng, resampling=rs)
    _check(res, ref)
    for r in runs:
        v = r["params"]
        assert v[0] >= 20 and 1.0 <= v[3] <= 4.0 and 1.00000001 <= v[2] <= 3.0
    par = res["solutions"]["parameters"]
    assert par["beta_stop"] > par["beta_start"] > 0 and par["population"] >= 4


@pytest.mark.parametrize("mode", ["replay", "counter"])
@pytest.mark.parametrize("name", list(CASES))
def test_ssmc_parameter_free_runs_match_oracle(name, mode):
    kind, gen, seed = CASES[name]
    off, ids, coef = gen()
    g = q.Model(kind, off=off, ids=ids, coef=coef)
    o = O.Model(kind, off=off, ids=ids, coef=coef)
    s = q.Solver(g, SSMCPF, {"params": {"seed": seed, "timeout": 20, "threads": 4,
                                        "rng_mode": mode}}).init().run()
    res = s.result()
    runs = res["benchmark"]["parameter_free"]["runs"]
    ref = O.ssmc_parameter_free_replay(o, seed=seed, threads=4, runs=[r["params"] for r in runs],
                                       sweep_size=g.n_vars, rng_mode=mode)
    _check(res, ref)
    for r in runs:
        v = r["params"]
        assert 1.0 <= v[2] <= 5.0 and 0.8 <= v[4] <= 1.0 and 1.0 <= v[6] <= 8.0
    par = res["solutions"]["parameters"]
    assert par["step_limit"] >= 2 and par["target_population"] >= 4


def test_ssmc_parameter_free_maxsat():
    """MaxSat models: a sweep is one variable (markov/model.h:169), so the
    step counts start at initial_sweeps."""
    off, ids, coef = I.weighted_maxsat(40, seed=63)
    g = q.Model("maxsat", off=off, ids=ids, coef=coef)
    o = O.Model("maxsat", off=off, ids=ids, coef=coef)
    s = q.Solver(g, SSMCPF, {"params": {"seed": 5, "timeout": 10, "threads": 4}}).init().run()
    res = s.result()
    runs = res["benchmark"]["parameter_free"]["runs"]
    assert runs[0]["params"][0] == 20.0
    ref = O.ssmc_parameter_free_replay(o, seed=5, threads=4, runs=[r["params"] for r in runs], sweep_size=1)
    _check(res, ref)


def test_parameter_free_time_limit_honoured():
    """A short time limit ends the search at about that time (the reference's
    HonoringTimeout test, solver/test/ssmc_pf_test.cc:152-195, with its own
    slack)."""
    off, ids, coef = I.er_ising(200, 600, seed=64)
    g = q.Model("ising", off=off, ids=ids, coef=coef)
    for target in (PAPF, SSMCPF):
        s = q.Solver(g, target, {"params": {"seed": 1, "timeout": 2, "threads": 4,
                                            "nonimprovement_limit": 1000}}).init().run()
        res = s.result()
        assert res["benchmark"]["parameter_free"]["stop"] == "time limit"
        assert res["benchmark"]["gb300"]["run_ms"] < 2000 * 1.5 + 1000
