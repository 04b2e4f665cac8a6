"""Parameter-free simulated annealing on the GPU against the oracle.

The library's search (linear search over sweep sample points, repeated SA
runs whose restarts fork from one continuing master stream) must make the
same runs with the same lowest costs as the oracle's restatement of
ParameterFreeLinearSearchSolver<SAParameterFree>, and return the same best
state and parameters.  The cases stop on the non-improvement rule, well
inside the time limit, and have no constant term (lowest costs compare
directly).
"""
import numpy as np
import pytest

import qiotoolkit_gb300 as q
from qiotoolkit_gb300 import instances as I
from oracle import oracle as O

pytestmark = pytest.mark.gpu

PF = "simulatedannealing-parameterfree.qiotoolkit"

CASES = {
    "er_ising": ("ising", lambda: I.er_ising(60, 150, seed=51), 11),
    "pubo": ("pubo", lambda: I.random_pubo(40, 100, seed=52), 12),
    "square_pm_j": ("ising", lambda: I.square_pm_j(8, seed=53), 13),
}


@pytest.mark.parametrize("name", list(CASES))
def test_sa_parameter_free_matches_oracle(name):
    kind, gen, seed = CASES[name]
    off, ids, coef = gen()
    terms = [(float(coef[k]), [int(x) for x in ids[off[k]:off[k + 1]]]) for k in range(len(coef))]
    g = q.Model(kind, off=off, ids=ids, coef=coef)
    o = O.Model(kind, off=off, ids=ids, coef=coef)
    params = {"seed": seed, "min_num_restarts": 4, "timeout": 120}
    s = q.Solver(g, PF, {"params": params}).init().run()
    res = s.result()
    runs = res["benchmark"]["parameter_free"]["runs"]
    assert res["benchmark"]["parameter_free"]["stop"] == "no improvement"
    ref = O.sa_parameter_free(o, kind, terms, seed=seed, min_num_restarts=4)
    assert [(r["sweeps"], r["restarts"], r["lowest"]) for r in runs] == \
        [(sl, r, obj) for sl, r, obj in ref["trace"]]
    sol = res["solutions"]
    assert (sol["parameters"]["sweeps"], sol["parameters"]["restarts"]) == ref["params"]
    b0, b1 = ref["betas"]
    assert sol["parameters"]["beta_start"] == b0 and sol["parameters"]["beta_stop"] == b1
    rep = s.replicas()
    np.testing.assert_array_equal(rep["lowest"], [ref["best"]])
    np.testing.assert_array_equal(rep["lowest_states"][0], ref["best_state"])


PTPF = "paralleltempering-parameterfree.qiotoolkit"


@pytest.mark.parametrize("name", list(CASES))
def test_pt_parameter_free_matches_oracle(name):
    kind, gen, seed = CASES[name]
    off, ids, coef = gen()
    terms = [(float(coef[k]), [int(x) for x in ids[off[k]:off[k + 1]]]) for k in range(len(coef))]
    g = q.Model(kind, off=off, ids=ids, coef=coef)
    o = O.Model(kind, off=off, ids=ids, coef=coef)
    params = {"seed": seed, "min_num_betas": 10, "timeout": 120}
    s = q.Solver(g, PTPF, {"params": params}).init().run()
    res = s.result()
    runs = res["benchmark"]["parameter_free"]["runs"]
    assert res["benchmark"]["parameter_free"]["stop"] == "no improvement"
    ref = O.pt_parameter_free(o, kind, terms, seed=seed, min_num_betas=10)
    assert [(r["sweeps"], r["restarts"], r["lowest"]) for r in runs] == list(ref["trace"])
    sol = res["solutions"]
    assert sol["parameters"]["sweeps"] == ref["sweeps"]
    ladder = sol["parameters"]["all_betas"]  # a list schedule renders as segments
    assert [seg["value"] for seg in ladder["segments"]] == ref["betas"]
    rep = s.replicas()
    np.testing.assert_array_equal(rep["lowest"], [ref["best"]])
    np.testing.assert_array_equal(rep["lowest_states"][0], ref["best_state"])


TABU_CASES = {
    "er_ising": ("ising", lambda: I.er_ising(60, 150, seed=1), 3),
    "cubic": ("ising", lambda: I.cubic_pm_j(4, seed=2), 3),
    "pubo": ("pubo", lambda: I.random_pubo(50, 150, seed=3), 3),
}


@pytest.mark.parametrize("name", list(TABU_CASES))
def test_tabu_parameter_free_matches_oracle(name):
    """ParameterFreeLinearSearchSolver<TabuParameterFree>: the same runs
    (sweeps, restarts, per-restart tenures, lowest costs), best state and
    parameters as the oracle's restatement."""
    kind, gen, seed = TABU_CASES[name]
    off, ids, coef = gen()
    g = q.Model(kind, off=off, ids=ids, coef=coef)
    o = O.Model(kind, off=off, ids=ids, coef=coef)
    s = q.Solver(g, "tabu-parameterfree.qiotoolkit",
                 {"params": {"seed": seed, "min_num_restarts": 8, "timeout": 120}}).init().run()
    res = s.result()
    pf = res["benchmark"]["parameter_free"]
    assert pf["stop"] == "no improvement"
    ref = O.tabu_parameter_free(o, seed=seed, min_num_restarts=8)
    assert [(r["sweeps"], r["restarts"], r["lowest"]) for r in pf["runs"]] == \
        [(sl, r, obj) for sl, r, obj in ref["trace"]]
    sol = res["solutions"]
    assert (sol["parameters"]["sweeps"], sol["parameters"]["restarts"]) == ref["params"]
    c, st = s.best()
    assert c == ref["best"]
    np.testing.assert_array_equal(st, ref["best_state"])
