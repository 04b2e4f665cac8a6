"""The field-cached sweep ("kernel": "fields") against the oracle, through the
C ABI (GPU required).

Bar: bit-exact, as every sweep kernel: under replayed PCG streams each
walker's final and lowest cost (== on FP64), attempt/accept counts and
final/lowest states equal the oracle's; counter streams likewise against the
oracle's counter mode.  The edge models drive the kernel's slow paths: rows of
more than 32 incidences (exact differences logged by the decider), 32-variable
blocks with more incidences than a shared-memory tile (records read from
global memory), terms with more than three co-members (members read from the
term lists), negated literals (MaxSat).
"""
import numpy as np
import pytest

import qiotoolkit_gb300 as q
from qiotoolkit_gb300 import instances as I
from oracle import oracle as O

pytestmark = pytest.mark.gpu

SA = "simulatedannealing.qiotoolkit"
PT = "paralleltempering.qiotoolkit"


def both(kind, off, ids, coef):
    return (q.Model(kind, off=off, ids=ids, coef=coef),
            O.Model(kind, off=off, ids=ids, coef=coef))


def assert_same_walkers(g, o):
    np.testing.assert_array_equal(g["cost"], o.cost)
    np.testing.assert_array_equal(g["lowest"], o.lowest)
    np.testing.assert_array_equal(g["attempts"], o.attempts)
    np.testing.assert_array_equal(g["accepts"], o.accepts)
    np.testing.assert_array_equal(g["states"], o.states)
    np.testing.assert_array_equal(g["lowest_states"], o.lowest_states)


def hub_pubo(n=300, seed=41, integer=False):
    """A random PUBO plus hub variables: variables 0 and 1 sit in 120 terms
    each (rows wider than 32 and blocks wider than a tile) and some terms
    have five or six members (more than three co-members)."""
    rng = np.random.default_rng(seed)
    terms = []
    for v in range(n):  # fields first: internal ids equal input ids
        terms.append((rng.normal(), [v]))
    for _ in range(3 * n):
        k = int(rng.choice([2, 3, 4, 5, 6], p=[0.4, 0.3, 0.15, 0.1, 0.05]))
        terms.append((rng.normal(), sorted(rng.choice(n, k, replace=False).tolist())))
    for hub in (0, 1):
        for _ in range(120):
            others = rng.choice(np.arange(2, n), 2, replace=False).tolist()
            terms.append((rng.normal(), sorted([hub] + others)))
    if integer:
        terms = [(float(np.round(3 * c)) or 1.0, ids) for c, ids in terms]
    return O.flatten_terms(terms)


def dense_block_ising(n=256, seed=42):
    """Ising couplings concentrated on the first 64 variables (blocks of more
    than 512 incidences) plus fields."""
    rng = np.random.default_rng(seed)
    terms = [(rng.uniform(-0.5, 0.5), [v]) for v in range(n)]
    seen = set()
    while len(seen) < 1200:
        i, j = sorted(rng.choice(64, 2, replace=False).tolist())
        seen.add((i, j))
    for i, j in sorted(seen):
        terms.append((float(rng.choice([-1.0, 1.0])), [i, j]))
    for _ in range(400):
        i, j = sorted(rng.choice(n, 2, replace=False).tolist())
        if (i, j) not in seen:
            seen.add((i, j))
            terms.append((rng.normal(), [i, j]))
    return O.flatten_terms(terms)


MODELS = {
    "ising_real": ("ising", lambda: I.er_ising(300, 900, seed=11)),
    "ising_int": ("ising", lambda: I.cubic_pm_j(6, seed=12)),
    "ising_dense_block": ("ising", dense_block_ising),
    "pubo_real": ("pubo", lambda: I.random_pubo(400, 1600, seed=14)),
    "pubo_int": ("pubo", lambda: I.random_pubo(300, 1200, seed=15, integer=True)),
    "pubo_hub": ("pubo", hub_pubo),
    "pubo_hub_int": ("pubo", lambda: hub_pubo(integer=True)),
    "maxsat_real": ("maxsat", lambda: I.weighted_maxsat(150, seed=17)),
    "maxsat_int": ("maxsat", lambda: I.weighted_maxsat(150, seed=18, integer=True)),
}


@pytest.mark.parametrize("name", list(MODELS))
@pytest.mark.parametrize("mode", ["replay", "counter"])
def test_fields_sa(name, mode):
    kind, gen = MODELS[name]
    g, o = both(kind, *gen())
    params = {"seed": 77, "sweeps": 50, "restarts": 10, "beta_start": 0.1, "beta_stop": 4.0,
              "rng_mode": mode, "maxsat_full_sweep": kind == "maxsat", "kernel": "fields"}
    s = q.Solver(g, SA, {"params": params}).init().run()
    assert s.stats().sweep_kernel == 8
    r = O.run(o, "sa", seed=77, step_limit=50, restarts=10, sched=("linear", 0.1, 4.0),
              rng_mode=mode, threads=4, full_maxsat_sweep=kind == "maxsat")
    assert_same_walkers(s.replicas(), r)
    assert s.best()[0] == r.best_cost


@pytest.mark.parametrize("name", ["ising_real", "ising_dense_block", "pubo_real", "pubo_hub",
                                  "pubo_int", "maxsat_real"])
@pytest.mark.parametrize("mode", ["replay", "counter"])
def test_fields_pt(name, mode):
    kind, gen = MODELS[name]
    g, o = both(kind, *gen())
    temps = {"type": "geometric", "initial": 0.05, "final": 3.0, "count": 8}
    params = {"seed": 42, "sweeps": 30, "temperatures": temps, "rng_mode": mode,
              "sweeps_per_replica": 2, "maxsat_full_sweep": True, "kernel": "fields"}
    s = q.Solver(g, PT, {"params": params}).init().run()
    assert s.stats().sweep_kernel == 8
    r = O.run(o, "pt", seed=42, step_limit=30, use_inverse=False,
              sched=("geometric", 0.05, 3.0), sched_count=8, sweeps_per_replica=2,
              rng_mode=mode, threads=4, full_maxsat_sweep=True)
    assert_same_walkers(s.replicas(), r)
    obs = s.pt_observables()
    np.testing.assert_array_equal(obs[:, :4], r.pt_obs[:, :4])


def test_fields_many_walkers_per_block():
    """512 walkers: four walkers (eight warps) share a block."""
    g, o = both("pubo", *I.random_pubo(500, 2000, seed=51))
    params = {"seed": 5, "sweeps": 20, "restarts": 512, "beta_start": 0.2, "beta_stop": 2.0,
              "kernel": "fields"}
    s = q.Solver(g, SA, {"params": params}).init().run()
    r = O.run(o, "sa", seed=5, step_limit=20, restarts=512, sched=("linear", 0.2, 2.0), threads=8)
    assert_same_walkers(s.replicas(), r)


def test_fields_chunked_launches_keep_fields():
    """A cost limit cuts the sweeps into one-sweep launches: the fields kept
    between launches must equal fields rebuilt from the state."""
    g, o = both("ising", *I.er_ising(300, 900, seed=61))
    params = {"seed": 9, "sweeps": 40, "restarts": 6, "beta_start": 0.1, "beta_stop": 3.0,
              "cost_limit": -1e9, "kernel": "fields"}
    s = q.Solver(g, SA, {"params": params}).init().run()
    r = O.run(o, "sa", seed=9, step_limit=40, restarts=6, sched=("linear", 0.1, 3.0), threads=4)
    assert_same_walkers(s.replicas(), r)


def test_fields_refuses_ineligible_models():
    off, ids, coef = I.er_ising(100, 300, seed=3)
    g = q.Model("ising_plain", off=off, ids=ids, coef=coef)
    with pytest.raises(q.QioError, match="fields"):
        q.Solver(g, SA, {"params": {"seed": 1, "sweeps": 5, "kernel": "fields"}}).init()
