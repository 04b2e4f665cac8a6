"""Edge cases of the sweep kernels against the oracle (bit-exact walkers).

* rows of more than 32 incidences (recomputed every round);
* a 32-variable block whose incidences overflow the shared tile (rows read
  from global memory);
* terms with more than six later co-members in the same block (the
  "recompute all" mark);
* coefficients outside the FP32 screen's range (every decision exact);
* single-variable and two-variable models.
"""
import numpy as np
import pytest

import qiotoolkit_gb300 as q
from qiotoolkit_gb300.instances import _pack
from oracle import oracle as O

pytestmark = pytest.mark.gpu

SA = "simulatedannealing.qiotoolkit"
PT = "paralleltempering.qiotoolkit"


def _same(g, o):
    np.testing.assert_array_equal(g["cost"], o.cost)
    np.testing.assert_array_equal(g["lowest"], o.lowest)
    np.testing.assert_array_equal(g["attempts"], o.attempts)
    np.testing.assert_array_equal(g["accepts"], o.accepts)
    np.testing.assert_array_equal(g["states"], o.states)
    np.testing.assert_array_equal(g["lowest_states"], o.lowest_states)


def _hub(kind, seed, n=120, hub_terms=90, integer=False):
    """Variables 0..n-1; variable 5 sits in hub_terms two- or three-body
    terms (a row far beyond 32 incidences), plus random terms."""
    rng = np.random.default_rng(seed)
    ids = [[i] for i in range(n)]
    for k in range(hub_terms):
        others = rng.choice([x for x in range(n) if x != 5], size=1 + (k % 2 if kind == "pubo" else 0),
                            replace=False).tolist()
        ids.append(sorted([5] + others))
    for _ in range(3 * n):
        o = 2 if kind == "ising" else int(rng.integers(1, 4))
        ids.append(sorted(rng.choice(n, size=o, replace=False).tolist()))
    c = rng.integers(-3, 4, len(ids)).astype(float) if integer else rng.standard_normal(len(ids))
    return _pack(ids, c)


def _dense_block(seed, n=64):
    """The first 32 variables each sit in ~40 terms: the block's incidences
    exceed the shared tile (640 FP64 / 768 integer incidences)."""
    rng = np.random.default_rng(seed)
    ids = [[i] for i in range(n)]
    for _ in range(700):
        a, b = rng.choice(32, size=2, replace=False)
        ids.append(sorted([int(a), int(b)]))
    for _ in range(2 * n):
        ids.append(sorted(rng.choice(n, size=2, replace=False).tolist()))
    return _pack(ids, rng.standard_normal(len(ids)))


def _long_terms(seed, n=96):
    """PUBO terms of order 8 over consecutive ids: each incidence has up to
    seven later co-members in its block."""
    rng = np.random.default_rng(seed)
    ids = [[i] for i in range(n)]
    for s0 in range(0, n - 8, 3):
        ids.append(list(range(s0, s0 + 8)))
    for _ in range(2 * n):
        ids.append(sorted(rng.choice(n, size=2, replace=False).tolist()))
    return _pack(ids, rng.standard_normal(len(ids)))


def _extreme(seed, n=150):
    """Coefficients of magnitude 1e-35 .. 1e35 (outside the FP32 screen)."""
    rng = np.random.default_rng(seed)
    ids = [[i] for i in range(n)] + [sorted(rng.choice(n, size=2, replace=False).tolist())
                                     for _ in range(3 * n)]
    mag = 10.0 ** rng.uniform(-35, 35, len(ids))
    return _pack(ids, mag * rng.choice([-1.0, 1.0], len(ids)))


CASES = {
    "hub_ising": ("ising", lambda: _hub("ising", 61)),
    "hub_pubo": ("pubo", lambda: _hub("pubo", 62)),
    "hub_pubo_int": ("pubo", lambda: _hub("pubo", 63, integer=True)),
    "dense_block": ("ising", lambda: _dense_block(64)),
    "long_terms": ("pubo", lambda: _long_terms(65)),
    "extreme_ising": ("ising", lambda: _extreme(66)),
    "extreme_pubo": ("pubo", lambda: _extreme(67)),
    "one_var": ("ising", lambda: _pack([[0]], [1.5])),
    "two_vars": ("pubo", lambda: _pack([[0, 1], [1], [0]], [-2.0, 1.0, 0.5])),
}


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("mode", ["replay", "counter"])
def test_edge_sa(name, mode):
    kind, gen = CASES[name]
    off, ids, coef = gen()
    g = q.Model(kind, off=off, ids=ids, coef=coef)
    o = O.Model(kind, off=off, ids=ids, coef=coef)
    params = {"seed": 31, "sweeps": 40, "restarts": 6, "beta_start": 0.05, "beta_stop": 3.0,
              "rng_mode": mode}
    s = q.Solver(g, SA, {"params": params}).init().run()
    r = O.run(o, "sa", seed=31, step_limit=40, restarts=6, sched=("linear", 0.05, 3.0),
              rng_mode=mode, threads=4)
    _same(s.replicas(), r)
    # the same walkers with the walker state in global memory
    s2 = q.Solver(g, SA, {"params": dict(params, smem_state=False)}).init().run()
    _same(s2.replicas(), r)


@pytest.mark.parametrize("name", ["hub_pubo", "dense_block", "long_terms", "extreme_pubo"])
def test_edge_pt(name):
    kind, gen = CASES[name]
    off, ids, coef = gen()
    g = q.Model(kind, off=off, ids=ids, coef=coef)
    o = O.Model(kind, off=off, ids=ids, coef=coef)
    temps = [0.2, 0.5, 1.0, 2.0, 4.0]
    s = q.Solver(g, PT, {"params": {"seed": 8, "sweeps": 25, "all_betas": temps}}).init().run()
    r = O.run(o, "pt", seed=8, step_limit=25, sched=("list", 0, 0), sched_values=temps, threads=4)
    _same(s.replicas(), r)


def test_dimacs_model_solves_like_term_lists():
    from qiotoolkit_gb300 import instances as I
    off, ids, coef = I.weighted_maxsat(60, seed=71)
    lines = [f"p wcnf 60 {len(coef)}"]
    for k in range(len(coef)):
        lits = " ".join(str(int(x)) for x in ids[off[k]:off[k + 1]])
        lines.append(f"{float(coef[k])!r} {lits} 0")
    text = "\n".join(lines) + "\n"
    d = q.Model.from_dimacs(text)
    g = q.Model("maxsat", off=off, ids=ids, coef=coef)
    o = O.Model("maxsat", off=off, ids=ids, coef=coef)
    params = {"seed": 5, "sweeps": 50, "restarts": 4, "beta_start": 0.1, "beta_stop": 2.0,
              "maxsat_full_sweep": True}
    rd = q.Solver(d, SA, {"params": params}).init().run()
    rg = q.Solver(g, SA, {"params": params}).init().run()
    assert rd.result()["solutions"] == rg.result()["solutions"]
    r = O.run(o, "sa", seed=5, step_limit=50, restarts=4, sched=("linear", 0.1, 2.0), threads=4,
              full_maxsat_sweep=True)
    _same(rd.replicas(), r)


def test_memory_saving_feature_gives_the_same_result():
    """enabled_features [3] selects the reference's memory-saving models
    (IsingCompact / PuboCompact): here the counter-free flavours; the result
    is the same as with the cached models."""
    from qiotoolkit_gb300 import instances as I
    for kind, (off, ids, coef) in (("ising", I.er_ising(150, 400, seed=81)),
                                   ("pubo", I.random_pubo(120, 360, seed=82))):
        doc = {"cost_function": {"type": kind, "version": "1.0",
                                 "terms": [{"c": float(coef[k]), "ids": [int(x) for x in ids[off[k]:off[k + 1]]]}
                                           for k in range(len(coef))]}}
        p = {"seed": 4, "sweeps": 60, "restarts": 4, "beta_start": 0.1, "beta_stop": 2.0}
        a = q.run_json(doc, {"params": p}, SA)
        b = q.run_json(doc, {"params": dict(p, enabled_features=[3])}, SA)
        assert a["solutions"]["cost"] == b["solutions"]["cost"]
        assert a["solutions"]["configuration"] == b["solutions"]["configuration"]


def test_compact_model_single_term_pins():
    """IsingCompact SingleTerm (model/test/ising_test.cc:572-611): seven
    one-spin terms; all spins down costs -7, each flip costs +2."""
    for kind in ("ising", "ising_plain"):
        m = q.Model(kind, [(1.0, [i]) for i in range(7)])
        st = np.ones((1, 7), np.uint8)
        assert m.calculate_cost(st)[0] == -7
        for i in range(7):
            assert m.calculate_cost_difference(st, [i])[0] == 2
            st = m.apply_transition(st, [i])
            assert m.calculate_cost(st)[0] == (i + 1) * 2 - 7
        for i in range(7):
            assert m.calculate_cost_difference(st, [i])[0] == -2
            st = m.apply_transition(st, [i])
            assert m.calculate_cost(st)[0] == 7 - 2 * (i + 1)


def test_proto_folders_cost_like_the_oracle(golden, tmp_path):
    """Models read from the reference's protobuf folders (data/*_pb) price
    states exactly as the oracle's model of the terms their writers put in."""
    g = golden("proto_pins.json")
    rng = np.random.default_rng(12)
    for name, exp in g["expected"].items():
        if exp["type"] == "softspin":
            continue
        d = tmp_path / name
        d.mkdir()
        for k, h in enumerate(g["folders"][name]):
            (d / f"{name}_{k}.pb").write_bytes(bytes.fromhex(h))
        m = q.Model.from_proto_folder(str(d))
        o = O.Model(exp["type"], [(c, ids) for c, ids in exp["terms"]])
        states = rng.integers(0, 2, (64, m.n_vars), dtype=np.uint8)
        got = m.calculate_cost(states)
        want = np.array([o.cost(s) for s in states])
        np.testing.assert_array_equal(got, want, err_msg=name)
        dg = m.calculate_cost_difference(states, 1)
        dw = np.array([o.cost_difference(s, 1) for s in states])
        np.testing.assert_array_equal(dg, dw, err_msg=name)
