"""The oracle against the reference's own known-answer tests (CPU only)."""
import math

import numpy as np
import pytest

from oracle import oracle as O


def pct(xs):
    return [int(x * 100) for x in xs]


def test_pcg_sequences(golden):
    g = golden("rng_pins.json")
    assert pct(O.pcg_uniform(None, 3)) == g["pcg_default"]
    assert pct(O.pcg_uniform(42, 3)) == g["pcg_42"]
    f = O.pcg_fork_uniform(42, 3, 12)
    for k in range(4):
        assert pct(f[:, k]) == g["pcg_42_fork"][k]


def test_twister_sequences(golden):
    g = golden("rng_pins.json")
    assert pct(O.twister_uniform(None, 3)) == g["twister_default"]
    assert pct(O.twister_uniform(42, 3)) == g["twister_42"]


def test_pt_toy_observables_seed42(golden):
    """Exact per-replica PT observables at seed 42 (6 decimals)."""
    g = golden("pt_toy_pin.json")
    t = g["temperatures"]
    temps = [t["initial"] + (i / (t["count"] - 1)) * (t["final"] - t["initial"])
             for i in range(t["count"])]
    obs, best = O.pt_toy(g["seed"], g["step_limit"], temps)
    for row, exp in zip(obs, g["observables"]):
        for v, e in zip(row, exp):
            if e is None:
                assert math.isnan(v)
            else:
                assert "%f" % v == "%f" % e
    assert best < 1


def test_uniform_ln_table():
    t = O.uniform_ln()
    assert np.isneginf(t[:, 0]).all()
    for row in range(4):
        for i in (1, 17, 255):
            assert t[row, i] == math.log(i / 256.0 ** (row + 1))


def test_metropolis_accept_rules():
    # downhill accepts without drawing
    assert O.metropolis_accept(-1.0, 1.0, []) == (True, 0)
    assert O.metropolis_accept(0.0, 1.0, []) == (True, 0)
    # four zero buckets in a row accept
    assert O.metropolis_accept(5.0, 1.0, [0, 256, 512, 0]) == (True, 4)
    # bucket 255 of row 0 at distance 0: value = ln(254/256) < -dE*beta ?
    acc, used = O.metropolis_accept(1e-9, 1.0, [255])
    assert used == 1 and acc
    acc, used = O.metropolis_accept(10.0, 1.0, [255])
    assert used == 1 and not acc
    # beta = +inf rejects every uphill move
    acc, _ = O.metropolis_accept(1.0, float("inf"), [0xFFFFFFFF])
    assert not acc


def _ring(kind, golden, name):
    pins = {p["name"]: p for p in golden("model_pins.json")}
    p = pins[name]
    return O.Model(kind, p["terms"]), p


@pytest.mark.parametrize("kind,name", [("ising", "ising_ring10"), ("ising_plain", "ising_ring10"),
                                       ("pubo", "pubo_ring10"), ("pubo_plain", "pubo_ring10")])
def test_single_updates(kind, name, golden):
    m, p = _ring(kind, golden, name)
    su = p["single_updates"]
    s = np.zeros(10, np.uint8)
    assert m.cost(s) == su["cost0"]
    assert m.cost_difference(s, 0) == su["diff0"]
    s[0] = 1
    assert m.cost(s) == su["cost1"]
    assert m.cost_difference(s, 0) == su["diff1"]
    s[0] = 0
    assert m.cost(s) == su["cost2"]
    tm = p["twister_min"]
    assert m.twister_min(tm["seed"], tm["iters"], tm["T"]) == tm["min"]


def test_const_terms_and_names(golden):
    pins = {p["name"]: p for p in golden("model_pins.json")}
    m = O.Model("ising", pins["ising_const"]["terms"])
    assert m.n_vars == 0 and m.const_cost == pins["ising_const"]["const_cost"]
    m = O.Model("pubo", pins["pubo_const"]["terms"])
    assert m.const_cost == pins["pubo_const"]["const_cost"]
    with pytest.raises(ValueError):
        O.Model("ising", pins["ising_dup"]["terms"])
    m = O.Model("pubo", pins["pubo_names"]["terms"])
    assert list(m.var_names()) == pins["pubo_names"]["var_names"]


def test_maxsat_costs_and_diffs(golden):
    p = {q["name"]: q for q in golden("model_pins.json")}["maxsat_small"]
    m = O.Model("maxsat", p["terms"])
    for bits, c in p["costs"].items():
        s = np.array([int(b) for b in bits], np.uint8)
        assert m.cost(s) == c
        assert [m.cost_difference(s, v) for v in range(2)] == p["diffs"][bits]


def _params(p):
    return dict(seed=p["seed"], step_limit=p["sweeps"])


@pytest.mark.parametrize("idx", range(63))
def test_solver_end_results(idx, golden):
    case = golden("solver_pins.json")["cases"][idx]
    p = case["params"]
    m = O.Model(case["kind"], case["terms"])
    if case["solver"] == "sa":
        r = O.run(m, "sa", seed=p["seed"], step_limit=p["sweeps"], restarts=p["restarts"],
                  sched=("linear", p["beta_start"], p["beta_stop"]), threads=4)
    elif case["solver"] == "pt":
        r = O.run(m, "pt", seed=p["seed"], step_limit=p["sweeps"],
                  sched=("list", 0, 0), sched_values=p["all_betas"], threads=4)
    elif case["solver"] == "ssmc":
        # params1.json leaves SSMC at its defaults: target population = thread
        # count, alpha 1 -> 0 and beta 0 -> 5 linear over the step limit
        # (solver/substochastic_monte_carlo.h:157-199)
        r = O.run(m, "ssmc", seed=p["seed"], step_limit=p["sweeps"], population=8, pa_threads=8,
                  sched=("linear", 1.0, 0.0), sched2=("linear", 0.0, 5.0))
    elif case["solver"] in ("sa_pf", "pt_pf"):
        # pf5s.json sets only a 5 s timeout: seed 0 and 8 restarts / betas
        # here; the restatements stop on the non-improvement rule.  A model
        # whose terms all fold into the constant has nothing to search.
        if m.n_vars == 0:
            class _E:
                best_cost = m.const_cost
                best_state = np.zeros(0, np.uint8)
            r = _E()
        else:
            terms = case["terms"]
            if case["solver"] == "sa_pf":
                res = O.sa_parameter_free(m, case["kind"], terms, seed=0, min_num_restarts=8)
            else:
                res = O.pt_parameter_free(m, case["kind"], terms, seed=0, min_num_betas=8)

            class _P:
                best_cost = res["best"]  # run results include the constant
                best_state = res["best_state"]
            r = _P()
    elif case["solver"] == "tabu_pf":
        # pf5s.json sets only a 5 s timeout: seed 0 and 8 restarts here; the
        # restatement stops on the non-improvement rule
        res = O.tabu_parameter_free(m, seed=0, min_num_restarts=8)

        class _R:
            best_cost = res["best"]
            best_state = res["best_state"]
        r = _R()
    elif case["solver"] in ("pa_pf", "ssmc_pf"):
        # pf5s.json sets only a 5 s timeout: seed 0 and 4 threads here.  The
        # Bayesian picks come from the library's own strategy, so the oracle
        # replays the search's four initial runs (the adapters' initial
        # parameter vectors on one master stream), which already reach the
        # reference's end results on these models; best by the 1e-11 rule.
        if m.n_vars == 0:
            class _E:
                best_cost = m.const_cost
                best_state = np.zeros(0, np.uint8)
            r = _E()
        else:
            if case["solver"] == "pa_pf":
                runs = O.pa_parameter_free_replay(m, case["kind"], case["terms"], seed=0, threads=4,
                                                  runs=[None] * 4)
            else:
                runs = O.ssmc_parameter_free_replay(m, seed=0, threads=4, runs=[None] * 4,
                                                    sweep_size=m.n_vars)
            best = None
            for _, _, low, st in runs:
                if best is None or best[0] - low > 10E-12:
                    best = (low, st)

            class _B:
                best_cost = best[0]
                best_state = best[1]
            r = _B()
    elif case["solver"] == "qmc":
        # params_qmc.json: beta_start defaults to beta_stop; the transverse
        # field runs linear low -> high (solver/quantum_monte_carlo.h:185-222)
        r = O.run(m, "qmc", seed=p["seed"], step_limit=p["sweeps"], restarts=p["restarts"],
                  trotter_number=p["trotter_number"],
                  sched=("linear", p["beta_stop"], p["beta_stop"]),
                  sched2=("linear", p["transverse_field_low"], p["transverse_field_high"]), threads=4)
    elif case["solver"] == "tabu":
        r = O.run(m, "tabu", seed=p["seed"], step_limit=p["sweeps"], restarts=p["restarts"],
                  tabu_tenure=p["tabu_tenure"], threads=4)
    else:
        # params1.json leaves PA at its defaults: population = thread count,
        # beta 0 -> 5 linear (solver/population_annealing.h:632-735)
        r = O.run(m, "pa", seed=p["seed"], step_limit=p["sweeps"], population=8,
                  pa_threads=8, sched=("linear", 0.0, 5.0), threads=4)
    exp = case["expected_cost"]
    if isinstance(exp, str):
        # EXPECT_LE(-12, cost): the reference only bounds this one from below
        assert r.best_cost >= float(exp[2:]) - 1e-9
    else:
        assert r.best_cost == exp
    names = list(m.var_names())
    for name, val in case["configuration"].items():
        v = r.best_state[names.index(int(name))]
        if case["kind"] == "ising":
            assert (-1 if v else 1) == val
        else:
            assert (0 if v else 1) == val


def test_all_solvers_three_spin(golden):
    p = {q["name"]: q for q in golden("model_pins.json")}["ising_3spin"]
    m = O.Model("ising", p["terms"])
    for solver in ("sa", "pt", "pa"):
        kw = dict(seed=p["seed"], step_limit=100)
        if solver == "sa":
            kw.update(restarts=4, sched=("linear", 0.0, 0.01))
        elif solver == "pt":
            kw.update(sched=("list", 0, 0), sched_values=[0.1, 0.5, 1, 2, 4])
        else:
            kw.update(population=4, pa_threads=4, sched=("linear", 0.0, 5.0))
        r = O.run(m, solver, **kw)
        assert r.best_cost == p["min"]


def test_planted_ground_energies(golden):
    """Quality pin: SA reaches the planted ground energy of the N=16 e2e
    instances shipped with the reference."""
    for inst in golden("planted.json")["instances"]:
        m = O.Model(inst["kind"], inst["terms"])
        r = O.run(m, "sa", seed=7, step_limit=200, restarts=16,
                  sched=("linear", 0.0, 3.0 / max(abs(c) for c, _ in inst["terms"])),
                  threads=4)
        assert r.best_cost == pytest.approx(inst["energy"], abs=1e-6)


def test_multinomial_exp_accuracy():
    """The resampling mode's own exp stays within 1 ulp of the C library's
    over the normal range (and underflows to 0 like it)."""
    import math
    xs = -np.concatenate([np.random.default_rng(0).uniform(0, 745, 4000),
                          np.random.default_rng(1).uniform(0, 1e-3, 1000), [0.0, 1e-300, 700.0]])
    worst = 0.0
    for x in xs:
        a, b = O.qexp(x), math.exp(x)
        if b > 2.2250738585072014e-308:
            worst = max(worst, abs(a - b) / math.ulp(b))
    assert worst <= 1.0
    assert O.qexp(0.0) == 1.0 and O.qexp(-800.0) == 0.0
