"""Tabu search, host side: parameters, and the oracle's tabu walker against a
pure-Python restatement of markov/tabu_walker.h:60-129 (with the hill
climber of markov/hill_climbing_walker.h:17-20) on small models.

The oracle's walkers start from its own random states (step_limit 0 returns
them); the restatement runs the deterministic sweeps from there.
"""
import numpy as np
import pytest

import qiotoolkit_gb300 as q
from qiotoolkit_gb300 import instances as I
from oracle import oracle as O

TABU = "tabu.qiotoolkit"


@pytest.mark.parametrize("params,msg", [
    ({"tabu_tenure": -1}, "tabu_tenure"),
    ({"restarts": 0}, "restarts"),
])
def test_parameter_errors(params, msg):
    m = q.Model("ising", [(1.0, [0, 1]), (-2.0, [1, 2])])
    with pytest.raises(q.QioError, match=msg):
        q.Solver(m, TABU, {"params": dict({"seed": 1}, **params)})


def test_maxsat_accepted():
    """MaxSat sweeps get_sweep_size() variables: 1 unless the full sweep is
    asked for (markov/model.h:169)."""
    m = q.Model("maxsat", [(1.0, [1, 2]), (2.0, [-1, 3])])
    q.Solver(m, TABU, {"params": {"seed": 1, "sweeps": 5}}).close()
    q.Solver(m, TABU, {"params": {"seed": 1, "sweeps": 5, "maxsat_full_sweep": True}}).close()


def test_defaults_accepted():
    m = q.Model("pubo", [(1.0, [0, 1]), (-2.0, [1, 2])])
    q.Solver(m, TABU, {"params": {"seed": 1, "sweeps": 5}}).close()


class PyTabu:
    """One tabu walker, restated with plain loops."""

    def __init__(self, om, spins, tenure):
        self.m = om
        self.s = np.array(spins, np.uint8)
        self.cost = om.cost(self.s)
        self.low = self.cost
        self.low_s = self.s.copy()
        self.tabu = [0] * len(spins)
        self.it = self.incomplete = 0
        self.tenure = tenure
        self.local = False
        self.att = self.acc = 0

    def diff(self, s, v):
        return self.m.cost_difference(s, v)

    def local_sweep(self):
        prev = self.hl
        for v in range(len(self.s)):
            d = self.diff(self.h, v)
            self.att += 1
            if d <= 0:
                self.h[v] ^= 1
                self.acc += 1
                self.hc += d
                if self.hc < self.hl:
                    self.hl = self.hc
                    self.hl_s = self.h.copy()
        if self.hl < prev:
            self.low = self.hl
            self.low_s = self.hl_s.copy()
        else:
            self.local = False

    def sweep(self):
        if self.local:
            self.local_sweep()
            return
        n = len(self.s)
        best = None
        for i in range(n):
            d = self.diff(self.s, i)
            self.att += 1
            if self.cost + d < self.low:
                self.s[i] ^= 1
                self.acc += 1
                self.cost += d
                self.low = self.cost
                self.low_s = self.s.copy()
                self.tabu[i] = self.it + self.tenure
                self.local = True
                self.h = self.s.copy()
                self.hc = self.m.cost(self.h)
                self.hl = self.hc
                self.hl_s = self.h.copy()
                self.incomplete += i
                if self.incomplete < n:
                    self.local_sweep()
                else:
                    self.incomplete -= n
                break
            if self.tabu[i] >= self.it:
                continue
            if best is None or d < best[0]:
                best = (d, i)
        else:
            if best is not None:
                d, i = best
                self.s[i] ^= 1
                self.cost += d
                if self.cost < self.low:
                    self.low = self.cost
                    self.low_s = self.s.copy()
                self.tabu[i] = self.it + self.tenure
        self.it += 1


@pytest.mark.parametrize("kind,gen", [
    ("ising", lambda: I.er_ising(40, 90, seed=8)),
    ("ising", lambda: I.cubic_pm_j(3, seed=9)),
    ("pubo", lambda: I.random_pubo(30, 80, seed=10)),
])
@pytest.mark.parametrize("tenure", [0, 3])
def test_oracle_matches_restatement(kind, gen, tenure):
    off, ids, coef = gen()
    om = O.Model(kind, off=off, ids=ids, coef=coef)
    start = O.run(om, "tabu", seed=6, step_limit=0, restarts=3, tabu_tenure=tenure)
    steps = 25
    r = O.run(om, "tabu", seed=6, step_limit=steps, restarts=3, tabu_tenure=tenure)
    for w in range(3):
        t = PyTabu(om, start.states[w], tenure)
        for _ in range(steps):
            t.sweep()
        assert t.cost == r.cost[w]
        assert t.low == r.lowest[w]
        assert (t.att, t.acc) == (r.attempts[w], r.accepts[w])
        np.testing.assert_array_equal(t.s, r.states[w])
        np.testing.assert_array_equal(t.low_s, r.lowest_states[w])


def test_parameter_free_tenures_like_the_reference():
    """determine_all_tenures_ (solver/tabu_parameter_free.h:86-124) as the
    oracle restates it: the optimal min(20, N/4), its half above 10, then
    steps below N."""
    assert O.tabu_tenures(10, 1000) == [20, 10, 50, 80, 110, 140, 170, 200, 230, 260]
    assert O.tabu_tenures(7, 30) == [7, 8, 9, 10, 11, 12, 13]
    assert O.tabu_tenures(5, 3) == [0, 1, 2, 0, 1]


def test_parameter_free_configuration_errors():
    m = q.Model("ising", [(1.0, [0, 1]), (-2.0, [1, 2])])
    pf = "tabu-parameterfree.qiotoolkit"
    with pytest.raises(q.QioError, match="min_num_restarts"):
        q.Solver(m, pf, {"params": {"seed": 1, "min_num_restarts": 0}})
    with pytest.raises(q.QioError, match="rng_mode"):
        q.Solver(m, pf, {"params": {"seed": 1, "rng_mode": "counter"}})
    q.Solver(m, pf, {"params": {"seed": 1}}).close()
