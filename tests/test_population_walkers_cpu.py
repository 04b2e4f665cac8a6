"""Substochastic and quantum Monte Carlo: the oracle's restatements against
independent pure-Python ones on small models (counter streams, whose draws
are positional), so the C oracle that the device is checked against is
itself checked line by line.

SSMC follows solver/substochastic_monte_carlo.h:67-169 (walker steps,
population statistics, resampling with utils::RandomSelector from
utils/random_selector.cc on the master PCG stream, Population::resample
layout); QMC follows solver/quantum_monte_carlo.h:128-175 with
markov/cluster_walker.h and markov/quantum_walker.h.  Initial states come
from the oracle itself (step_limit 0); everything after is restated here.
"""
import math

import numpy as np
import pytest

from qiotoolkit_gb300 import instances as I
from oracle import oracle as O

M64 = (1 << 64) - 1
MULT, INC = 6364136223846793005, 1442695040888963407


class Pcg32:
    """pcg32 (setseq default increment), seeded as utils::PCG."""

    def __init__(self, seed):
        self.state = ((seed + INC) * MULT + INC) & M64

    def next(self):
        old = self.state
        self.state = (old * MULT + INC) & M64
        xs = (((old >> 18) ^ old) >> 27) & 0xFFFFFFFF
        rot = old >> 59
        return ((xs >> rot) | (xs << ((32 - rot) & 31))) & 0xFFFFFFFF

    def uniform(self):
        # libstdc++ generate_canonical<double, 53> over two 32-bit outputs
        a, b = self.next(), self.next()
        u = (float(a) + float(b) * 4294967296.0) * 2.0 ** -64
        return u if u < 1.0 else 0.99999999999999988898


def cuni(key, ctr):
    return float(O.counter_draw(key, ctr) >> 11) * 2.0 ** -53


class Selector:
    """utils::RandomSelector: cumulative weights in a Fenwick-style array."""

    def __init__(self):
        self.ids, self.w, self.total = [], [0.0, 0.0], 0.0

    def cum(self, pos):
        p, w, k = 0, 0.0, len(self.w) - 1
        while k > 0:
            if pos & k:
                p |= k
                w += self.w[p]
            k >>= 1
        return w

    def get(self, pos):
        return self.cum(pos + 1) - self.cum(pos)

    def add(self, pos, wt):
        k = 1
        while k < len(self.w):
            if pos & k:
                pos ^= k
            else:
                self.w[pos + k] += wt
            k <<= 1

    def insert(self, i, wt):
        pos = len(self.ids)
        self.ids.append(i)
        self.total += wt
        if pos + 1 >= len(self.w):
            tot = self.w[-1]
            self.w = self.w + [0.0] * (len(self.w) - 1)
            self.w[-1] = tot
        self.add(pos, wt)

    def select_and_remove(self, u):
        if len(self.ids) == 1:
            pos = 0
        else:
            wt, pos, k = u * self.total, 0, len(self.w) - 1
            while k > 0:
                if wt >= self.w[pos + k]:
                    pos += k
                    wt -= self.w[pos]
                k >>= 1
            pos = min(pos, len(self.ids) - 1)
        i = self.ids[pos]
        self.ids[pos] = self.ids[-1]
        self.ids.pop()
        before, after = self.get(pos), self.get(len(self.ids))
        self.total -= before
        self.add(pos, after - before)
        self.add(len(self.ids), -after)
        return i


def linear(a, b, stop):
    def f(x):
        p = min(1.0, max(0.0, x / stop))
        return a + p * (b - a)
    return f


@pytest.mark.parametrize("kind,gen", [
    ("ising", lambda: I.er_ising(40, 100, seed=21)),
    ("pubo", lambda: I.random_pubo(30, 90, seed=22)),
    ("maxsat", lambda: I.weighted_maxsat(30, seed=25)),
])
def test_ssmc_oracle_matches_restatement(kind, gen):
    off, ids, coef = gen()
    m = O.Model(kind, off=off, ids=ids, coef=coef)
    seed, R, T, spw, steps = 17, 23, 4, 3, 30
    kw = dict(seed=seed, population=R, pa_threads=T, steps_per_walker=spw, rng_mode="counter",
              sched=("linear", 1.0, 0.0), sched2=("linear", 0.0, 5.0))
    start = O.run(m, "ssmc", step_limit=0, **kw)
    ref = O.run(m, "ssmc", step_limit=steps, **kw)
    n = m.n_vars
    master = Pcg32(seed)
    for _ in range(T):
        master.next()  # rngs_[t] = rng_->fork()
    alpha, beta = linear(1.0, 0.0, steps), linear(0.0, 5.0, steps)
    pop = [{"s": np.array(start.states[j], np.uint8), "c": m.cost(start.states[j])} for j in range(R)]
    for w in pop:
        w["low"], w["ls"], w["att"] = w["c"], w["s"].copy(), 0
    best = (pop[0]["c"], pop[0]["s"].copy())
    for step in range(steps):
        p_step = alpha(step) / spw
        for j, w in enumerate(pop):
            key = O.counter_key(seed, j)
            for k in range(spw):
                c = step * spw + k
                if cuni(key, 2 * c) < p_step:
                    v = int(cuni(key, 2 * c + 1) * n)
                    d = m.cost_difference(w["s"], v)
                    w["s"][v] ^= 1
                    w["c"] += d
                    w["att"] += 1
                    if w["c"] < w["low"]:
                        w["low"], w["ls"] = w["c"], w["s"].copy()
        mn = mx = pop[0]["c"]
        for w in pop:
            mn, mx = min(mn, w["c"]), max(mx, w["c"])
            if w["low"] < best[0]:
                best = (w["low"], w["ls"].copy())
        b = beta(step)
        if mx - mn > 0:
            wts = [math.exp(b * (mx - w["c"]) / (mx - mn)) for w in pop]
            total = 0.0
            for x in wts:
                total += x
            count, got, sel = [], 0, Selector()
            for i, x in enumerate(wts):
                rel = float(R) * x / total
                iw = math.floor(rel)
                count.append(iw)
                got += iw
                sel.insert(i, rel - iw)
            while got < R:
                count[sel.select_and_remove(master.uniform())] += 1
                got += 1
            pop = [{key_: (val.copy() if isinstance(val, np.ndarray) else val)
                    for key_, val in pop[i].items()} for i in range(R) for _ in range(count[i])]
    assert [w["c"] for w in pop] == list(ref.cost)
    assert [w["low"] for w in pop] == list(ref.lowest)
    assert [w["att"] for w in pop] == list(ref.attempts)
    np.testing.assert_array_equal(np.array([w["s"] for w in pop]), ref.states)
    assert best[0] + 0.0 == ref.best_cost - 0.0


@pytest.mark.parametrize("kind,gen,full", [
    ("ising", lambda: I.er_ising(30, 80, seed=23), False),
    ("pubo", lambda: I.random_pubo(25, 70, seed=24), False),
    ("maxsat", lambda: I.weighted_maxsat(25, seed=26), False),
    ("maxsat", lambda: I.weighted_maxsat(25, seed=26), True),
])
def test_qmc_oracle_matches_restatement(kind, gen, full):
    off, ids, coef = gen()
    m = O.Model(kind, off=off, ids=ids, coef=coef)
    seed, R, P, steps = 9, 3, 6, 12
    kw = dict(seed=seed, restarts=R, trotter_number=P, rng_mode="counter",
              sched=("linear", 0.5, 3.0), sched2=("linear", 0.2, 2.0), full_maxsat_sweep=full)
    start = O.run(m, "qmc", step_limit=0, **kw)
    ref = O.run(m, "qmc", step_limit=steps, **kw)
    n = m.n_vars
    # get_sweep_size(): 1 for MaxSat unless the full sweep is asked for
    sw = 1 if kind == "maxsat" and not full else n
    stop = max(1, steps - 1)
    bsch, fsch = linear(0.5, 3.0, stop), linear(0.2, 2.0, stop)
    S = [np.array(start.states[i], np.uint8) for i in range(R * P)]
    cost = [m.cost(s) for s in S]
    acc_n = [0] * (R * P)
    low, low_s = [], []
    for r in range(R):
        k = min(range(P), key=lambda q: (cost[r * P + q], q))
        low.append(cost[r * P + k])
        low_s.append(S[r * P + k].copy())
    for step in range(steps):
        b, g = bsch(step), fsch(step)
        be, bp = b / P, 1 - math.tanh(g * b / P)
        for r in range(R):
            for v in range(sw):
                c = 2 * (step * n + v)
                diff, bond = [], []
                for k in range(P):
                    i = r * P + k
                    diff.append(m.cost_difference(S[i], v))
                    bd = False
                    if k > 0 and S[i - 1][v] == S[i][v]:
                        bd = cuni(O.counter_key(seed, i), c) < bp
                    bond.append(bd)
                acc = [False] * P
                for k in range(P):
                    if bond[k]:
                        continue
                    tot, e = diff[k], k + 1
                    while e < P and bond[e]:
                        tot += diff[e]
                        e += 1
                    ok = True
                    if not tot < 10e-12:
                        ok = cuni(O.counter_key(seed, r * P + k), c + 1) < math.exp(-be * tot)
                    for q in range(k, e):
                        acc[q] = ok
                for k in range(P):
                    if acc[k]:
                        i = r * P + k
                        S[i][v] ^= 1
                        cost[i] += diff[k]
                        acc_n[i] += 1
            k = min(range(P), key=lambda q: (cost[r * P + q], q))
            if cost[r * P + k] < low[r]:
                low[r], low_s[r] = cost[r * P + k], S[r * P + k].copy()
    assert cost == list(ref.cost)
    assert acc_n == list(ref.accepts)
    assert [low[i // P] for i in range(R * P)] == list(ref.lowest)
    np.testing.assert_array_equal(np.array(S), ref.states)
