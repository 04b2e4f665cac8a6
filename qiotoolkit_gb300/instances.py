"""Seeded synthetic instances in the reference's input format.

No public benchmark or dataset belongs to this path; these generators follow
the workload shapes and value distributions of the five benchmark
configurations (sparse Erdos-Renyi Ising, random PUBO, 3D and 2D +-J lattices,
mixed serving requests including weighted random MaxSAT).  Each returns
(offsets int64, ids int32, coefficients float64) in term order, ready for
Model(kind, off=..., ids=..., coef=...), and `to_json` renders the reference's
{"cost_function": ...} document.
"""
from __future__ import annotations

import json

import numpy as np


def _pack(ids_list, coef):
    off = np.zeros(len(ids_list) + 1, np.int64)
    off[1:] = np.cumsum([len(t) for t in ids_list])
    ids = np.concatenate([np.asarray(t, np.int32) for t in ids_list]) if ids_list else \
        np.zeros(0, np.int32)
    return off, ids.astype(np.int32), np.asarray(coef, np.float64)


def er_ising(n=1000, n_edges=3000, seed=0, field_range=0.5):
    """N spins, n_edges distinct Erdos-Renyi couplings with weights in {-1,+1}
    and one field per spin uniform in [-field_range, field_range].  Fields
    come first so that first-appearance order equals spin id."""
    rng = np.random.default_rng(seed)
    edges = set()
    while len(edges) < n_edges:
        a, b = rng.integers(0, n, 2)
        if a != b:
            edges.add((min(a, b), max(a, b)))
    edges = sorted(edges)
    ids = [[i] for i in range(n)] + [[a, b] for a, b in edges]
    coef = list(rng.uniform(-field_range, field_range, n)) + \
        list(rng.choice([-1.0, 1.0], len(edges)))
    return _pack(ids, coef)


def random_pubo(n=4096, n_terms=20000, seed=1, orders=(1, 2, 3, 4),
                probs=(0.1, 0.5, 0.3, 0.1), integer=False):
    """PUBO terms whose order is drawn from `orders` with `probs`, variables
    uniform without replacement, weights N(0,1) (or +-1..3 integers)."""
    rng = np.random.default_rng(seed)
    ords = rng.choice(orders, size=n_terms, p=probs)
    ids = [sorted(rng.choice(n, size=o, replace=False).tolist()) for o in ords]
    coef = rng.integers(-3, 4, n_terms).astype(float) if integer else rng.standard_normal(n_terms)
    return _pack(ids, coef)


def cubic_pm_j(L, seed=2):
    """3D periodic cubic lattice, L^3 spins, couplings +-1 at p = 0.5."""
    rng = np.random.default_rng(seed)
    idx = np.arange(L ** 3).reshape(L, L, L)
    pairs = []
    for axis in range(3):
        nb = np.roll(idx, -1, axis=axis)
        pairs.append(np.stack([idx.ravel(), nb.ravel()], 1))
    pairs = np.concatenate(pairs)
    if L == 2:
        pairs = np.unique(np.sort(pairs, 1), axis=0)
    order = np.lexsort((pairs[:, 1], pairs[:, 0]))
    pairs = pairs[order]
    coef = rng.choice([-1.0, 1.0], len(pairs))
    off = np.arange(0, 2 * len(pairs) + 1, 2, dtype=np.int64)
    return off, pairs.astype(np.int32).ravel(), coef


def square_pm_j(L=256, seed=3):
    """2D periodic square lattice, L^2 spins, couplings +-1 at p = 0.5."""
    rng = np.random.default_rng(seed)
    idx = np.arange(L * L).reshape(L, L)
    pairs = np.concatenate([np.stack([idx.ravel(), np.roll(idx, -1, a).ravel()], 1)
                            for a in range(2)])
    order = np.lexsort((pairs[:, 1], pairs[:, 0]))
    pairs = pairs[order]
    coef = rng.choice([-1.0, 1.0], len(pairs))
    off = np.arange(0, 2 * len(pairs) + 1, 2, dtype=np.int64)
    return off, pairs.astype(np.int32).ravel(), coef


def weighted_maxsat(n=1000, ratio=4.2, k=3, seed=4, wmin=1.0, wmax=10.0, integer=False):
    """Weighted random k-SAT: round(ratio*n) clauses of k distinct variables
    (names 1..n), random signs, weights uniform in [wmin, wmax]."""
    rng = np.random.default_rng(seed)
    m = int(round(ratio * n))
    ids = []
    for _ in range(m):
        vs = rng.choice(n, size=k, replace=False) + 1
        sg = rng.choice([-1, 1], size=k)
        ids.append((vs * sg).tolist())
    coef = rng.integers(int(wmin), int(wmax) + 1, m).astype(float) if integer else \
        rng.uniform(wmin, wmax, m)
    return _pack(ids, coef)


def to_json(kind, off, ids, coef) -> str:
    terms = [{"c": float(coef[t]), "ids": [int(x) for x in ids[off[t]:off[t + 1]]]}
             for t in range(len(coef))]
    return json.dumps({"cost_function": {"type": kind, "version": "1.0", "terms": terms}})


def er_ising_gauss(n, mean_degree, seed=0):
    """Sparse Erdos-Renyi Ising model: round(n * mean_degree / 2) distinct
    couplings with N(0,1) weights rounded to FP32 (no fields)."""
    rng = np.random.default_rng(seed)
    m = int(round(n * mean_degree / 2))
    edges = set()
    while len(edges) < m:
        a = rng.integers(0, n, 2 * (m - len(edges)) + 8)
        b = rng.integers(0, n, a.size)
        for x, y in zip(a.tolist(), b.tolist()):
            if x != y:
                edges.add((min(x, y), max(x, y)))
                if len(edges) == m:
                    break
    edges = sorted(edges)
    ids = [[a, b] for a, b in edges]
    coef = rng.standard_normal(m).astype(np.float32).astype(np.float64)
    return _pack(ids, coef)

