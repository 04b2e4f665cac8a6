"""Allocation-free cost entry point (qio_states_cost_noalloc) on the GPU.

The call evaluates device-resident states with its scratch in a fixed array
of the library; its results must equal qio_states_cost's exactly (tolerance
0: both run the same ordered sums), on two calls in a row that reuse the
shared scratch.  The file name keeps it last in collection order; it also
passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

import qiotoolkit_gb300 as q
from qiotoolkit_gb300 import instances as I
from qiotoolkit_gb300._lib import QioError, check, load

torch = pytest.importorskip("torch")

MAX_WORDS = 1 << 18  # scratch words of the allocation-free call (1 MiB)


def _noalloc(model, d_states, d_out):
    stream = torch.cuda.current_stream().cuda_stream
    check(load().qio_states_cost_noalloc(model._h, d_states.shape[0],
                                         ctypes.c_void_p(d_states.data_ptr()),
                                         ctypes.c_void_p(d_out.data_ptr()),
                                         ctypes.c_void_p(stream)))
    torch.cuda.synchronize()
    return d_out.cpu().numpy()


def _models():
    off, ids, coef = I.random_pubo(700, 3000, seed=5)
    yield "pubo", q.Model("pubo", off=off, ids=ids, coef=coef)
    off, ids, coef = I.er_ising(333, 900, seed=6)
    yield "ising", q.Model("ising", off=off, ids=ids, coef=coef)
    off, ids, coef = I.random_pubo(257, 800, seed=7, integer=True)
    yield "pubo_int", q.Model("pubo", off=off, ids=ids, coef=coef)
    off, ids, coef = I.er_ising(200, 600, seed=9)
    yield "ising_plain", q.Model("ising_plain", off=off, ids=ids, coef=coef)
    off, ids, coef = I.random_pubo(220, 700, seed=10)
    yield "pubo_plain", q.Model("pubo_plain", off=off, ids=ids, coef=coef)
    off, ids, coef = I.weighted_maxsat(150, seed=12)
    yield "maxsat", q.Model("maxsat", off=off, ids=ids, coef=coef)


NAMES = ["pubo", "ising", "pubo_int", "ising_plain", "pubo_plain", "maxsat"]


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_noalloc_cost_equals_states_cost(name):
    model = dict(_models())[name]
    rng = np.random.default_rng(11)
    n_vars = model.n_vars
    for n in (37, 300):  # two calls in a row through the shared scratch
        states = rng.integers(0, 2, size=(n, n_vars), dtype=np.uint8)
        ref = model.calculate_cost(states)  # existing entry point (host buffers)
        d_states = torch.from_numpy(states).cuda()
        d_out = torch.full((n,), float("nan"), dtype=torch.float64, device="cuda")
        got = _noalloc(model, d_states, d_out)
        np.testing.assert_array_equal(got, ref)


@pytest.mark.gpu
def test_noalloc_rejects_oversized_batches():
    off, ids, coef = I.er_ising(4096, 8000, seed=8)
    model = q.Model("ising", off=off, ids=ids, coef=coef)
    model.calculate_cost(np.zeros((1, model.n_vars), np.uint8))
    n = MAX_WORDS // ((model.n_vars + 31) // 32) + 1
    d_states = torch.zeros((n, model.n_vars), dtype=torch.uint8, device="cuda")
    d_out = torch.zeros(n, dtype=torch.float64, device="cuda")
    with pytest.raises(QioError, match="scratch words; the maximum is 262144"):
        _noalloc(model, d_states, d_out)


@pytest.mark.gpu
def test_noalloc_refuses_a_model_not_yet_on_the_device():
    off, ids, coef = I.er_ising(64, 150, seed=13)
    model = q.Model("ising", off=off, ids=ids, coef=coef)  # never run on the GPU
    d_states = torch.zeros((2, model.n_vars), dtype=torch.uint8, device="cuda")
    d_out = torch.zeros(2, dtype=torch.float64, device="cuda")
    with pytest.raises(QioError, match="not on the device yet"):
        _noalloc(model, d_states, d_out)


@pytest.mark.gpu
def test_noalloc_refuses_host_buffers():
    off, ids, coef = I.er_ising(64, 150, seed=14)
    model = q.Model("ising", off=off, ids=ids, coef=coef)
    model.calculate_cost(np.zeros((1, model.n_vars), np.uint8))
    states = np.zeros((2, model.n_vars), np.uint8)
    out = np.zeros(2)
    stream = torch.cuda.current_stream().cuda_stream
    with pytest.raises(QioError, match="must be device pointers"):
        check(load().qio_states_cost_noalloc(model._h, 2,
                                             ctypes.c_void_p(states.ctypes.data),
                                             ctypes.c_void_p(out.ctypes.data),
                                             ctypes.c_void_p(stream)))
