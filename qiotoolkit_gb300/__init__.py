"""GB300-native Metropolis hot path of QIOToolkit.

Simulated annealing, parallel tempering and population annealing over Ising,
PUBO and weighted MaxSAT cost functions, run by sm_103a kernels behind the C
ABI in include/qio_gb300.h (libqio_gb300.so).  This package is the Python
mirror of the reference's model/solver interface over that ABI.
"""
from ._lib import QioError, SYMBOLS, lib_path, load  # noqa: F401
from .api import KINDS, TARGETS, Batch, Model, Server, Solver, bayes_recommend, flatten_terms, run_json  # noqa: F401

__all__ = ["Model", "Solver", "Batch", "Server", "run_json", "QioError", "load", "lib_path", "KINDS",
           "TARGETS", "flatten_terms", "SYMBOLS", "bayes_recommend"]
