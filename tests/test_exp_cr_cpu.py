"""The correctly rounded exp that decides near-tie replica swaps
(qiotoolkit_gb300/csrc/exp_cr.cuh), compiled as host code: on random
arguments of the swap range and near rounding midpoints it equals exp(x)
rounded to nearest from 80-digit arithmetic (mpmath, from sympy)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROG = r'''
#include <cstdio>
#include "exp_cr.cuh"
int main() {
  double x;
  while (std::scanf("%la", &x) == 1) std::printf("%a\n", qio::dd::exp_cr(x));
}
'''


def test_exp_cr_is_correctly_rounded(tmp_path):
    mp = pytest.importorskip("mpmath")
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no C++ compiler")
    src = tmp_path / "t.cc"
    src.write_text(PROG)
    exe = str(tmp_path / "t")
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I",
                    os.path.join(ROOT, "qiotoolkit_gb300", "csrc"), str(src), "-o", exe], check=True)
    rng = np.random.default_rng(5)
    xs = list(rng.uniform(-700.0, 5.0, 3000)) + list(rng.uniform(-2.0, 0.0, 3000)) + [0.0, -1e-300, 1.0]
    out = subprocess.run([exe], input="\n".join(float(x).hex() for x in xs), capture_output=True,
                         text=True, check=True).stdout.split()
    mp.mp.dps = 80
    for x, y in zip(xs, out):
        assert float.fromhex(y) == float(mp.exp(mp.mpf(float(x)))), x
