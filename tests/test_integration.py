"""The C ABI as a C++ caller sees it: tests/integration/binding.cc, written as
the INTEGRATION.md bindings, is compiled against include/qio_gb300.h and
linked with the built libqio_gb300.so.  The host-side paths (model
construction, properties, error statuses and messages) run anywhere; the
solve runs on the GPU."""
import os
import shutil
import subprocess

import pytest

import qiotoolkit_gb300 as q

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def binary(tmp_path_factory):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no C++ compiler")
    q.load()
    lib = q.lib_path()
    out = str(tmp_path_factory.mktemp("binding") / "binding")
    cmd = [cxx, "-std=c++17", "-O1", os.path.join(ROOT, "tests", "integration", "binding.cc"),
           "-I", os.path.join(ROOT, "include"), lib, "-Wl,-rpath," + os.path.dirname(lib), "-o", out]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return out


def test_binding_host_paths(binary):
    r = subprocess.run([binary], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "OK (0 failures)" in r.stdout


@pytest.mark.gpu
def test_binding_solve(binary):
    r = subprocess.run([binary, "--gpu"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "OK (0 failures)" in r.stdout
