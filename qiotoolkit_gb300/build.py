"""Compile libqio_gb300.so for sm_103a (nvcc, one -gencode, parallel TUs).

The library is built in-tree at qiotoolkit_gb300/_lib/libqio_gb300.so.  No
torch extension machinery is involved: the boundary is a C ABI.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "libqio_gb300.so")
SOURCES = ["kernels.cu", "sweep.cu", "fields.cu", "lanes.cu", "levels.cu", "pa_device.cu", "model_host.cc", "solvers.cc", "pa.cc", "bayes.cc", "serve.cc", "capi.cc", "json.cc", "dimacs.cc", "proto.cc"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _flags(src: str) -> list:
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "-I", os.path.join(HERE, "..", "include")]
    if src.endswith(".cu"):
        return common + ARCH + ["-lineinfo", "--extended-lambda", "-Xptxas", "-O3"]
    return common


def _compile(src: str, obj: str, verbose: bool) -> None:
    cmd = [nvcc(), "-c", os.path.join(CSRC, src), "-o", obj] + _flags(src)
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compiling {src} failed:\n{r.stdout}\n{r.stderr}")
    if r.stderr.strip() and verbose:
        print(r.stderr, file=sys.stderr)


def needs_build() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    for f in os.listdir(CSRC):
        if os.path.getmtime(os.path.join(CSRC, f)) > t:
            return True
    hdr = os.path.join(HERE, "..", "include", "qio_gb300.h")
    return os.path.getmtime(hdr) > t


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not needs_build():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    objs = []
    tag = str(os.getpid())  # builds running at once keep apart
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        futs = []
        for s in SOURCES:
            obj = os.path.join(OUT_DIR, os.path.splitext(s)[0] + "." + tag + ".o")
            objs.append(obj)
            futs.append(ex.submit(_compile, s, obj, verbose))
        for f in futs:
            f.result()
    tmp = LIB + "." + tag + ".tmp"
    cmd = [nvcc(), "-shared", "-o", tmp] + objs + ARCH + ["-Xcompiler", "-fPIC", "-lcudart_static",
                                                           "-lpthread", "-ldl", "-lrt"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"linking failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    for o in objs:
        os.remove(o)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
