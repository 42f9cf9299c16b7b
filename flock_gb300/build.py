"""Build recipe for the native library (no cmake): nvcc compiles the two
translation units in parallel for sm_103a and links libflock_gb300.so in
place, next to this file.  Also builds the `flock` command-line driver.

    python -m flock_gb300.build            # library + CLI
"""
from __future__ import annotations

import os
import platform
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libflock_gb300.so")
CLI = os.path.join(HERE, "flock")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
                  "-I", os.path.join(ROOT, "include")]


def _nvcc() -> str:
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    # objects built on another machine architecture are never reused
    marker = os.path.join(BUILD, ".arch")
    arch = platform.machine()
    if not os.path.exists(marker) or open(marker).read().strip() != arch:
        force = True
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(ROOT, "include", "flock.h"))
    units = [("kernels.cu", "kernels.o"), ("serve.cu", "serve.o"), ("host.cpp", "host.o"), ("cli.cpp", "cli.o")]
    jobs = []
    for src, obj in units:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, obj)
        if force or _stale(o, [s] + headers):
            lang = ["-x", "cu"] if src.endswith(".cu") else []
            jobs.append([nvcc] + NVFLAGS + lang + ["-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for f in [ex.submit(_run, j) for j in jobs]:
            f.result()
    objs = [os.path.join(BUILD, o) for o in ("kernels.o", "serve.o", "host.o")]
    if force or _stale(LIB, objs):
        tmp = LIB + ".tmp"
        _run([nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"])
        os.replace(tmp, LIB)
    cli_obj = os.path.join(BUILD, "cli.o")
    if force or _stale(CLI, [cli_obj, LIB]):
        _run([nvcc] + ARCH + ["-o", CLI, cli_obj, "-L", HERE, "-lflock_gb300", "-Xlinker", "-rpath,$ORIGIN"])
    with open(marker, "w") as f:
        f.write(arch)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
