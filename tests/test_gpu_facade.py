"""The C++ facade and the command line on the GPU, on the reference's own
instance files (tests/golden/reference_fixtures.json, written back as .dat
files in the reference's layout):

- the shipped CLI (flock_gb300/flock, a driver of the reference's
  src/main.cpp shape) for -a parallel_uv, parallel_ss and switch_hybrid: its
  BASIC STATISTICS objective equals the reference build's objective (exact
  decimal against the reference's float sum, within its float rounding) and
  the exact solve of the Python binding; the LVL1 / LVL2 lines carry the
  reference's labels and the phase times;
- a committed driver (tests/drivers/facade_main.cpp) compiled here with g++
  against include/flock/algos.h and linked with the library: objVal equals
  the exact objective, and the flows that create_flows() wrote reproduce it.
"""
import json
import os
import re
import subprocess

import numpy as np
import pytest

import flock_gb300 as fg

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
CLI = os.path.join(ROOT, "flock_gb300", "flock")
ALGOS = ("parallel_uv", "parallel_ss", "switch_hybrid")


def _fixtures():
    with open(os.path.join(GOLDEN, "reference_fixtures.json")) as f:
        return json.load(f)


@pytest.fixture(scope="module")
def fixture_files(tmp_path_factory):
    d = tmp_path_factory.mktemp("fixtures")
    out = []
    for e in _fixtures():
        m, n, scale = e["m"], e["n"], e["scale"]
        inst = fg.Instance(np.array(e["supply"], np.int32), np.array(e["demand"], np.int32),
                           np.array(e["cost"], np.int32).reshape(m, n))
        p = str(d / e["file"])
        fg.write_dat(inst, p, scale)
        out.append((p, e, inst))
    return out


def _num(line, label):
    m = re.search(re.escape(label) + r": (-?[0-9.e+]+)", line)
    assert m, (label, line)
    return float(m.group(1))


def _lines(stdout, tag):
    return [ln for ln in stdout.splitlines() if tag in ln]


def _check_objective(text, e, inst, scale):
    """The printed exact objective: equal to the library's exact solve, and to
    the reference build's float objective within its float rounding when the
    reference ended optimal."""
    exact = fg.solve(inst).objective
    assert text == (str(exact) if scale == 0 else f"{exact // 10 ** scale}.{exact % 10 ** scale:0{scale}d}")
    if e["status"] == 0:
        assert abs(exact / 10 ** scale - e["objective"]) <= 1e-6 * max(1.0, abs(e["objective"])) + 0.01


@pytest.mark.parametrize("algo", ALGOS)
def test_cli_statistics_on_reference_fixtures(fixture_files, algo):
    assert os.path.exists(CLI), "CLI not built"
    for path, e, inst in fixture_files:
        r = subprocess.run([CLI, "-i", path, "-a", algo], capture_output=True, text=True, timeout=120)
        assert r.returncode == 0, (e["file"], r.returncode, r.stderr)
        basic = _lines(r.stdout, "BASIC STATISTICS")
        assert len(basic) == 1, r.stdout
        obj = re.search(r"Objective: (-?[0-9.]+) \|", basic[0]).group(1)
        _check_objective(obj, e, inst, e["scale"])
        assert f"MATRIX : {e['m']} X {e['n']}" in basic[0]
        lvl2 = _lines(r.stdout, "LVL2 PIVOT STATISTICS")
        assert len(lvl2) == 1
        for label in ("Total Pivot Time", "RESOLVE Time", "ADJUST Time"):
            assert _num(lvl2[0], label) >= 0
        if algo == "parallel_uv":
            lvl1 = _lines(r.stdout, "LVL1 STATISTICS |")
            assert len(lvl1) == 1
            for label in ("Total Time", "UV Time", "R Time", "PIVOT Time"):
                assert _num(lvl1[0], label) >= 0
        elif algo == "parallel_ss":
            lvl1 = _lines(r.stdout, "LVL1 STATISTICS |")
            assert len(lvl1) == 1 and _num(lvl1[0], "PIVOT Time") >= 0
        else:
            assert len(_lines(r.stdout, "LVL1 STATISTICS(A)")) == 1
            assert len(_lines(r.stdout, "LVL1 STATISTICS(B)")) == 1
            assert "CYCLE Time (parallel BFS + seq DFS)" in lvl2[0]
        flock = _lines(r.stdout, "FLOCK STATISTICS")
        assert len(flock) == 1 and "CERTIFIED: 1" in flock[0] and "STATUS: 0" in flock[0]


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("driver") / "facade_main")
    lib_dir = os.path.join(ROOT, "flock_gb300")
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "drivers", "facade_main.cpp"), "-L", lib_dir, "-lflock_gb300",
                        f"-Wl,-rpath,{lib_dir}", "-o", exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    return exe


@pytest.mark.parametrize("algo", ALGOS)
def test_facade_driver_on_reference_fixtures(fixture_files, driver, algo):
    for path, e, inst in fixture_files:
        r = subprocess.run([driver, "-i", path, "-a", algo], capture_output=True, text=True, timeout=120)
        assert r.returncode == 0, (e["file"], r.returncode, r.stdout, r.stderr)
        basic = _lines(r.stdout, "BASIC STATISTICS")[0]
        check = _lines(r.stdout, ">>>> CHECK")[0]
        exact = int(re.search(r"Exact: (-?[0-9]+)", check).group(1))
        scale = int(re.search(r"Scale: ([0-9]+)", check).group(1))
        assert scale == e["scale"]
        assert exact == fg.solve(inst).objective
        obj = _num(basic, "Objective")
        assert abs(obj - exact / 10 ** scale) <= 1e-9 * max(1.0, abs(obj))
        # the created flows (float quantities, float costs) reproduce the objective
        assert abs(_num(check, "Flow cost") - obj) <= 1e-6 * max(1.0, abs(obj))
        if e["status"] == 0:
            assert abs(obj - e["objective"]) <= 1e-6 * max(1.0, abs(e["objective"])) + 0.01
        phases = _lines(r.stdout, ">>>> PHASES")[0]
        for label in ("UV Time", "R Time", "PIVOT Time", "CYCLE Time", "RESOLVE Time", "ADJUST Time"):
            assert _num(phases, label) >= 0


@pytest.mark.parametrize("name,m,n,pivot", [("uniform100", None, None, "sequential"),
                                            ("degenerate1000", None, None, "parallel"),
                                            ("degenerate1000", 2048, 2048, "switch")])
def test_phase_times_cover_the_loop(name, m, n, pivot):
    """flock_stats' phase times (device clock) add up to the pivot loop's
    device time (CUDA events) plus the start tree's dual rebuild; each phase
    the pivot method uses is nonzero.  The 2048 x 2048 instance runs the
    grid-wide rounds, the others the one-block rounds."""
    inst = fg.config_instance(name, 0, m=m, n=n)
    r = fg.solve(inst, pivot=pivot)
    assert r.status == 0 and r.certified
    total = r.ms_dual + r.ms_sweep + r.ms_pivot
    assert abs(r.ms_pivot - (r.ms_cycle + r.ms_resolve + r.ms_adjust)) < 1e-9
    assert 0.5 * r.ms_simplex <= total <= r.ms_simplex + r.ms_bfs + 0.5, (total, r.ms_simplex, r.ms_bfs)
    assert r.ms_sweep > 0 and r.ms_cycle > 0 and r.ms_adjust > 0 and r.ms_dual > 0
    if pivot == "parallel":
        assert r.ms_resolve > 0
    if pivot == "sequential":
        assert r.ms_resolve == 0
    # the batched form leaves them 0
    b = fg.batch_solve([inst])[0] if inst.m + inst.n <= 4096 else None
    if b is not None:
        assert b.ms_dual == b.ms_sweep == b.ms_pivot == 0
