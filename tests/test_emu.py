"""The device-side solve on the CPU: the unmodified CTA-level device
functions (Vogel, start tree, rebuilds, sweeps, pivots, certificate) run on
an emulated CTA of fibers (flock_gb300/csrc/emu) under AddressSanitizer and
UBSan.  Every barrier checks that all threads arrived from the same call
site, and after every single pivot the incrementally updated depths, duals,
int32 duals and preorder intervals are compared with a full rebuild.  Each
run must end optimal and certified with no mismatch."""
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EMU_DIR = os.path.join(ROOT, "flock_gb300", "csrc", "emu")
EMU = os.path.join(EMU_DIR, "emu_check")


@pytest.fixture(scope="module")
def emu():
    if shutil.which("g++") is None or shutil.which("make") is None:
        pytest.skip("no host C++ toolchain")
    r = subprocess.run(["make", "-C", EMU_DIR], capture_output=True, text=True)
    if r.returncode != 0:
        pytest.skip("emulator does not build here: " + r.stderr[-300:])
    return EMU


def run(emu, args, env=None, timeout=300):
    e = dict(os.environ)
    e.update(env or {})
    r = subprocess.run([emu] + [str(a) for a in args], capture_output=True, text=True, env=e, timeout=timeout)
    lines = [l for l in r.stdout.splitlines() if l.startswith("k=")]
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    assert lines and all(l.endswith(" ok") for l in lines), r.stdout[-2000:]
    assert "bad=0" in r.stdout
    assert not re.search(r"ERROR: AddressSanitizer|runtime error:", r.stderr), r.stderr[-2000:]
    return lines


# (mode, pricing, threads): mode 0 sequential, 1 parallel, 2 switch; pricing 0
# full, 1 partial, 2 partial with the row keys overwritten between rounds
@pytest.mark.parametrize("mode,pricing,threads", [(0, 1, 64), (1, 1, 96), (2, 1, 32), (2, 2, 128), (1, 0, 64)])
def test_emulated_solves(emu, mode, pricing, threads):
    run(emu, [20251203, 6, 10, 60, 0, 5, mode, pricing], {"EMU_THREADS": str(threads)})


def test_emulated_degenerate(emu):
    """Costs and quantities in 1..3: ties everywhere, degenerate bases."""
    run(emu, [77, 6, 5, 50, 0, 5, 2, 1], {"EMU_THREADS": "64", "EMU_COST_HI": "3", "EMU_QTY_LO": "1",
                                          "EMU_QTY_HI": "3"})


def test_emulated_short_candidate_lists(emu):
    """Partial pricing with 8 candidate rows and a full sweep every 2 rounds:
    the first histogram bin often holds more rows than kept."""
    run(emu, [99, 6, 20, 70, 0, 5, 2, 1], {"EMU_THREADS": "64", "EMU_PP_ROWS": "8", "EMU_PP_REFRESH": "2"})
