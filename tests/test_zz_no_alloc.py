"""flock_vogel_static, the allocation-free Vogel entry point (no counterpart in
the reference): called through the C ABI twice in a row per instance, its
allocation lists and event counts must equal flock_vogel's bit for bit and
the oracle's (the reference's Vogel restated on the CPU), and the calls must
leave the device's free memory unchanged (nothing allocated, nothing freed).

The file name sorts last so that the test also runs after every other test of
the session (a warm library, scratch left over from other calls); it passes
alone in a fresh process as well.  Instances go from large to small, so each
call finds the previous instance's data in the static scratch.
"""
import ctypes

import numpy as np
import pytest

import flock_gb300 as fg
import oracle

MAX_V = 8192
MAX_CELLS = 1048576


def _static_fn():
    L = fg.lib()
    f = L.flock_vogel_static
    f.argtypes = [ctypes.POINTER(fg.CInstance), ctypes.POINTER(fg.CFlow), ctypes.POINTER(ctypes.c_int32)]
    f.restype = ctypes.c_int
    return f


def vogel_static(inst):
    ci = inst.c()
    flows = np.full((inst.m + inst.n - 1, 3), -7, np.int32)
    ev = ctypes.c_int32(-99)
    rc = _static_fn()(ctypes.byref(ci), flows.ctypes.data_as(ctypes.POINTER(fg.CFlow)), ctypes.byref(ev))
    return rc, flows, int(ev.value)


def _cases():
    out = [
        ("max vertices 128x8064", fg.generate(0, 11, 128, 8064, 1, 1000, 100, 1000)),
        ("max cells 1024x1024", fg.generate(0, 12, 1024, 1024, 1, 1000, 100, 1000)),
        ("tall 8064x128", fg.generate(0, 13, 8064, 128, 1, 50, 1, 50)),
        ("degenerate 300x250", fg.config_instance("degenerate1000", 3, m=300, n=250)),
        ("uniform 100x100", fg.config_instance("uniform100", 5)),
        ("ragged 26x10", fg.generate(0, 14, 26, 10, 1, 1000, 100, 1000)),
    ]
    for s in range(60):
        out.append((f"tiny tied {s}", fg.generate(0, 1000 + s, 2 + s % 4, 2 + (s // 4) % 4, 1, 3, 1, 3)))
    out.append(("single cell 1x1", fg.generate(0, 15, 1, 1, 1, 9, 5, 5)))
    return out


def _cudart():
    """The CUDA runtime the native library was linked against (found among the
    process's mapped files once the library is loaded)."""
    fg.lib()
    with open("/proc/self/maps") as f:
        paths = sorted({ln.split()[-1] for ln in f if "libcudart.so" in ln})
    assert paths, "libcudart is not mapped"
    rt = ctypes.CDLL(paths[0])
    rt.cudaMemGetInfo.argtypes = [ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(ctypes.c_size_t)]
    return rt


def _free_bytes(rt):
    free, total = ctypes.c_size_t(), ctypes.c_size_t()
    assert rt.cudaMemGetInfo(ctypes.byref(free), ctypes.byref(total)) == 0
    return int(free.value)


def _oracle_list(inst):
    """The oracle's allocation list in the C ABI's (source, destination, qty)
    layout (the reference writes 1e-6 for a zero allocation), cut before the
    first entry where the reference indexes past its arrays (events -1), from
    where its result is undefined."""
    src, dst, q, oev = oracle.vogel(inst.supply, inst.demand, inst.cost)
    qi = np.where(q < 0.5, 0, q).astype(np.int64)
    out = np.stack([src, dst, qi], 1)
    if oev < 0:
        out = out[:int(np.argmax(src < 0))]
    return out, oev


@pytest.mark.gpu
def test_static_vogel_matches_vogel_twice():
    cases = _cases()
    # expected results first: flock_vogel grows its own device buffers
    expected = []
    for name, inst in cases:
        ref_flows, ref_ev = fg.vogel(inst)
        orc_flows, orc_ev = _oracle_list(inst)
        assert ref_ev == orc_ev, (name, ref_ev, orc_ev)
        np.testing.assert_array_equal(ref_flows[:len(orc_flows)].astype(np.int64), orc_flows, err_msg=name)
        expected.append((ref_flows, ref_ev, orc_flows))
    rt = _cudart()
    rc, _, _ = vogel_static(cases[0][1])        # set-up call (module and per-thread stream)
    assert rc == fg.FLOCK_OK, fg.lib().flock_last_error()
    free0 = _free_bytes(rt)
    for (name, inst), (ref_flows, ref_ev, orc_flows) in zip(cases, expected):
        for call in (1, 2):
            rc, flows, ev = vogel_static(inst)
            assert rc == fg.FLOCK_OK, (name, call, rc, fg.lib().flock_last_error())
            assert ev == ref_ev, (name, call, ev, ref_ev)
            np.testing.assert_array_equal(flows, ref_flows, err_msg=f"{name}, call {call}")
            np.testing.assert_array_equal(flows[:len(orc_flows)].astype(np.int64), orc_flows,
                                          err_msg=f"{name}, call {call}, oracle")
    assert _free_bytes(rt) == free0, "device free memory changed across the calls"


def test_static_vogel_rejects_oversize():
    """Sizes beyond the static scratch are refused before any CUDA call."""
    L = fg.lib()
    L.flock_last_error.restype = ctypes.c_char_p
    for m, n in ((1, MAX_V), (MAX_V // 2, MAX_V // 2 + 1), (1025, 1024), (2048, 600)):
        inst = fg.generate(0, 21, m, n, 1, 9, 1, 9)
        assert m + n > MAX_V or m * ((n + 3) // 4 * 4) > MAX_CELLS
        rc, _, _ = vogel_static(inst)
        assert rc == fg.FLOCK_ERR_RANGE, (m, n, rc)
        assert b"static scratch" in L.flock_last_error()


def test_static_vogel_declared():
    """The header declares the entry point and its limits."""
    import os
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    h = open(os.path.join(root, "include", "flock.h")).read()
    assert "int flock_vogel_static(const flock_instance* inst, flock_flow* flows, int32_t* events);" in h
    assert f"#define FLOCK_VOGEL_STATIC_MAX_V {MAX_V}" in h
    assert f"#define FLOCK_VOGEL_STATIC_MAX_CELLS {MAX_CELLS}" in h
