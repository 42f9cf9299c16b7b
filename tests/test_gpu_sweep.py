"""Reduced-cost sweep parity: the grid-wide k_sweep and the CTA-local sweep of
the batched form against an exact int64 restatement in numpy.

The row key is min over j of (clamp32(c_ij - u_i - v_j), j), the smaller
column winning ties.  Cases cover the int32 (narrow) form, ragged and tiny
widths, several column tiles, zero-demand columns (dual kDeadPot), reduced
costs below INT32_MIN (exact rescan) and duals too wide for int32.
"""
import ctypes

import numpy as np
import pytest

import flock_gb300 as fg

pytestmark = pytest.mark.gpu

DEAD = -(1 << 61)


def expected_keys(cost, pot):
    m, n = cost.shape
    u = pot[:m].astype(np.int64)
    v = pot[m:].astype(np.int64)
    r = cost.astype(np.int64) - u[:, None] - v[None, :]
    rc = np.clip(r, -(1 << 31), (1 << 31) - 1)
    hi = (rc.astype(np.int64) ^ np.int64(-(1 << 31))) & 0xFFFFFFFF   # (uint32)value ^ 0x80000000
    keys = (hi.astype(np.uint64) << np.uint64(32)) | np.arange(n, dtype=np.uint64)[None, :]
    return keys.min(axis=1)


def gpu_keys(cost, pot, cta_form=0, threads=256):
    L = fg.lib()
    f = L.flock_test_sweep
    f.argtypes = [ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.c_int32, ctypes.c_int32]
    cost = np.ascontiguousarray(cost, np.int32)
    pot = np.ascontiguousarray(pot, np.int64)
    m, n = cost.shape
    keys = np.zeros(m, np.uint64)
    rc = f(m, n, cost.ctypes.data, pot.ctypes.data, keys.ctypes.data, cta_form, threads)
    assert rc == 0, L.flock_last_error()
    return keys


def case(seed, m, n, lo=1, hi=1000, plo=-500, phi=500):
    rng = np.random.default_rng(seed)
    cost = rng.integers(lo, hi + 1, size=(m, n), dtype=np.int64).astype(np.int32)
    pot = rng.integers(plo, phi + 1, size=m + n, dtype=np.int64)
    return cost, pot


SHAPES = [(1, 1), (3, 2), (5, 3), (7, 4), (37, 53), (64, 1023), (9, 1024), (9, 1025), (4, 2050),
          (300, 301), (2, 8192), (3, 8193), (2, 20003)]


@pytest.mark.parametrize("m,n", SHAPES)
def test_sweep_narrow(m, n):
    cost, pot = case(m * 7919 + n, m, n)
    exp = expected_keys(cost, pot)
    np.testing.assert_array_equal(gpu_keys(cost, pot), exp)
    if n <= 3000:
        for thr in (32, 128, 256):
            np.testing.assert_array_equal(gpu_keys(cost, pot, 1, thr), exp)


@pytest.mark.parametrize("m,n", [(1, 1), (3, 2), (7, 9), (37, 53), (9, 2047), (9, 2048), (9, 2049), (4, 4100),
                                 (300, 301), (3, 8193), (2, 20003)])
def test_sweep_16bit_copy(m, n):
    """The bulk sweep on the 16-bit copy of the costs (the grid path's sweeps
    when every cost fits): keys identical to the int32 form's, costs at the
    16-bit limits included."""
    cost, pot = case(m * 131 + n, m, n, lo=-32768, hi=32767, plo=-40000, phi=40000)
    exp = expected_keys(cost, pot)
    np.testing.assert_array_equal(gpu_keys(cost, pot, -1), exp)
    np.testing.assert_array_equal(gpu_keys(cost, pot, 0), exp)


@pytest.mark.parametrize("m,n", [(5, 7), (40, 1500), (3, 9000)])
def test_sweep_ties_and_dead_columns(m, n):
    cost = np.full((m, n), 5, np.int32)
    pot = np.zeros(m + n, np.int64)
    pot[m + 1::3] = DEAD              # zero-demand columns: never the row best while others are negative
    pot[:m] = 7                       # every live reduced cost is -2: first live column wins
    exp = expected_keys(cost, pot)
    np.testing.assert_array_equal(gpu_keys(cost, pot), exp)
    np.testing.assert_array_equal(gpu_keys(cost, pot, -1), exp)
    if n <= 3000:
        np.testing.assert_array_equal(gpu_keys(cost, pot, 1, 256), exp)
    # a dead column holds the int32 minimum (cheaper cost, live duals at the
    # window's lower edge): the row is recomputed exactly
    dead = np.zeros(n, bool)
    dead[1::3] = True
    cost[:, dead] = 0
    pot[:m] = 0
    pot[m:][~dead] = -(1 << 30) + 2
    exp = expected_keys(cost, pot)
    np.testing.assert_array_equal(gpu_keys(cost, pot), exp)
    if n <= 3000:
        np.testing.assert_array_equal(gpu_keys(cost, pot, 1, 128), exp)


def test_sweep_clamped_rows():
    """Reduced costs below INT32_MIN: several columns clamp, the first wins."""
    cost, pot = case(11, 50, 3000)
    pot[:25] = (1 << 40)              # huge row duals: every r < INT32_MIN in rows 0..24
    exp = expected_keys(cost, pot)
    np.testing.assert_array_equal(gpu_keys(cost, pot), exp)
    np.testing.assert_array_equal(gpu_keys(cost, pot, 1, 256), exp)


def test_sweep_wide_duals():
    """A column dual outside the int32 window: the exact int64 form runs."""
    cost, pot = case(12, 60, 2500, plo=-(1 << 20), phi=(1 << 20))
    pot[60 + 17] = (1 << 35)
    pot[60 + 2000] = -(1 << 33)
    exp = expected_keys(cost, pot)
    np.testing.assert_array_equal(gpu_keys(cost, pot), exp)
    np.testing.assert_array_equal(gpu_keys(cost, pot, 1, 256), exp)


def test_sweep_extreme_costs():
    """Costs at the accepted limits +-2^30 with duals at the narrow window's edge."""
    rng = np.random.default_rng(13)
    m, n = 20, 777
    cost = rng.choice(np.array([-(1 << 30), (1 << 30), 0, 1, -1], np.int64), size=(m, n)).astype(np.int32)
    pot = rng.integers(-(1 << 30) + 2, (1 << 30) - 1, size=m + n, dtype=np.int64)
    exp = expected_keys(cost, pot)
    np.testing.assert_array_equal(gpu_keys(cost, pot), exp)
    np.testing.assert_array_equal(gpu_keys(cost, pot, 1, 256), exp)


# ---------------------------------------------------------------------------
# Partial pricing's candidate-row selection (select_candidate_rows): rows with
# negative keys, a 32-bin histogram over [rmin, 0) whose leading bins hold at
# most kPPRows rows (the first bin always), then the first kPPRows such rows
# in row order; every other key cleared.  The returned entering row is the
# smallest (value, row) among the rows kept.
NOKEY = (1 << 64) - 1


def pack(v, idx):
    return ((((v & 0xFFFFFFFF) ^ 0x80000000)) << 32) | idx


def expect_select(vals, kpp):
    m = len(vals)
    neg = [v for v in vals if v is not None and v < 0]
    rmin = min(neg) if neg else 0
    span = -rmin if rmin < 0 else 1
    last = -1
    if rmin < 0:
        hist = [0] * 32
        for v in neg:
            hist[((v - rmin) * 32) // span] += 1
        cum, last = hist[0], 0
        for b in range(1, 32):
            if cum + hist[b] > kpp:
                break
            cum += hist[b]
            last = b
    sel = [v is not None and v < 0 and ((v - rmin) * 32) // span <= last for v in vals]
    kept = [i for i in range(m) if sel[i]][:kpp]
    best = min((vals[i], i) for i in kept) if kept else None
    return kept, sum(sel), best


def gpu_select(keys, threads=256):
    L = fg.lib()
    f = L.flock_test_select_rows
    f.argtypes = [ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32]
    keys = np.ascontiguousarray(keys, np.uint64)
    out = np.zeros_like(keys)
    prow = np.full(1024, -1, np.int32)
    pn, kpp = ctypes.c_int32(-1), ctypes.c_int32(-1)
    best = np.zeros(1, np.uint64)
    rc = f(len(keys), keys.ctypes.data, out.ctypes.data, prow.ctypes.data, ctypes.addressof(pn),
           ctypes.addressof(kpp), best.ctypes.data, threads)
    assert rc == 0, L.flock_last_error()
    return out, prow[:pn.value].tolist(), kpp.value, int(best[0])


def check_select(vals, threads=256):
    keys = np.array([NOKEY if v is None else pack(v, i % 7) for i, v in enumerate(vals)], np.uint64)
    out, prow, kpp, best = gpu_select(keys, threads)
    kept, total, eb = expect_select(vals, kpp)
    assert prow == kept
    want = NOKEY if eb is None else pack(eb[0], eb[1])
    assert best == want, (hex(best), eb)
    keep = set(kept)
    for i in range(len(vals)):
        assert int(out[i]) == (int(keys[i]) if i in keep else NOKEY), i


def test_select_rows_crowded_first_bin():
    """More rows than kPPRows in the first histogram bin: the rows past
    kPPRows in row order are dropped, among them the overall best one, and the
    entering row returned is the best row kept."""
    vals = [-100] * 200
    vals[150] = -101
    check_select(vals)
    check_select(vals, threads=64)


@pytest.mark.parametrize("seed", range(6))
def test_select_rows_random(seed):
    rng = np.random.default_rng(seed)
    m = int(rng.integers(1, 700))
    lo = int(rng.choice([3, 50, 100000]))
    vals = [None if rng.random() < 0.2 else int(rng.integers(-lo, lo)) for _ in range(m)]
    check_select(vals, threads=int(rng.choice([32, 128, 256, 1024])))
