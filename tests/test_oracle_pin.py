"""CPU: the oracle (C restatement of the reference CPU path) pinned to the
reference itself -- golden outputs of the reference's own functions
(tests/golden, made by make_golden.py from the reference build), the
reference's published run logs, and, where the reference sources are
present, the reference build run live.  Also checks the certificate checker
by planting mistakes in its inputs.  The published-log pins take the data
files under 500 KB by default; FLOCK_PIN_ALL=1 takes every one present (22
per log, about a minute and a half)."""
import json
import os

import numpy as np
import pytest

import oracle
from conftest import GOLDEN, REFERENCE
from golden_util import float_costs, tiny


def load(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


def check_against(e, s, d, cf):
    src, dst, q, ev = oracle.vogel(s, d, cf)
    if ev >= 0:
        assert src.tolist() == e["vogel_src"]
        assert dst.tolist() == e["vogel_dst"]
        assert np.array_equal(q, np.asarray(e["vogel_qty"], np.float32))
    else:   # undefined in the reference from the first marked step on
        k = int(np.argmax(src < 0))
        assert src[:k].tolist() == e["vogel_src"][:k]
        return
    r = oracle.solve_ref(s, d, cf)
    assert r["iterations"] == e["iterations"]
    assert r["status"] == e["status"]
    assert r["objective"] == e["objective"]
    assert r["active"] == e["active"]


@pytest.mark.parametrize("e", load("reference_fixtures.json"), ids=lambda e: e["file"])
def test_reference_fixtures(orc, e):
    s = np.array(e["supply"], np.int32)
    d = np.array(e["demand"], np.int32)
    cf = np.array(e["cost_f32"], np.float32) if "cost_f32" in e else float_costs(e["cost"], e["scale"])
    check_against(e, s, d, cf)


def test_reference_random(orc):
    g = load("reference_random.json")
    insts = tiny(g["seed"], g["count"], g["max_dim"])
    for (s, d, c), e in zip(insts, g["results"]):
        check_against(e, s, d, c.astype(np.float32))


def test_reference_synthetic(orc):
    fg = pytest.importorskip("flock_gb300")
    from golden_util import checksum
    for e in load("reference_synthetic.json"):
        inst = fg.config_instance(e["name"], e["seed"], m=e["m"], n=e["n"])
        assert checksum(inst.supply, inst.demand, inst.cost) == e["checksum"]
        check_against(e, inst.supply, inst.demand, inst.cost.astype(np.float32))


def test_known_optima(orc):
    # integer fixtures: optimum also confirmed with an LP solver
    known = {"test_simple1_degenerate.dat": 92, "test_simple2.dat": 743, "test_simple4.dat": 555,
             "test_TransportModel_10_10_0.dat": 13084, "test_TransportModel_100_100_0.dat": 64823}
    for e in load("reference_fixtures.json"):
        if e["file"] in known:
            r = oracle.solve_ref(np.array(e["supply"], np.int32), np.array(e["demand"], np.int32),
                                 float_costs(e["cost"], 0))
            assert r["status"] == 0 and r["objective"] == known[e["file"]]


def _published_data_files(key="pure_sequencial"):
    d = os.path.join(REFERENCE, "data")
    if not os.path.isdir(d):
        return []
    pub = load("published.json")[key]
    out = []
    for f, v in sorted(pub.items()):
        p = os.path.join(d, f)
        if os.path.exists(p) and (os.path.getsize(p) < 500_000 or os.environ.get("FLOCK_PIN_ALL") == "1"):
            out.append((p, v))
    return out


@pytest.mark.parametrize("path,pub", _published_data_files(), ids=lambda x: os.path.basename(str(x)))
def test_published_cpu_path(orc, path, pub):
    """Iterations and objective of results/pure_sequencial, reproduced."""
    tok = open(path).read().split()
    m, n = int(tok[0]), int(tok[1])
    s = np.array(tok[2:2 + m], np.int32)
    d = np.array(tok[2 + m:2 + m + n], np.int32)
    c = np.array([float(x) for x in tok[2 + m + n:]], np.float32)
    r = oracle.solve_ref(s, d, c)
    assert r["iterations"] == pub["iterations"]
    assert "%g" % r["objective"] == pub["objective"]


@pytest.mark.parametrize("path,pub", _published_data_files("parallel_uv"), ids=lambda x: os.path.basename(str(x)))
def test_published_device_vogel_path(orc, path, pub):
    """Iterations and objective of results/parallel_uv (BFS vam_device, host
    duals, sequential cycle search, first-minimum sweep), reproduced by the
    restatement of the reference's device Vogel feeding the CPU path."""
    tok = open(path).read().split()
    m, n = int(tok[0]), int(tok[1])
    s = np.array(tok[2:2 + m], np.int32)
    d = np.array(tok[2 + m:2 + m + n], np.int32)
    c = np.array([float(x) for x in tok[2 + m + n:]], np.float32)
    r = oracle.solve_ref(s, d, c, bfs=2)
    assert r["iterations"] == pub["iterations"]
    assert "%g" % r["objective"] == pub["objective"]


@pytest.mark.skipif(not oracle.ref_available(), reason="reference build not present")
def test_live_reference_build(orc):
    """The restatement against the reference's own compiled functions."""
    rng = np.random.default_rng(77)
    for (s, d, c) in tiny(4242, 200):
        cf = c.astype(np.float32)
        a = oracle.ref_vogel(s, d, cf)
        b = oracle.vogel(s, d, cf)
        if b[3] < 0:
            continue
        for x, y in zip(a, b[:3]):
            assert np.array_equal(x, y)
        ra, rb = oracle.ref_solve(s, d, cf), oracle.solve_ref(s, d, cf)
        assert (ra["iterations"], ra["status"], ra["objective"]) == (rb["iterations"], rb["status"], rb["objective"])
    del rng


def test_certificate_checker_plants(orc):
    """Mistakes planted in the checker's inputs are all caught."""
    e = [x for x in load("reference_fixtures.json") if x["file"] == "test_TransportModel_10_10_0.dat"][0]
    s = np.array(e["supply"], np.int32)
    d = np.array(e["demand"], np.int32)
    c = np.array(e["cost"], np.int32).reshape(e["m"], e["n"])
    r = oracle.solve_ref(s, d, c.astype(np.float32))
    ok, u, v = oracle.tree_duals(c, r["tree"])
    assert ok == 0
    flows = r["flows"]
    bits, obj = oracle.certify(s, d, c, flows, u, v)
    assert bits == 0 and obj == 13084
    f = flows.copy(); f[0, 2] = -1
    assert oracle.certify(s, d, c, f, u, v)[0] & 1
    f = flows.copy(); f[0, 2] += 1
    assert oracle.certify(s, d, c, f, u, v)[0] & 6
    u2 = u.copy(); u2[0] += 1000
    assert oracle.certify(s, d, c, flows, u2, v)[0] & 8
    u3 = u.copy(); u3[int(flows[0, 0])] -= 1
    assert oracle.certify(s, d, c, flows, u3, v)[0] & 16


def test_reference_path_matches_lp_optimum(orc):
    """The restated reference CPU path against an independent LP solver
    (HiGHS) on seeded instances where it terminates by optimality."""
    pytest.importorskip("scipy")
    from lp_check import lp_optimum
    import flock_gb300 as fg
    checked = 0
    for seed in range(12):
        m, n = 8 + 3 * seed, 12 + 2 * seed
        inst = fg.generate(0, 3000 + seed, m, n, 1, 100, 10, 100)
        r = oracle.solve_ref(inst.supply, inst.demand, inst.cost.astype(np.float32))
        if oracle.verdict(inst.supply, inst.demand, inst.cost, r) != "optimal":
            continue
        assert round(r["objective"]) == lp_optimum(inst.supply, inst.demand, inst.cost), seed
        checked += 1
    assert checked >= 8


def test_generator_restatement_matches_library():
    """The oracle's restatement of the instance generator (used by the
    benchmark's reference arm, which does not load the product library)
    makes the library's instances bit for bit: the mixed batch, the uniform
    and the Euclidean generators."""
    import flock_gb300 as fg
    a = oracle.mixed_batch(20251203, 96, 10, 500)
    b = fg.mixed_batch(20251203, 96, 10, 500)
    for x, y in zip(a, b):
        for u, w in zip(x, (y.supply, y.demand, y.cost)):
            np.testing.assert_array_equal(u, w)
    for kind, args in ((0, (1, 20, 1, 50)), (1, (0, 0, 1, 10000)), (0, (5, 5, 0, 0))):
        s, d, c = oracle.generate(kind, 77, 123, 211, *args)
        y = fg.generate(kind, 77, 123, 211, *args)
        np.testing.assert_array_equal(c, y.cost)
        np.testing.assert_array_equal(s, y.supply)
        np.testing.assert_array_equal(d, y.demand)
    ms, ns = oracle.generate_sizes(5, 1000, 10, 2000)
    gm, gn = fg.generate_sizes(5, 1000, 10, 2000)
    np.testing.assert_array_equal(ms, gm)
    np.testing.assert_array_equal(ns, gn)


def test_bounded_cpu_samples_follow_the_pinned_path():
    """The bounded CPU samples of large instances (the first Vogel steps, one
    sequential scan) are the pinned functions cut short: the first k
    allocations equal the full Vogel's, and the scan finds the same entering
    cell as a numpy restatement of the reference's row-major first strict
    minimum."""
    rng = np.random.default_rng(3)
    for m, n in ((40, 30), (7, 90), (120, 5)):
        s = rng.integers(1, 50, m).astype(np.int32)
        d = rng.integers(1, 50, n).astype(np.int32)
        d[-1] += int(s.sum() - d.sum()) if s.sum() > d.sum() else 0
        s[-1] += int(d.sum() - s.sum()) if d.sum() > s.sum() else 0
        c = rng.integers(1, 20, (m, n)).astype(np.int32)
        src, dst, q, ev = oracle.vogel(s, d, c)
        for k in (1, 5, m + n - 1):
            a, b, qq, ev2, done = oracle.vogel_steps(s, d, c, k)
            assert done == k
            np.testing.assert_array_equal(a[:k], src[:k])
            np.testing.assert_array_equal(b[:k], dst[:k])
            np.testing.assert_array_equal(qq[:k], q[:k])
        h = rng.integers(-30, 30, m + n).astype(np.float32)
        r = c.astype(np.float32) - h[:m, None] - h[None, m:]
        flat = int(np.argmin(r))       # first minimum in row-major order
        v, i, j = oracle.sweep(c, h)
        assert (i, j) == divmod(flat, n) and v == r.min()
