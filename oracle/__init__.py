"""TEST INFRASTRUCTURE ONLY -- the checker, never the product.

ctypes bindings of the C restatement of the reference CPU path (oracle.c ->
liborc.so; also the restatement of the reference's device Vogel,
vogel_device) and, where it was built, of the reference's own functions
(oracle/_ref/libflockref.so).  Only tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg import this package.
"""
from __future__ import annotations

import ctypes
import os
import platform
import subprocess
from typing import Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORC = os.path.join(HERE, "liborc.so")
REF = os.path.join(HERE, "_ref", "libflockref.so")
P = ctypes.POINTER
i32, i64 = ctypes.c_int32, ctypes.c_int64


class OrcResult(ctypes.Structure):
    _fields_ = [("iterations", i32), ("status", i32), ("active_flows", i32), ("vogel_events", i32),
                ("objective", ctypes.c_double)]


def build(reference_dir: Optional[str] = None) -> None:
    """Compile liborc.so (and oracle/_ref when the reference sources exist).
    Libraries built on another machine architecture are rebuilt."""
    marker = os.path.join(HERE, ".arch")
    arch = platform.machine()
    stale = not os.path.exists(marker) or open(marker).read().strip() != arch
    subprocess.run(["make", "-s"] + (["-B"] if stale else []) + ["-C", HERE, "liborc.so"], check=True)
    if reference_dir and os.path.isdir(os.path.join(reference_dir, "src")):
        subprocess.run(["make", "-s"] + (["-B"] if stale else []) + ["-C", HERE, "ref", f"REF={reference_dir}"],
                       check=True)
    with open(marker, "w") as f:
        f.write(arch)


_orc = None
_ref = None


def orc() -> ctypes.CDLL:
    global _orc
    if _orc is None:
        if not os.path.exists(ORC):
            build()
        L = ctypes.CDLL(ORC)
        L.orc_vogel.argtypes = [i32, i32, P(i32), P(i32), P(ctypes.c_float), P(i32), P(i32), P(ctypes.c_float)]
        L.orc_nwc.argtypes = [i32, i32, P(i32), P(i32), P(i32), P(i32), P(ctypes.c_float)]
        L.orc_vogel_device.argtypes = [i32, i32, P(i32), P(i32), P(ctypes.c_float), P(i32), P(i32),
                                       P(ctypes.c_float)]
        L.orc_solve_ref.argtypes = [i32, i32, P(i32), P(i32), P(ctypes.c_float), i32, i32,
                                    P(i32), P(i32), P(ctypes.c_float), P(i32), P(i32), P(OrcResult)]
        L.orc_solve_ref_batch.argtypes = [i32, P(i32), P(i32), P(i64), P(i64), P(i64), P(i32), P(i32),
                                          P(ctypes.c_float), i32, i32, i32, P(ctypes.c_double), P(i32), P(i32)]
        L.orc_tree_duals.argtypes = [i32, i32, P(i32), i32, P(i32), P(i32), P(i64), P(i64)]
        L.orc_certify.argtypes = [i32, i32, P(i32), P(i32), P(i32), i32, P(i32), P(i32), P(i64),
                                  P(i64), P(i64), P(i64)]
        L.orc_vogel_steps.argtypes = [i32, i32, P(i32), P(i32), P(ctypes.c_float), i32, P(i32), P(i32),
                                      P(ctypes.c_float), P(i32)]
        L.orc_sweep.argtypes = [i32, i32, P(ctypes.c_float), P(ctypes.c_float), P(i32), P(i32)]
        L.orc_sweep.restype = ctypes.c_float
        L.orc_generate.argtypes = [i32, ctypes.c_uint64, i32, i32, i32, i32, i32, i32, P(i32), P(i32), P(i32)]
        L.orc_generate_sizes.argtypes = [ctypes.c_uint64, i32, i32, i32, P(i32), P(i32)]
        _orc = L
    return _orc


def ref_available() -> bool:
    return os.path.exists(REF)


def ref() -> ctypes.CDLL:
    global _ref
    if _ref is None:
        L = ctypes.CDLL(REF)
        L.ref_vogel.argtypes = [ctypes.c_int, ctypes.c_int, P(ctypes.c_int), P(ctypes.c_int), P(ctypes.c_float),
                                P(ctypes.c_int), P(ctypes.c_int), P(ctypes.c_float)]
        L.ref_solve.argtypes = [ctypes.c_int, ctypes.c_int, P(ctypes.c_int), P(ctypes.c_int), P(ctypes.c_float),
                                ctypes.c_int, P(ctypes.c_int), P(ctypes.c_double), P(ctypes.c_int),
                                P(ctypes.c_int), P(ctypes.c_int), P(ctypes.c_float), P(ctypes.c_int)]
        _ref = L
    return _ref


def _p(a, t=i32):
    return a.ctypes.data_as(P(t))


def _prep(s, d, c):
    s = np.ascontiguousarray(s, dtype=np.int32)
    d = np.ascontiguousarray(d, dtype=np.int32)
    cf = np.ascontiguousarray(np.asarray(c).reshape(-1), dtype=np.float32)
    return s, d, cf


def vogel(s, d, c):
    """Reference Vogel (float costs).  Returns (src, dst, qty float32, events)."""
    s, d, cf = _prep(s, d, c)
    m, n = len(s), len(d)
    src = np.zeros(m + n - 1, np.int32)
    dst = np.zeros(m + n - 1, np.int32)
    q = np.zeros(m + n - 1, np.float32)
    ev = orc().orc_vogel(m, n, _p(s), _p(d), _p(cf, ctypes.c_float), _p(src), _p(dst), _p(q, ctypes.c_float))
    return src, dst, q, int(ev)


def vogel_device(s, d, c):
    """The reference's device Vogel ("vam_device", float costs).  Returns
    (src, dst, qty float32, rc); rc -1: undefined in the reference from the
    first (-1, -1) flow on."""
    s, d, cf = _prep(s, d, c)
    m, n = len(s), len(d)
    src = np.zeros(m + n - 1, np.int32)
    dst = np.zeros(m + n - 1, np.int32)
    q = np.zeros(m + n - 1, np.float32)
    rc = orc().orc_vogel_device(m, n, _p(s), _p(d), _p(cf, ctypes.c_float), _p(src), _p(dst),
                                _p(q, ctypes.c_float))
    return src, dst, q, int(rc)


def vogel_steps(s, d, c, max_steps: int):
    """The reference Vogel stopped after max_steps allocations.  Returns
    (src, dst, qty float32, events, steps made)."""
    s, d, cf = _prep(s, d, c)
    m, n = len(s), len(d)
    src = np.zeros(m + n - 1, np.int32)
    dst = np.zeros(m + n - 1, np.int32)
    q = np.zeros(m + n - 1, np.float32)
    k = i32()
    ev = orc().orc_vogel_steps(m, n, _p(s), _p(d), _p(cf, ctypes.c_float), max_steps, _p(src), _p(dst),
                               _p(q, ctypes.c_float), ctypes.byref(k))
    return src, dst, q, int(ev), int(k.value)


def sweep(c, h):
    """One sequential reduced-cost scan (float).  c: (m, n) costs, h: m row
    duals then n column duals.  Returns (min reduced cost, row, col)."""
    cf = np.ascontiguousarray(c, dtype=np.float32)
    m, n = cf.shape
    hf = np.ascontiguousarray(h, dtype=np.float32)
    assert hf.shape == (m + n,)
    r, q = i32(), i32()
    v = orc().orc_sweep(m, n, _p(cf, ctypes.c_float), _p(hf, ctypes.c_float), ctypes.byref(r), ctypes.byref(q))
    return float(v), int(r.value), int(q.value)


def generate(kind: int, seed: int, m: int, n: int, c_lo: int, c_hi: int, q_lo: int, q_hi: int):
    """The benchmark's instance generator (same integers as the library's
    flock_generate).  Returns (supply, demand, cost (m, n))."""
    s = np.empty(m, np.int32)
    d = np.empty(n, np.int32)
    c = np.empty((m, n), np.int32)
    if orc().orc_generate(kind, seed, m, n, c_lo, c_hi, q_lo, q_hi, _p(s), _p(d), _p(c)):
        raise ValueError("bad generator arguments")
    return s, d, c


def generate_sizes(seed: int, count: int, lo: int, hi: int):
    ms = np.empty(count, np.int32)
    ns = np.empty(count, np.int32)
    if orc().orc_generate_sizes(seed, count, lo, hi, _p(ms), _p(ns)):
        raise ValueError("bad size arguments")
    return ms, ns


def mixed_batch(seed: int, count: int, lo: int, hi: int):
    """The batched workload as (supply, demand, cost) triples: m and n
    log-uniform in [lo, hi], costs 1..1000, quantities 100..1000 (the same
    instances as the library's batch generator for the same seed)."""
    ms, ns = generate_sizes(seed, count, lo, hi)
    return [generate(0, seed * 1000003 + k + 1, int(ms[k]), int(ns[k]), 1, 1000, 100, 1000) for k in range(count)]


def nwc(s, d):
    s = np.ascontiguousarray(s, dtype=np.int32)
    d = np.ascontiguousarray(d, dtype=np.int32)
    m, n = len(s), len(d)
    src = np.zeros(m + n - 1, np.int32)
    dst = np.zeros(m + n - 1, np.int32)
    q = np.zeros(m + n - 1, np.float32)
    orc().orc_nwc(m, n, _p(s), _p(d), _p(src), _p(dst), _p(q, ctypes.c_float))
    return src, dst, q


def solve_ref(s, d, c, bfs: int = 1, max_iter: int = 30000):
    """Reference CPU path.  Returns dict(iterations, status, objective, flows, tree)."""
    s, d, cf = _prep(s, d, c)
    m, n = len(s), len(d)
    V = m + n
    fs, fd = np.zeros(V, np.int32), np.zeros(V, np.int32)
    fq = np.zeros(V, np.float32)
    ts, td = np.zeros(V, np.int32), np.zeros(V, np.int32)
    r = OrcResult()
    orc().orc_solve_ref(m, n, _p(s), _p(d), _p(cf, ctypes.c_float), bfs, max_iter, _p(fs), _p(fd),
                        _p(fq, ctypes.c_float), _p(ts), _p(td), ctypes.byref(r))
    a = r.active_flows
    return dict(iterations=r.iterations, status=r.status, objective=r.objective, active=a,
                vogel_events=r.vogel_events, flows=np.stack([fs[:a], fd[:a], fq[:a].astype(np.int64)], 1),
                tree=np.stack([ts[:V - 1], td[:V - 1]], 1))


def solve_ref_batch(insts: Sequence, nthreads: int, bfs: int = 1, max_iter: int = 30000):
    """insts: sequence of (s, d, c).  Returns (objectives, iterations, status)."""
    k = len(insts)
    ms = np.array([len(x[0]) for x in insts], np.int32)
    ns = np.array([len(x[1]) for x in insts], np.int32)
    so = np.zeros(k, np.int64); do = np.zeros(k, np.int64); co = np.zeros(k, np.int64)
    so[1:] = np.cumsum(ms)[:-1]; do[1:] = np.cumsum(ns)[:-1]; co[1:] = np.cumsum(ms.astype(np.int64) * ns)[:-1]
    S = np.ascontiguousarray(np.concatenate([np.asarray(x[0], np.int32) for x in insts]))
    D = np.ascontiguousarray(np.concatenate([np.asarray(x[1], np.int32) for x in insts]))
    C = np.ascontiguousarray(np.concatenate([np.asarray(x[2], np.float32).reshape(-1) for x in insts]))
    obj = np.zeros(k, np.float64); it = np.zeros(k, np.int32); st = np.zeros(k, np.int32)
    orc().orc_solve_ref_batch(k, _p(ms), _p(ns), _p(so, i64), _p(do, i64), _p(co, i64), _p(S), _p(D),
                              _p(C, ctypes.c_float), bfs, max_iter, nthreads,
                              _p(obj, ctypes.c_double), _p(it), _p(st))
    return obj, it, st


def tree_duals(c_int, tree):
    c = np.ascontiguousarray(c_int, dtype=np.int32)
    m, n = c.shape
    ts = np.ascontiguousarray(tree[:, 0], dtype=np.int32)
    td = np.ascontiguousarray(tree[:, 1], dtype=np.int32)
    u = np.zeros(m, np.int64); v = np.zeros(n, np.int64)
    ok = orc().orc_tree_duals(m, n, _p(c), len(ts), _p(ts), _p(td), _p(u, i64), _p(v, i64))
    return ok, u, v


def certify(s, d, c_int, flows, u, v):
    """Exact certificate.  flows: (k, 3) ints.  Returns (bits, objective)."""
    s = np.ascontiguousarray(s, dtype=np.int32)
    d = np.ascontiguousarray(d, dtype=np.int32)
    c = np.ascontiguousarray(c_int, dtype=np.int32)
    f = np.asarray(flows)
    fs = np.ascontiguousarray(f[:, 0], dtype=np.int32)
    fd = np.ascontiguousarray(f[:, 1], dtype=np.int32)
    fq = np.ascontiguousarray(f[:, 2], dtype=np.int64)
    u = np.ascontiguousarray(u, dtype=np.int64)
    v = np.ascontiguousarray(v, dtype=np.int64)
    obj = i64()
    bits = orc().orc_certify(len(s), len(d), _p(s), _p(d), _p(c), len(fs), _p(fs), _p(fd), _p(fq, i64),
                             _p(u, i64), _p(v, i64), ctypes.byref(obj))
    return int(bits), int(obj.value)


def ref_vogel(s, d, c):
    """The reference's own find_vogel_bfs_sequencial (oracle/_ref)."""
    s, d, cf = _prep(s, d, c)
    m, n = len(s), len(d)
    src = np.zeros(m + n - 1, np.int32); dst = np.zeros(m + n - 1, np.int32); q = np.zeros(m + n - 1, np.float32)
    ref().ref_vogel(m, n, _p(s, ctypes.c_int), _p(d, ctypes.c_int), _p(cf, ctypes.c_float),
                    _p(src, ctypes.c_int), _p(dst, ctypes.c_int), _p(q, ctypes.c_float))
    return src, dst, q


def ref_solve(s, d, c, max_iter: int = 30000):
    """The reference's own CPU path (oracle/_ref)."""
    s, d, cf = _prep(s, d, c)
    m, n = len(s), len(d)
    V = m + n
    it, obj, act, st = ctypes.c_int(), ctypes.c_double(), ctypes.c_int(), ctypes.c_int()
    fs = np.zeros(V, np.int32); fd = np.zeros(V, np.int32); fq = np.zeros(V, np.float32)
    ref().ref_solve(m, n, _p(s, ctypes.c_int), _p(d, ctypes.c_int), _p(cf, ctypes.c_float), max_iter,
                    ctypes.byref(it), ctypes.byref(obj), ctypes.byref(act), _p(fs, ctypes.c_int),
                    _p(fd, ctypes.c_int), _p(fq, ctypes.c_float), ctypes.byref(st))
    a = act.value
    return dict(iterations=it.value, status=st.value, objective=obj.value, active=a,
                flows=np.stack([fs[:a], fd[:a], fq[:a].astype(np.int64)], 1))


def verdict(s, d, c_int, r):
    """Classify a result of solve_ref with the exact certificate:
    'optimal' (its basis is a spanning tree whose exact duals certify the
    flows), 'feasible' (flows satisfy every constraint, not certified),
    'infeasible', or 'stopped' (forest guard / cap with infeasible flows)."""
    c = np.asarray(c_int, dtype=np.int32).reshape(len(s), len(d))
    ok, u, v = tree_duals(c, r["tree"])
    bits, _ = certify(s, d, c, r["flows"], u, v)
    if ok == 0 and bits == 0 and r["status"] == 0:
        return "optimal"
    if bits & 7 == 0:
        return "feasible"
    return "infeasible" if r["status"] == 0 else "stopped"

