"""Regenerates the golden fixtures in this folder from the REFERENCE ITSELF:
the reference's own CPU-path functions compiled from its sources into
oracle/_ref (see oracle/Makefile), plus its published run logs.

    make -C oracle ref REF=<reference checkout>
    python tests/golden/make_golden.py <reference checkout>

Outputs (committed):
  reference_fixtures.json  small instance files from the reference's tests/
                           folder (costs as exact integers x 10^scale) with
                           the reference's Vogel allocations and solve result
  reference_random.json    the reference's Vogel + solve results on seeded
                           tiny degenerate instances (regenerated by seed)
  reference_synthetic.json the reference's results on generator instances
                           (regenerated by the product's generator; checksum)
  published.json           iterations/objectives of the published CPU-path,
                           GPU uv-path and Gurobi logs (results/pure_sequencial,
                           parallel_uv, gurobi); `--published-only` rewrites
                           just this file
"""
import ctypes
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

import oracle  # noqa: E402
from golden_util import checksum, float_costs, tiny  # noqa: E402

FIXTURES = ["test_simple1.dat", "test_simple2.dat", "test_simple3.dat", "test_simple4.dat",
            "test_simple1_degenerate.dat", "test_TransportModel_10_10_0.dat",
            "test_TransportModel_5_10_1.dat", "test_TransportModel_5_25_1.dat",
            "test_TransportModel_25_25_1.dat", "test_TransportModel_25_50_1.dat",
            "test_TransportModel_50_50_1.dat", "test_TransportModel_100_100_0.dat",
            "test_TransportModel_100_100_1.dat", "test_TransportModel_100_100_6.dat"]


def read_tokens(path):
    tok = open(path).read().split()
    m, n = int(tok[0]), int(tok[1])
    s = [int(x) for x in tok[2:2 + m]]
    d = [int(x) for x in tok[2 + m:2 + m + n]]
    c = tok[2 + m + n:2 + m + n + m * n]
    return m, n, s, d, c


def exact_scaled(c, scale):
    out = []
    for x in c:
        neg = x.startswith("-")
        x = x.lstrip("+-")
        ip, _, fp = x.partition(".")
        fp = (fp + "0" * scale)[:scale]
        v = int(ip or "0") * 10 ** scale + int(fp or "0")
        out.append(-v if neg else v)
    return out


_libc = ctypes.CDLL("libc.so.6")
_libc.strtof.restype = ctypes.c_float
_libc.strtof.argtypes = [ctypes.c_char_p, ctypes.c_void_p]


def _strtof(x):
    return _libc.strtof(x.encode(), None)


def ref_outputs(s, d, cf):
    src, dst, q = oracle.ref_vogel(s, d, cf)
    r = oracle.ref_solve(s, d, cf)
    return {"vogel_src": src.tolist(), "vogel_dst": dst.tolist(), "vogel_qty": [float(v) for v in q],
            "iterations": r["iterations"], "status": r["status"], "objective": r["objective"],
            "active": r["active"]}


def write_published(refdir):
    """Iterations and objectives of the published run logs: the CPU path
    (vam_host BFS), the GPU uv path (vam_device BFS, host duals, sequential
    cycle search) and Gurobi."""
    pub = {"pure_sequencial": {}, "parallel_uv": {}, "gurobi": {}}
    for key in pub:
        lines = open(os.path.join(refdir, "results", key)).read().splitlines()
        fname = None
        for ln in lines:
            mm = re.search(r"File Name = \S*/(\S+\.dat)", ln)
            if mm:
                fname = mm.group(1)
            mm = re.search(r"BASIC STATISTICS \| Objective: (\S+) \| Iterations: (\d+) \| Time: (\d+)", ln)
            if mm and fname:
                pub[key][fname] = {"objective": mm.group(1), "iterations": int(mm.group(2)),
                                   "time_ms": int(mm.group(3))}
            mm = re.search(r"Optimal objective\s+(\S+)", ln)
            if mm and fname and key == "gurobi":
                pub[key].setdefault(fname, {})["optimal"] = mm.group(1)
    json.dump(pub, open(os.path.join(HERE, "published.json"), "w"), indent=1)


def main(refdir):
    assert oracle.ref_available(), "build oracle/_ref first (make -C oracle ref)"
    # 1. the reference's own test fixtures
    fx = []
    for f in FIXTURES:
        m, n, s, d, c = read_tokens(os.path.join(refdir, "tests", f))
        scale = max((len(x.split(".")[1].rstrip("0")) if "." in x else 0) for x in c)
        ci = exact_scaled(c, scale)
        cf = np.array([_strtof(x) for x in c], np.float32)   # what the reference's stream parse gives
        e = {"file": f, "m": m, "n": n, "scale": scale, "supply": s, "demand": d, "cost": ci}
        if not np.array_equal(cf, float_costs(ci, scale)):   # store only when not reconstructible
            e["cost_f32"] = [float(v) for v in cf]
        e.update(ref_outputs(np.array(s, np.int32), np.array(d, np.int32), cf))
        fx.append(e)
    json.dump(fx, open(os.path.join(HERE, "reference_fixtures.json"), "w"), separators=(",", ":"))
    # 2. tiny degenerate instances (regenerated by seed in the tests)
    rnd = []
    for (s, d, c) in tiny(101, 300):
        rnd.append(ref_outputs(s, d, c.astype(np.float32)))
    json.dump({"seed": 101, "count": 300, "max_dim": 8, "results": rnd},
              open(os.path.join(HERE, "reference_random.json"), "w"), separators=(",", ":"))
    # 3. generator instances (regenerated by the product's generator)
    import flock_gb300 as fg
    syn = []
    for name, seed, m, n in [("uniform100", 0, None, None), ("uniform100", 1, None, None),
                             ("uniform100", 2, None, None), ("degenerate1000", 0, 200, 200),
                             ("degenerate1000", 1, 300, 250), ("euclid8000", 0, 150, 200)]:
        inst = fg.config_instance(name, seed, m=m, n=n)
        e = {"name": name, "seed": seed, "m": inst.m, "n": inst.n,
             "checksum": checksum(inst.supply, inst.demand, inst.cost)}
        e.update(ref_outputs(inst.supply, inst.demand, inst.cost.astype(np.float32)))
        syn.append(e)
    json.dump(syn, open(os.path.join(HERE, "reference_synthetic.json"), "w"), separators=(",", ":"))
    # 4. published logs
    write_published(refdir)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if a != "--published-only"]
    ref = args[0] if args else os.environ.get("FLOCK_REFERENCE", "/root/reference")
    if "--published-only" in sys.argv:
        write_published(ref)       # the run logs only (no reference build needed)
    else:
        main(ref)
