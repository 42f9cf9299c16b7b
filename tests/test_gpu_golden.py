"""GPU vs the reference itself: golden outputs of the reference's own
functions (tests/golden, made from the reference build) -- Vogel
allocations bit-identical and optimal objectives identical, every solution
certified exactly."""
import json
import os

import numpy as np
import pytest

import flock_gb300 as fg
import oracle
from conftest import GOLDEN
from golden_util import checksum, tiny

pytestmark = pytest.mark.gpu


def load(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


def vogel_equal(inst, e):
    gv, ev = fg.vogel(inst)
    src, dst, q = (np.array(e["vogel_src"]), np.array(e["vogel_dst"]), np.array(e["vogel_qty"], np.float32))
    if ev < 0:
        k = int(np.argmax(gv[:, 0] < 0))
        gv, src, dst, q = gv[:k], src[:k], dst[:k], q[:k]
    assert gv[:, 0].tolist() == src.tolist()
    assert gv[:, 1].tolist() == dst.tolist()
    assert gv[:, 2].tolist() == np.where(q < 0.5, 0, q).astype(np.int64).tolist()


def certified(inst, res):
    assert res.status == 0 and res.certified
    bits, obj = oracle.certify(inst.supply, inst.demand, inst.cost, res.flows, res.u, res.v)
    assert bits == 0 and obj == res.objective


@pytest.mark.parametrize("e", load("reference_fixtures.json"), ids=lambda e: e["file"])
def test_reference_fixtures(e):
    inst = fg.Instance(np.array(e["supply"], np.int32), np.array(e["demand"], np.int32),
                       np.array(e["cost"], np.int32).reshape(e["m"], e["n"]))
    if e["scale"] == 0:
        vogel_equal(inst, e)
    for pivot in ("parallel", "sequential", "switch"):
        res = fg.solve(inst, pivot=pivot)
        certified(inst, res)
        if e["status"] == 0 and e["scale"] == 0:
            live = oracle.solve_ref(inst.supply, inst.demand, inst.cost)
            assert oracle.verdict(inst.supply, inst.demand, inst.cost, live) == "optimal"
            assert res.objective == int(round(e["objective"]))
        elif e["status"] == 0:   # the reference computes in float on non-exact decimals
            assert abs(res.objective / 10 ** e["scale"] - e["objective"]) < 1.0
        else:       # the reference stopped early (forest): ours is optimal, so no worse
            assert res.objective / 10 ** e["scale"] <= e["objective"] + 1e-6


def test_reference_random():
    g = load("reference_random.json")
    for (s, d, c), e in zip(tiny(g["seed"], g["count"], g["max_dim"]), g["results"]):
        inst = fg.Instance(s, d, c)
        vogel_equal(inst, e)
        res = fg.solve(inst)
        certified(inst, res)
        live = oracle.solve_ref(s, d, c)      # pinned to the golden entry by test_oracle_pin
        if live["status"] == 3:               # undefined in the reference (out-of-range index)
            continue
        assert live["objective"] == e["objective"]
        v = oracle.verdict(s, d, c, live)
        if v == "optimal":
            assert res.objective == int(round(e["objective"]))
        elif v == "feasible":
            assert res.objective <= int(round(e["objective"]))


@pytest.mark.parametrize("e", load("reference_synthetic.json"), ids=lambda e: f"{e['name']}-{e['seed']}")
def test_reference_synthetic(e):
    inst = fg.config_instance(e["name"], e["seed"], m=e["m"], n=e["n"])
    assert checksum(inst.supply, inst.demand, inst.cost) == e["checksum"]
    vogel_equal(inst, e)
    res = fg.solve(inst)
    certified(inst, res)
    live = oracle.solve_ref(inst.supply, inst.demand, inst.cost)
    assert oracle.verdict(inst.supply, inst.demand, inst.cost, live) == "optimal"
    assert e["status"] == 0 and res.objective == int(round(e["objective"]))
