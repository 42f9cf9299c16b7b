"""GPU: served form (continuous batching).  Requests submitted while others
run are admitted as launch slots and budget free up; each result must equal
the instance solved alone (exact objective) and carry the certificate."""
import time

import numpy as np
import pytest

import flock_gb300 as fg
import oracle

pytestmark = pytest.mark.gpu


def test_served_results_equal_alone():
    insts = fg.mixed_batch(17, 120, 10, 300)
    srv = fg.Server(memory_budget_bytes=64 << 20, max_inflight_batches=3, max_batch=16)
    tickets = {}
    for k, x in enumerate(insts):
        tickets[srv.submit(x)] = k
        if k % 10 == 0:
            time.sleep(0.002)        # arrivals while earlier launches run
    srv.drain()
    got = {}
    while len(got) < len(insts):
        for (t, status, obj, lat, st, cert) in srv.poll():
            got[tickets[t]] = (status, obj, lat, st, cert)
    srv.close()
    for k, x in enumerate(insts):
        status, obj, lat, st, cert = got[k]
        assert status == 0 and st == 0 and cert and lat > 0
        alone = fg.solve(x)
        assert alone.status == 0 and alone.objective == obj
        bits, o = oracle.certify(x.supply, x.demand, x.cost, alone.flows, alone.u, alone.v)
        assert bits == 0 and o == obj


def test_served_budget_serialises():
    """A budget that fits one request at a time still completes everything."""
    insts = fg.mixed_batch(5, 12, 20, 60)
    big = max(4 * x.m * ((x.n + 3) // 4 * 4) + 256 * (x.m + x.n) + 4096 for x in insts)
    srv = fg.Server(memory_budget_bytes=big, max_inflight_batches=2, max_batch=8)
    for x in insts:
        srv.submit(x)
    srv.drain()
    res = srv.poll()
    srv.close()
    assert len(res) == len(insts)
    assert all(r[1] == 0 and r[5] for r in res)
