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
    big = max(fg.Server.request_bytes(x.m, x.n) for x in insts)
    srv = fg.Server(memory_budget_bytes=big, max_inflight_batches=2, max_batch=8)
    for x in insts:
        srv.submit(x)
    srv.drain()
    res = srv.poll()
    srv.close()
    assert len(res) == len(insts)
    assert all(r[1] == 0 and r[5] for r in res)


def test_served_backfill_no_head_of_line_blocking():
    """A large instance is on the GPU; small requests that arrive after it are
    admitted, overlap with it and retire before it does."""
    big = fg.generate(0, 77, 1800, 1900, 1, 1000, 100, 1000)
    small = [fg.generate(0, 78 + k, 20 + k, 25, 1, 1000, 100, 1000) for k in range(24)]
    srv = fg.Server()
    t_big = srv.submit(big)
    time.sleep(0.02)
    t_small = [srv.submit(x) for x in small]
    order = []
    res = {}
    while len(order) < 1 + len(small):
        for r in srv.poll():
            order.append(r[0])
            res[r[0]] = r
        time.sleep(0.001)
    srv.close()
    assert all(res[t][1] == 0 and res[t][5] for t in order)
    assert order[-1] == t_big, "small requests waited behind the large one"
    assert max(res[t][3] for t in t_small) < res[t_big][3]
    assert res[t_big][2] == fg.solve(big).objective


def test_served_plain_path_request():
    """m + n above the staged limit: solved by the plain solver inside the server."""
    inst = fg.generate(0, 79, 2100, 2050, 1, 1000, 100, 1000)
    small = fg.generate(0, 80, 30, 40, 1, 1000, 100, 1000)
    srv = fg.Server()
    srv.submit(inst)
    srv.submit(small)
    srv.drain()
    res = srv.poll()
    srv.close()
    assert len(res) == 2 and all(r[1] == 0 and r[5] for r in res)
    objs = sorted(r[2] for r in res)
    assert objs == sorted([fg.solve(inst).objective, fg.solve(small).objective])
