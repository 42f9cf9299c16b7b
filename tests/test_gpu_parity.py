"""GPU parity: the CUDA path through the C ABI against the oracle (the
reference CPU path restated in C) on the same seeded inputs.

Bar: Vogel allocations bit-identical; objective identical wherever the
reference path's own result is optimal (its final basis and exact duals pass
the certificate -- on degenerate input the reference can report optimality
with a basis that is not a tree), never worse elsewhere; every GPU solution
passes the exact int64 certificate (feasibility, all reduced costs >= 0,
complementary slackness)."""
import numpy as np
import pytest

import flock_gb300 as fg
import oracle

pytestmark = pytest.mark.gpu


def tiny_instances(seed, count, max_dim=8):
    rng = np.random.default_rng(seed)
    out = []
    while len(out) < count:
        m = int(rng.integers(1, max_dim + 1)); n = int(rng.integers(1, max_dim + 1))
        if m + n < 3:
            continue
        hi = int(rng.choice([3, 5, 20, 100]))
        c = rng.integers(0, hi, size=(m, n)).astype(np.int32)
        qh = int(rng.choice([2, 4, 10, 50]))
        s = rng.integers(0, qh, size=m).astype(np.int32)
        d = rng.integers(0, qh, size=n).astype(np.int32)
        diff = int(s.sum() - d.sum())
        if diff > 0:
            d[-1] += diff
        else:
            s[-1] -= diff
        out.append(fg.Instance(s, d, c))
    return out


def assert_vogel_parity(inst):
    gpu, ev = fg.vogel(inst)
    src, dst, q, oev = oracle.vogel(inst.supply, inst.demand, inst.cost)
    assert ev == oev
    if oev < 0:      # the reference is undefined from the first (-1) entry on
        k = int(np.argmax(src < 0))
        src, dst, q, gpu = src[:k], dst[:k], q[:k], gpu[:k]
    qi = np.where(q < 0.5, 0, q).astype(np.int64)     # the reference writes 1e-6 for zero
    np.testing.assert_array_equal(gpu[:, 0], src)
    np.testing.assert_array_equal(gpu[:, 1], dst)
    np.testing.assert_array_equal(gpu[:, 2].astype(np.int64), qi)


def assert_optimal(inst, res, ref=None):
    assert res.status == 0, f"status {res.status}"
    assert res.certified
    bits, obj = oracle.certify(inst.supply, inst.demand, inst.cost, res.flows, res.u, res.v)
    assert bits == 0, f"certificate bits {bits}"
    assert obj == res.objective
    if ref is None:
        ref = oracle.solve_ref(inst.supply, inst.demand, inst.cost)
    v = oracle.verdict(inst.supply, inst.demand, inst.cost, ref)
    if v == "optimal":        # the reference's own result is certified: same optimum
        assert res.objective == int(round(ref["objective"]))
    elif v == "feasible":     # the reference stopped short of the optimum
        assert res.objective <= int(round(ref["objective"]))
    return ref


def test_vogel_tiny_degenerate():
    for inst in tiny_instances(11, 400):
        assert_vogel_parity(inst)


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_vogel_uniform100(seed):
    assert_vogel_parity(fg.config_instance("uniform100", seed))


def test_vogel_degenerate_shape():
    assert_vogel_parity(fg.config_instance("degenerate1000", 3, m=300, n=250))


def test_vogel_euclid_shape():
    assert_vogel_parity(fg.config_instance("euclid8000", 5, m=200, n=300))


def assert_vogel_device_parity(inst):
    """The reference's device Vogel ("vam_device"): every allocation and the
    undefined marker bit-identical to the oracle's restatement (both write
    (-1, -1, 0) from the step where the reference indexes past its arrays)."""
    gpu, ev = fg.vogel_device(inst)
    src, dst, q, rc = oracle.vogel_device(inst.supply, inst.demand, inst.cost)
    assert (ev < 0) == (rc < 0)
    qi = np.where(q < 0.5, 0, q).astype(np.int64)     # the reference writes 1e-6 for zero
    np.testing.assert_array_equal(gpu[:, 0], src)
    np.testing.assert_array_equal(gpu[:, 1], dst)
    np.testing.assert_array_equal(gpu[:, 2].astype(np.int64), qi)
    return rc


def test_vogel_device_tiny_degenerate():
    for inst in tiny_instances(31, 400):
        assert_vogel_device_parity(inst)


@pytest.mark.parametrize("name,seed,m,n", [("uniform100", 0, None, None), ("uniform100", 1, None, None),
                                           ("degenerate1000", 0, None, None), ("euclid8000", 5, 200, 300)])
def test_vogel_device_shapes(name, seed, m, n):
    assert assert_vogel_device_parity(fg.config_instance(name, seed, m=m, n=n)) == 0


def test_vogel_device_sentinel_costs():
    """Costs around the reference's 32767 book sentinels: defined runs agree,
    and so does the step where the reference's run becomes undefined."""
    rng = np.random.default_rng(77)
    undefined = 0
    for _ in range(60):
        m, n = int(rng.integers(1, 30)), int(rng.integers(1, 30))
        c = rng.integers(32760, 32776, size=(m, n)).astype(np.int32)
        s = rng.integers(0, 20, size=m).astype(np.int32)
        d = rng.integers(0, 20, size=n).astype(np.int32)
        diff = int(s.sum() - d.sum())
        if diff > 0:
            d[-1] += diff
        else:
            s[-1] -= diff
        undefined += assert_vogel_device_parity(fg.Instance(s, d, c)) < 0
    assert undefined > 0


def test_vogel_device_line_limit():
    inst = fg.Instance(np.ones(16383, np.int32), np.array([16383], np.int32), np.ones((16383, 1), np.int32))
    with pytest.raises(fg.FlockError) as ex:
        fg.vogel_device(inst)
    assert ex.value.status == fg.FLOCK_ERR_RANGE


@pytest.mark.parametrize("pivot", ["sequential", "switch"])
def test_solve_vam_device_start(pivot):
    """flock_solve from the device-Vogel start: optimal and certified, the
    objective of the reference path run from the same start."""
    for inst in tiny_instances(41, 60) + [fg.config_instance("uniform100", 3),
                                          fg.config_instance("degenerate1000", 2, m=300, n=250)]:
        ref = oracle.solve_ref(inst.supply, inst.demand, inst.cost, bfs=2)
        assert_optimal(inst, fg.solve(inst, bfs="vam_device", pivot=pivot), ref)


def test_facade_bfs_method_switch(monkeypatch):
    """The model classes follow the BFS_METHOD switch as the reference's
    compile-time define: vam_device reaches the same optimum."""
    inst = fg.config_instance("uniform100", 4)
    prob = fg.ProblemInstance()
    prob.numSupplies, prob.numDemands = inst.m, inst.n
    prob.supplies, prob.demands, prob.int_costs, prob.cost_scale = inst.supply, inst.demand, inst.cost, 0
    objs = []
    for bfs in ["vam_host", "vam_device"]:
        monkeypatch.setattr(fg, "BFS_METHOD", bfs)
        model = fg.uvModel_parallel(prob, [])
        model.execute()
        objs.append(model.objVal)
    ref = oracle.solve_ref(inst.supply, inst.demand, inst.cost, bfs=2)
    assert objs[0] == objs[1] == round(ref["objective"])


def test_vam_device_batch_rejected():
    inst = fg.config_instance("uniform100", 0)
    with pytest.raises(fg.FlockError) as ex:
        fg.batch_solve([inst], bfs="vam_device")
    assert ex.value.status == fg.FLOCK_ERR_ARG


@pytest.mark.parametrize("pivot", ["parallel", "sequential", "switch"])
def test_solve_tiny(pivot):
    for inst in tiny_instances(23, 150):
        res = fg.solve(inst, pivot=pivot)
        assert_optimal(inst, res)


@pytest.mark.parametrize("pivot", ["parallel", "sequential", "switch"])
@pytest.mark.parametrize("seed", [0, 1])
def test_solve_uniform100(pivot, seed):
    inst = fg.config_instance("uniform100", seed)
    assert_optimal(inst, fg.solve(inst, pivot=pivot))


def test_solve_nwc_start():
    inst = fg.config_instance("uniform100", 7)
    res = fg.solve(inst, bfs="nwc")
    assert_optimal(inst, res)


def test_solve_degenerate_mid():
    inst = fg.config_instance("degenerate1000", 1, m=400, n=300)
    assert_optimal(inst, fg.solve(inst))


@pytest.mark.parametrize("pivot", ["parallel", "switch"])
def test_degenerate_1000_full_size(pivot):
    """The 1000 x 1000 degenerate-prone workload itself (costs 1..20,
    quantities 1..50, seed 0) with parallel pivots and deconfliction: the
    reference path's own result is optimal here, and the objective must be
    identical to it (int64)."""
    inst = fg.config_instance("degenerate1000", 0)
    ref = oracle.solve_ref(inst.supply, inst.demand, inst.cost)
    assert oracle.verdict(inst.supply, inst.demand, inst.cost, ref) == "optimal"
    res = fg.solve(inst, pivot=pivot)
    assert_optimal(inst, res, ref)
    assert res.objective == int(round(ref["objective"]))
    b = fg.batch_solve([inst], pivot=pivot)[0]          # batched results carry no duals
    assert b.status == 0 and b.certified and b.objective == res.objective


@pytest.mark.parametrize("shape", [(1, 1), (1, 7), (6, 1), (2, 2), (3, 50), (50, 3)])
def test_edge_shapes(shape):
    m, n = shape
    rng = np.random.default_rng(m * 100 + n)
    s = rng.integers(0, 20, m).astype(np.int32)
    d = np.zeros(n, np.int32)
    d[:] = s.sum() // n
    d[-1] += s.sum() - d.sum()
    c = rng.integers(1, 30, (m, n)).astype(np.int32)
    inst = fg.Instance(s, d, c)
    assert_vogel_parity(inst)
    assert_optimal(inst, fg.solve(inst))


def test_zero_quantities():
    m, n = 6, 7
    rng = np.random.default_rng(5)
    c = rng.integers(1, 9, (m, n)).astype(np.int32)
    s = np.array([0, 4, 0, 3, 0, 5], np.int32)
    d = np.array([0, 0, 6, 0, 6, 0, 0], np.int32)
    inst = fg.Instance(s, d, c)
    assert_optimal(inst, fg.solve(inst))
    inst0 = fg.Instance(np.zeros(m, np.int32), np.zeros(n, np.int32), c)
    res = fg.solve(inst0)
    assert res.status == 0 and res.objective == 0


def test_batch_matches_plain():
    insts = fg.mixed_batch(3, 64, 10, 120)
    out = fg.batch_solve(insts)
    for inst, r in zip(insts, out):
        p = fg.solve(inst)
        assert r.status == 0 and r.certified
        assert r.objective == p.objective
        bits, obj = oracle.certify(inst.supply, inst.demand, inst.cost, r.flows, p.u, p.v)
        assert obj == r.objective


@pytest.mark.parametrize("form", ["persistent", "round"])
def test_batch_forms_all_buckets(form, monkeypatch):
    """Both batched forms on instances from every size bucket (V up to 4096,
    the last bucket with light staging) plus one above it (plain path):
    certified optima equal to the plain solver's, and the same pricing
    rounds in both forms."""
    monkeypatch.setenv("FLOCK_BATCH_FORM", form)
    shapes = [(5, 7), (30, 30), (60, 60), (100, 150), (200, 300), (400, 500), (900, 1000),
              (1500, 1444), (1000, 2072), (1600, 1600), (2000, 2000), (2100, 2000), (12, 40), (3, 3)]
    insts = [fg.generate(0, 500 + k, m, n, 1, 1000, 100, 1000) for k, (m, n) in enumerate(shapes)]
    insts += fg.mixed_batch(17, 96, 10, 300)
    out = fg.batch_solve(insts, pricing="full")      # the plain solver prices fully
    for k, (inst, r) in enumerate(zip(insts, out)):
        assert r.status == 0 and r.certified, (k, inst.m, inst.n, r.status)
        if inst.m * inst.n <= 300 * 300 or k < len(shapes):
            p = fg.solve(inst, pricing="full")
            assert r.objective == p.objective, (k, inst.m, inst.n)
            assert r.iterations == p.iterations, (k, inst.m, inst.n)


def test_batch_validation_first_failure():
    """The batch reports the first failing instance's first failing check,
    as validate_instance would one instance at a time."""
    good = [fg.generate(0, 900 + k, 20 + k, 30, 1, 100, 10, 50) for k in range(8)]
    bad_cost = fg.generate(0, 950, 25, 25, 1, 100, 10, 50)
    bad_cost.cost = bad_cost.cost.copy()
    bad_cost.cost[3, 7] = (1 << 30) + 1
    bad_supply = fg.generate(0, 951, 25, 25, 1, 100, 10, 50)
    bad_supply.supply = bad_supply.supply.copy()
    bad_supply.supply[0] = -1
    with pytest.raises(RuntimeError) as e1:
        fg.batch_solve(good[:3] + [bad_cost] + good[3:5] + [bad_supply] + good[5:])
    assert "cost out of range" in str(e1.value)
    with pytest.raises(RuntimeError) as e2:
        fg.batch_solve(good[:3] + [bad_supply] + good[3:5] + [bad_cost] + good[5:])
    assert "negative supply" in str(e2.value)
    # the runner still works after a rejected batch
    out = fg.batch_solve(good)
    assert all(r.status == 0 and r.certified for r in out)


def test_batch_validation_after_launch():
    """Costs are range-checked while each size bucket is packed, largest
    bucket first: a bad cost in a small instance is found after the large
    buckets were launched, and the call still fails with the first failing
    instance's error and no results; a shape error later in the list does
    not hide an earlier cost error in another bucket."""
    big = [fg.generate(0, 960 + k, 300, 280, 1, 100, 10, 50) for k in range(3)]
    small_bad = fg.generate(0, 970, 12, 9, 1, 100, 10, 50)
    small_bad.cost = small_bad.cost.copy()
    small_bad.cost[5, 2] = -(1 << 30) - 1
    with pytest.raises(RuntimeError) as e1:
        fg.batch_solve(big + [small_bad])
    assert "cost out of range" in str(e1.value)
    bad_shape = fg.generate(0, 971, 40, 30, 1, 100, 10, 50)
    bad_shape.demand = bad_shape.demand.copy()
    bad_shape.demand[1] = -5
    with pytest.raises(RuntimeError) as e2:
        fg.batch_solve([big[0], small_bad, big[1], bad_shape])
    assert "cost out of range" in str(e2.value)
    out = fg.batch_solve(big + [fg.generate(0, 972, 12, 9, 1, 100, 10, 50)])
    assert all(r.status == 0 and r.certified for r in out)


@pytest.mark.parametrize("form", ["persistent", "round"])
def test_batch_partial_pricing_all_buckets(form, monkeypatch):
    """Partial pricing (candidate rows) in both batched forms on every size
    bucket plus one instance above it: certified optima equal to full
    pricing's.  The round form restages row keys in every launch, so it also
    covers rounds whose non-candidate keys start out as garbage."""
    monkeypatch.setenv("FLOCK_BATCH_FORM", form)
    shapes = [(5, 7), (30, 30), (60, 60), (100, 150), (200, 300), (400, 500), (900, 1000),
              (1500, 1444), (1000, 2072), (1600, 1600), (2100, 2000), (12, 40), (3, 3)]
    insts = [fg.generate(0, 600 + k, m, n, 1, 1000, 100, 1000) for k, (m, n) in enumerate(shapes)]
    insts += fg.mixed_batch(23, 96, 10, 300)
    insts.append(fg.config_instance("degenerate1000", 1, m=400, n=300))
    full = fg.batch_solve(insts, pricing="full")
    part = fg.batch_solve(insts, pricing="partial")
    for k, (f, p) in enumerate(zip(full, part)):
        assert f.status == 0 and f.certified, k
        assert p.status == 0 and p.certified, (k, insts[k].m, insts[k].n, p.status, p.notes)
        assert p.objective == f.objective, (k, insts[k].m, insts[k].n)


@pytest.mark.parametrize("bfs,pivot,pricing", [("nwc", "switch", "partial"), ("vogel", "sequential", "full"),
                                               ("vogel", "parallel", "partial"), ("nwc", "parallel", "full")])
def test_batch_option_combinations(bfs, pivot, pricing):
    """Every start / pivot / pricing combination of the batched form gives the
    plain solver's certified optimum on a mixed batch."""
    insts = fg.mixed_batch(41, 80, 10, 400)
    out = fg.batch_solve(insts, bfs=bfs, pivot=pivot, pricing=pricing)
    for k, (inst, r) in enumerate(zip(insts, out)):
        assert r.status == 0 and r.certified, (k, inst.m, inst.n, r.status)
        assert r.objective == fg.solve(inst).objective, (k, inst.m, inst.n)


def test_batch_iteration_cap_reported():
    """A round cap below what an instance needs stops it with ST_ITER_CAP and
    FLOCK_ERR_NOT_OPTIMAL, without disturbing the instances that finish."""
    big = fg.generate(0, 42, 200, 220, 1, 1000, 100, 1000)
    small = fg.generate(0, 43, 3, 3, 1, 1000, 100, 1000)
    need = fg.solve(small).iterations
    out = fg.batch_solve([big, small], max_iterations=need + 2, pricing="full")
    assert out[0].status & fg.ST_ITER_CAP and not out[0].certified
    assert out[1].status == 0 and out[1].certified and out[1].objective == fg.solve(small).objective


@pytest.mark.parametrize("kind", ["uniform", "degenerate"])
def test_plain_grid_round_matches_batched(kind):
    """m + n = 4096: the plain solver runs its grid-wide pivot rounds, the
    batched form its persistent kernel; both certified, same optimum."""
    if kind == "uniform":
        inst = fg.generate(0, 77, 2048, 2048, 1, 1000, 100, 1000)
    else:
        inst = fg.config_instance("degenerate1000", 7, m=2048, n=2048)
    b = fg.batch_solve([inst], pricing="full")[0]
    assert b.status == 0 and b.certified
    for pivot in ("switch", "sequential"):
        for pricing in ("full", "partial"):
            p = fg.solve(inst, pivot=pivot, pricing=pricing)
            assert p.status == 0 and p.certified, (pivot, pricing, p.status, p.notes)
            assert p.objective == b.objective, (pivot, pricing)


def test_lp_optimum_cross_check():
    """GPU optima (plain and batched) equal an independent LP solver's
    (HiGHS) on medium instances, including a degenerate one."""
    pytest.importorskip("scipy")
    from lp_check import lp_optimum
    insts = [fg.generate(0, 4000 + k, 60 + 40 * k, 90 + 25 * k, 1, 1000, 100, 1000) for k in range(4)]
    insts.append(fg.config_instance("degenerate1000", 9, m=150, n=120))
    batch = fg.batch_solve(insts)
    for k, inst in enumerate(insts):
        opt = lp_optimum(inst.supply, inst.demand, inst.cost)
        p = fg.solve(inst)
        assert p.status == 0 and p.certified and p.objective == opt, k
        assert batch[k].status == 0 and batch[k].certified and batch[k].objective == opt, k


# Certified optimum of the 8000 x 8000 Euclidean workload, seed 0 (the
# reference CPU path cannot finish an instance of this size -- its Vogel
# refreshes up to m*n cells per allocation and its loop stops at 30000
# iterations -- so the pin is the exact certificate, checked on the host).
EUCLID8000_OPTIMUM = 614_260_730


def test_euclid8000_full_size_certified():
    """The 8000 x 8000 Euclidean workload at full size on the plain solver
    (grid-wide rounds, partial pricing): the host oracle's exact certificate
    over all 64 M cells (row and column sums, every reduced cost >= 0 in
    int64, complementary slackness) and the objective, computed on the host
    from the returned flows."""
    inst = fg.config_instance("euclid8000", 0)
    res = fg.solve(inst)
    assert res.status == 0 and res.certified, (res.status, res.notes)
    bits, obj = oracle.certify(inst.supply, inst.demand, inst.cost, res.flows, res.u, res.v)
    assert bits == 0, f"certificate bits {bits}"
    assert obj == res.objective == EUCLID8000_OPTIMUM


@pytest.mark.parametrize("kind", ["uniform", "degenerate"])
def test_grid_cluster_rounds_match_six_kernel_rounds(kind, monkeypatch):
    """Partial pricing on the grid path (m + n >= 4096): the candidate rounds
    inside one thread-block cluster take the same pivots as the six-kernel
    rounds (same rounds, pivots and objective), both certified by the host
    oracle."""
    if kind == "uniform":
        inst = fg.generate(0, 91, 2048, 2600, 1, 1000, 100, 1000)
    else:
        inst = fg.config_instance("degenerate1000", 13, m=2500, n=2048)
    monkeypatch.setenv("FLOCK_GRID_FORM", "rounds")
    a = fg.solve(inst)
    monkeypatch.delenv("FLOCK_GRID_FORM")
    b = fg.solve(inst)
    for r in (a, b):
        assert r.status == 0 and r.certified
        bits, obj = oracle.certify(inst.supply, inst.demand, inst.cost, r.flows, r.u, r.v)
        assert bits == 0 and obj == r.objective
    assert (a.objective, a.iterations, a.pivots) == (b.objective, b.iterations, b.pivots)


def test_ss_tiny_degenerate():
    """-a parallel_ss (every negative cell a candidate, greedy edge-disjoint
    cycles) on tiny tied instances: certified, the reference path's optimum."""
    for inst in tiny_instances(41, 200):
        r = fg.solve(inst, pivot="ss")
        assert_optimal(inst, r)


@pytest.mark.parametrize("name,seed,m,n", [("uniform100", 0, None, None), ("uniform100", 3, None, None),
                                           ("degenerate1000", 2, 300, 250), ("euclid8000", 4, 150, 260)])
def test_ss_shapes(name, seed, m, n):
    inst = fg.config_instance(name, seed, m=m, n=n)
    r = fg.solve(inst, pivot="ss")
    assert_optimal(inst, r)
    assert r.pivots >= r.iterations - 1       # several pivots in some rounds, at least one in each but the last


def test_ss_degenerate_1000_full_size():
    """The 1000 x 1000 degenerate workload: the same optimum as the reference
    CPU path (which certifies optimal) and as the u-v mode's sequential
    pivots, certified by the host oracle; every round but the last pivots."""
    inst = fg.config_instance("degenerate1000", 0)
    ss = fg.solve(inst, pivot="ss")
    uv = fg.solve(inst, pivot="sequential", pricing="full")
    assert ss.status == 0 and ss.certified and uv.status == 0 and uv.certified
    bits, obj = oracle.certify(inst.supply, inst.demand, inst.cost, ss.flows, ss.u, ss.v)
    assert bits == 0 and obj == ss.objective == uv.objective == 25797
    assert ss.pivots >= ss.iterations - 1


def test_ss_plain_sizes_and_batched_rejected():
    """ss pivots on plain instances across the size range (round kernel at
    every size, up to 4096 vertices): the same optima as the default pivots.
    The batched and served forms refuse the mode (flock_solve only)."""
    sizes = [(20, 30), (100, 120), (400, 500), (1400, 1500), (2048, 2048)]
    for k, (m, n) in enumerate(sizes):
        inst = fg.generate(0, 600 + k, m, n, 1, 1000, 100, 1000)
        r = fg.solve(inst, pivot="ss")
        d = fg.solve(inst)
        assert r.status == 0 and r.certified and r.objective == d.objective, (m, n)
    small = fg.generate(0, 650, 30, 40, 1, 1000, 100, 1000)
    with pytest.raises(fg.FlockError) as ex:
        fg.batch_solve([small], pivot="ss")
    assert ex.value.status == fg.FLOCK_ERR_ARG
