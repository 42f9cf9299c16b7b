"""flock_gb300 -- Python host mirror of the flock solver API over the native
library (libflock_gb300.so, CUDA for sm_103a).

The native library is required: every entry point raises if it is missing
or was not built, there is no CPU fallback.  Names follow the reference
(researchgroup-zx93920/flock): ProblemInstance, make_problem,
uvModel_parallel / ssModel_parallel / switchModel_parallel with execute(),
create_flows(), objVal, totalIterations, totalSolveTime.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass, field
from typing import List, Optional, Sequence, Tuple

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libflock_gb300.so")

# --------------------------------------------------------------- ctypes ---
i32 = ctypes.c_int32
i64 = ctypes.c_int64
P = ctypes.POINTER


class CInstance(ctypes.Structure):
    _fields_ = [("m", i32), ("n", i32), ("supply", P(i32)), ("demand", P(i32)), ("cost", P(i32))]


class CFlow(ctypes.Structure):
    _fields_ = [("source", i32), ("destination", i32), ("qty", i32)]


class COptions(ctypes.Structure):
    _fields_ = [("bfs_method", i32), ("pivot_method", i32), ("max_iterations", i32), ("verify", i32),
                ("pricing", i32)]


class CStats(ctypes.Structure):
    _fields_ = [("objective", i64), ("iterations", i32), ("pivots", i32), ("active_flows", i32),
                ("status", i32), ("notes", i32), ("certified", i32), ("vogel_events", i32),
                ("ms_total", ctypes.c_double), ("ms_bfs", ctypes.c_double), ("ms_simplex", ctypes.c_double),
                ("ms_dual", ctypes.c_double), ("ms_sweep", ctypes.c_double), ("ms_pivot", ctypes.c_double),
                ("ms_cycle", ctypes.c_double), ("ms_resolve", ctypes.c_double), ("ms_adjust", ctypes.c_double)]


class CServerConfig(ctypes.Structure):
    _fields_ = [("memory_budget_bytes", i64), ("max_inflight_batches", i32), ("max_batch", i32),
                ("options", COptions)]


class CResult(ctypes.Structure):
    _fields_ = [("ticket", ctypes.c_uint64), ("status", i32), ("stats", CStats), ("latency_ms", ctypes.c_double)]


FLOCK_OK, FLOCK_ERR_ARG, FLOCK_ERR_UNBALANCED, FLOCK_ERR_FILE, FLOCK_ERR_PARSE, FLOCK_ERR_INEXACT, \
    FLOCK_ERR_RANGE, FLOCK_ERR_CUDA, FLOCK_ERR_NOT_OPTIMAL, FLOCK_ERR_BUDGET, FLOCK_ERR_CAPACITY = range(11)

ST_ITER_CAP, ST_TREE_CORRUPT, ST_SF_FAIL, ST_CERT_FAIL, ST_RANGE = 1, 2, 4, 32, 64
NOTE_VOGEL_UNDEF, NOTE_START_REPAIRED = 8, 16

BFS = {"nwc": 0, "nwc_host": 0, "vogel": 1, "vam_host": 1, "vogel_device": 2, "vam_device": 2}
PIVOT = {"sequential": 0, "parallel_uv": 0, "parallel": 1, "switch": 2, "switch_hybrid": 2, "ss": 3, "parallel_ss": 3}


class FlockError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"flock status {status}: {msg}")
        self.status = status


class FileNotFoundException(FlockError):
    """The reference's FileNotFoundException (src/instance.h:5-11)."""


_lib = None


def lib() -> ctypes.CDLL:
    """Load the native library.  Raises when it is missing: no fallback."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"native library missing: {LIB_PATH}; run python -m flock_gb300.build")
    L = ctypes.CDLL(LIB_PATH)
    L.flock_last_error.restype = ctypes.c_char_p
    L.flock_version.restype = ctypes.c_char_p
    L.flock_solve.argtypes = [P(CInstance), P(COptions), P(CFlow), P(i64), P(i64), P(CStats)]
    L.flock_vogel.argtypes = [P(CInstance), P(CFlow), P(i32)]
    L.flock_batch_solve.argtypes = [i32, P(CInstance), P(COptions), P(CFlow), P(i64), P(CStats)]
    L.flock_generate.argtypes = [i32, ctypes.c_uint64, i32, i32, i32, i32, i32, i32, P(i32), P(i32), P(i32)]
    L.flock_generate_sizes.argtypes = [ctypes.c_uint64, i32, i32, i32, P(i32), P(i32)]
    L.flock_dat_shape.argtypes = [ctypes.c_char_p, P(i32), P(i32)]
    L.flock_dat_scale.argtypes = [ctypes.c_char_p, P(i32)]
    L.flock_read_dat.argtypes = [ctypes.c_char_p, i32, i32, i32, P(i32), P(i32), P(i32)]
    L.flock_write_bin.argtypes = [ctypes.c_char_p, P(CInstance)]
    L.flock_write_dat.argtypes = [ctypes.c_char_p, P(CInstance), i32]
    L.flock_bin_shape.argtypes = [ctypes.c_char_p, P(i32), P(i32)]
    L.flock_read_bin.argtypes = [ctypes.c_char_p, i32, i32, P(i32), P(i32), P(i32)]
    L.flock_server_create.argtypes = [P(CServerConfig), P(ctypes.c_void_p)]
    L.flock_server_submit.argtypes = [ctypes.c_void_p, P(CInstance), P(ctypes.c_uint64)]
    L.flock_server_poll.argtypes = [ctypes.c_void_p, P(CResult), P(P(CFlow)), i32, P(i32)]
    L.flock_server_drain.argtypes = [ctypes.c_void_p]
    L.flock_server_destroy.argtypes = [ctypes.c_void_p]
    L.flock_default_server_config.argtypes = [P(CServerConfig)]
    L.flock_server_request_bytes.argtypes = [i32, i32]
    L.flock_server_request_bytes.restype = i64
    L.flock_default_options.argtypes = [P(COptions)]
    L.flock_bench_batch_rerun.argtypes = [P(ctypes.c_float), P(i32)]
    _lib = L
    return L


def _err(rc: int) -> FlockError:
    msg = lib().flock_last_error().decode(errors="replace")
    if rc == FLOCK_ERR_FILE:
        return FileNotFoundException(rc, msg)
    return FlockError(rc, msg)


def _p(a: np.ndarray, t=i32):
    return a.ctypes.data_as(P(t))


def _arr(x) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(x, dtype=np.int32))


def version() -> str:
    return lib().flock_version().decode()


# ----------------------------------------------------------- instances ---
@dataclass
class Instance:
    supply: np.ndarray
    demand: np.ndarray
    cost: np.ndarray          # (m, n) int32

    @property
    def m(self) -> int:
        return int(self.supply.shape[0])

    @property
    def n(self) -> int:
        return int(self.demand.shape[0])

    def c(self) -> CInstance:
        # The C view points into the arrays; it is rebuilt whenever an array
        # attribute was replaced (in-place edits need no rebuild).
        key = (id(self.supply), id(self.demand), id(self.cost))
        cached = self.__dict__.get("_c")
        if cached is not None and cached[0] == key:
            return cached[1]
        self.supply = _arr(self.supply)
        self.demand = _arr(self.demand)
        self.cost = _arr(self.cost).reshape(self.m, self.n)
        ci = CInstance(self.m, self.n, _p(self.supply), _p(self.demand), _p(self.cost))
        self.__dict__["_c"] = ((id(self.supply), id(self.demand), id(self.cost)), ci)
        return ci


def generate(kind: int, seed: int, m: int, n: int, c_lo: int, c_hi: int, q_lo: int, q_hi: int) -> Instance:
    s = np.empty(m, np.int32)
    d = np.empty(n, np.int32)
    c = np.empty((m, n), np.int32)
    rc = lib().flock_generate(kind, seed, m, n, c_lo, c_hi, q_lo, q_hi, _p(s), _p(d), _p(c))
    if rc:
        raise _err(rc)
    return Instance(s, d, c)


def generate_sizes(seed: int, count: int, lo: int, hi: int) -> Tuple[np.ndarray, np.ndarray]:
    ms = np.empty(count, np.int32)
    ns = np.empty(count, np.int32)
    rc = lib().flock_generate_sizes(seed, count, lo, hi, _p(ms), _p(ns))
    if rc:
        raise _err(rc)
    return ms, ns


# The five workloads of the benchmark description, as generator calls.
def config_instance(name: str, seed: int = 0, m: Optional[int] = None, n: Optional[int] = None) -> Instance:
    if name == "uniform100":      # 100x100, costs 1..100, quantities 100..1000
        return generate(0, seed, m or 100, n or 100, 1, 100, 100, 1000)
    if name == "degenerate1000":  # 1000x1000, costs 1..20, quantities 1..50
        return generate(0, seed, m or 1000, n or 1000, 1, 20, 1, 50)
    if name == "euclid8000":      # 8000x8000 Euclidean costs, quantities 1..10000
        return generate(1, seed, m or 8000, n or 8000, 0, 0, 1, 10000)
    raise ValueError(name)


def mixed_batch(seed: int, count: int, lo: int, hi: int) -> List[Instance]:
    """count instances, m and n log-uniform in [lo, hi], costs 1..1000,
    quantities 100..1000 (the batched / served workloads)."""
    ms, ns = generate_sizes(seed, count, lo, hi)
    return [generate(0, seed * 1000003 + k + 1, int(ms[k]), int(ns[k]), 1, 1000, 100, 1000) for k in range(count)]


def read_dat(path: str, scale: Optional[int] = None) -> Tuple[Instance, int]:
    """The reference's .dat format; costs scaled by 10**scale to exact int32
    (scale None: the smallest exact one)."""
    L = lib()
    m, n, sc = i32(), i32(), i32()
    bp = path.encode()
    rc = L.flock_dat_shape(bp, ctypes.byref(m), ctypes.byref(n))
    if rc:
        raise _err(rc)
    if scale is None:
        rc = L.flock_dat_scale(bp, ctypes.byref(sc))
        if rc:
            raise _err(rc)
        scale = sc.value
    s = np.empty(m.value, np.int32)
    d = np.empty(n.value, np.int32)
    c = np.empty((m.value, n.value), np.int32)
    rc = L.flock_read_dat(bp, scale, m.value, n.value, _p(s), _p(d), _p(c))
    if rc:
        raise _err(rc)
    return Instance(s, d, c), scale


def write_dat(inst: Instance, path: str, scale: int = 0) -> None:
    """The reference's .dat layout; costs written as cost / 10**scale."""
    rc = lib().flock_write_dat(path.encode(), ctypes.byref(inst.c()), int(scale))
    if rc:
        raise _err(rc)


def write_bin(inst: Instance, path: str) -> None:
    """Binary instance file (int32 little-endian; see include/flock.h)."""
    rc = lib().flock_write_bin(path.encode(), ctypes.byref(inst.c()))
    if rc:
        raise _err(rc)


def read_bin(path: str) -> Instance:
    L = lib()
    m, n = i32(), i32()
    bp = path.encode()
    rc = L.flock_bin_shape(bp, ctypes.byref(m), ctypes.byref(n))
    if rc:
        raise _err(rc)
    s = np.empty(m.value, np.int32)
    d = np.empty(n.value, np.int32)
    c = np.empty((m.value, n.value), np.int32)
    rc = L.flock_read_bin(bp, m.value, n.value, _p(s), _p(d), _p(c))
    if rc:
        raise _err(rc)
    return Instance(s, d, c)


# ------------------------------------------------------------- solving ---
@dataclass
class Result:
    objective: int
    flows: np.ndarray            # (m+n-1, 3) int32: source, destination, qty (nonzero first)
    active_flows: int
    iterations: int
    pivots: int
    status: int
    notes: int
    certified: bool
    vogel_events: int
    ms_total: float
    ms_bfs: float
    ms_simplex: float
    u: Optional[np.ndarray] = None
    v: Optional[np.ndarray] = None
    # device time per simplex phase (plain solver; 0 in the batched and served forms)
    ms_dual: float = 0.0
    ms_sweep: float = 0.0
    ms_pivot: float = 0.0
    ms_cycle: float = 0.0
    ms_resolve: float = 0.0
    ms_adjust: float = 0.0

    @property
    def optimal(self) -> bool:
        return self.status == 0


PRICING = {"full": 0, "partial": 1}


def _options(bfs="vogel", pivot="switch", max_iterations=0, verify=True, pricing="partial") -> COptions:
    return COptions(BFS[bfs], PIVOT[pivot], int(max_iterations), 1 if verify else 0, PRICING[pricing])


def _result(st: CStats, flows: np.ndarray, u=None, v=None) -> Result:
    return Result(int(st.objective), flows, int(st.active_flows), int(st.iterations), int(st.pivots),
                  int(st.status), int(st.notes), bool(st.certified), int(st.vogel_events), float(st.ms_total),
                  float(st.ms_bfs), float(st.ms_simplex), u, v, float(st.ms_dual), float(st.ms_sweep),
                  float(st.ms_pivot), float(st.ms_cycle), float(st.ms_resolve), float(st.ms_adjust))


def solve(inst: Instance, bfs: str = "vogel", pivot: str = "switch", max_iterations: int = 0,
          verify: bool = True, duals: bool = True, raise_on_error: bool = True, pricing: str = "partial") -> Result:
    ci = inst.c()
    opt = _options(bfs, pivot, max_iterations, verify, pricing)
    V = inst.m + inst.n
    flows = np.zeros((V - 1, 3), np.int32)
    u = np.zeros(inst.m, np.int64) if duals else None
    v = np.zeros(inst.n, np.int64) if duals else None
    st = CStats()
    rc = lib().flock_solve(ctypes.byref(ci), ctypes.byref(opt), flows.ctypes.data_as(P(CFlow)),
                           _p(u, i64) if duals else None, _p(v, i64) if duals else None, ctypes.byref(st))
    if rc and rc != FLOCK_ERR_NOT_OPTIMAL and raise_on_error:
        raise _err(rc)
    return _result(st, flows, u, v)


def vogel(inst: Instance) -> Tuple[np.ndarray, int]:
    """Vogel's approximation on the GPU: (m+n-1, 3) allocations in order, events."""
    ci = inst.c()
    V = inst.m + inst.n
    flows = np.zeros((V - 1, 3), np.int32)
    ev = i32()
    rc = lib().flock_vogel(ctypes.byref(ci), flows.ctypes.data_as(P(CFlow)), ctypes.byref(ev))
    if rc:
        raise _err(rc)
    return flows, int(ev.value)


def vogel_device(inst: Instance) -> Tuple[np.ndarray, int]:
    """Vogel with the reference's device semantics ("vam_device") on the GPU:
    (m+n-1, 3) allocations in order, events (-1: undefined in the reference
    from the first (-1, -1, 0) allocation on)."""
    ci = inst.c()
    V = inst.m + inst.n
    flows = np.zeros((V - 1, 3), np.int32)
    ev = i32()
    rc = lib().flock_vogel_device(ctypes.byref(ci), flows.ctypes.data_as(P(CFlow)), ctypes.byref(ev))
    if rc:
        raise _err(rc)
    return flows, int(ev.value)


def batch_solve(insts: Sequence[Instance], bfs: str = "vogel", pivot: str = "switch",
                max_iterations: int = 0, verify: bool = True, pricing: str = "partial") -> List[Result]:
    k = len(insts)
    arr = (CInstance * k)(*[x.c() for x in insts])
    total = sum(x.m + x.n - 1 for x in insts)
    flows = np.zeros((max(total, 1), 3), np.int32)
    stats = (CStats * k)()
    opt = _options(bfs, pivot, max_iterations, verify, pricing)
    rc = lib().flock_batch_solve(k, arr, ctypes.byref(opt), flows.ctypes.data_as(P(CFlow)), None, stats)
    if rc and rc != FLOCK_ERR_NOT_OPTIMAL:
        raise _err(rc)
    out, off = [], 0
    for x, st in zip(insts, stats):
        V1 = x.m + x.n - 1
        out.append(_result(st, flows[off:off + V1].copy()))
        off += V1
    return out


def bench_batch_rerun() -> Tuple[float, int]:
    """Benchmark hook: device time (ms) of re-solving the last batch with its
    inputs already resident on the GPU, and the kernels it launched."""
    ms = ctypes.c_float()
    n = i32()
    rc = lib().flock_bench_batch_rerun(ctypes.byref(ms), ctypes.byref(n))
    if rc:
        raise _err(rc)
    return float(ms.value), int(n.value)


class Server:
    """Served form: continuous batching with a device-memory budget."""

    @staticmethod
    def request_bytes(m: int, n: int) -> int:
        """Device bytes one m x n request holds while served (its budget charge)."""
        return int(lib().flock_server_request_bytes(m, n))

    def __init__(self, memory_budget_bytes: int = 40 << 30, max_inflight_batches: int = 16, max_batch: int = 512,
                 bfs: str = "vogel", pivot: str = "switch", verify: bool = True, pricing: str = "partial"):
        L = lib()
        cfg = CServerConfig()
        L.flock_default_server_config(ctypes.byref(cfg))
        cfg.memory_budget_bytes = memory_budget_bytes
        cfg.max_inflight_batches = max_inflight_batches
        cfg.max_batch = max_batch
        cfg.options = _options(bfs, pivot, 0, verify, pricing)
        self._h = ctypes.c_void_p()
        rc = L.flock_server_create(ctypes.byref(cfg), ctypes.byref(self._h))
        if rc:
            raise _err(rc)
        self._sizes = {}

    def submit(self, inst: Instance) -> int:
        ci = inst.c()
        t = ctypes.c_uint64()
        rc = lib().flock_server_submit(self._h, ctypes.byref(ci), ctypes.byref(t))
        if rc:
            raise _err(rc)
        self._sizes[t.value] = inst.m + inst.n - 1
        return int(t.value)

    def poll(self, max_results: int = 1024, with_flows: bool = False):
        res = (CResult * max_results)()
        cnt = i32()
        rc = lib().flock_server_poll(self._h, res, None, max_results, ctypes.byref(cnt))
        if rc:
            raise _err(rc)
        return [(int(r.ticket), int(r.status), r.stats.objective, float(r.latency_ms), int(r.stats.status),
                 bool(r.stats.certified)) for r in res[:cnt.value]]

    def drain(self) -> None:
        lib().flock_server_drain(self._h)

    def close(self) -> None:
        if self._h:
            lib().flock_server_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------ reference-named facade ---------
class ProblemInstance:
    """Container for the problem (src/structs.h:19-40).  Costs are exact
    integers (cost_scale decimal digits); `costs` keeps the float view."""

    def __init__(self):
        self.filename = ""
        self.algo = "parallel_uv"
        self.numSupplies = 0
        self.numDemands = 0
        self.supplies = np.zeros(0, np.int32)
        self.demands = np.zeros(0, np.int32)
        self.int_costs = np.zeros((0, 0), np.int32)
        self.cost_scale = 0
        self.active_flows = 0
        self.totalFlowCost = 0.0
        self.solveTime = 0.0

    @property
    def costs(self) -> np.ndarray:
        return self.int_costs.astype(np.float64) / (10 ** self.cost_scale)


def make_problem(filename: str, algo: str = "parallel_uv") -> ProblemInstance:
    """src/instance.cpp:149-179: read the .dat file into a ProblemInstance."""
    inst, scale = read_dat(filename)
    p = ProblemInstance()
    p.filename = filename
    p.algo = algo
    p.numSupplies, p.numDemands = inst.m, inst.n
    p.supplies, p.demands, p.int_costs = inst.supply, inst.demand, inst.cost
    p.cost_scale = scale
    p.active_flows = inst.m + inst.n - 1
    return p


@dataclass
class flowInformation:
    source: int
    destination: int
    qty: float


# The reference's compile-time BFS switch (BFS_METHOD, parallel_structs.h:45):
# "vam_host" (the default), "vam_device" or "nwc_host"; the model classes
# below read it at execute().
BFS_METHOD = "vam_host"


class _Model:
    _pivot = "parallel"

    def __init__(self, problem: ProblemInstance, flows: Optional[list] = None):
        self.data = problem
        self.optimal_flows = flows if flows is not None else []
        self.uv_time = self.reduced_cost_time = self.pivot_time = 0.0
        self.cycle_discovery_time = self.resolve_time = self.adjustment_time = 0.0
        self.objVal = 0.0
        self.totalIterations = 0
        self.totalSolveTime = 0.0
        self.result: Optional[Result] = None

    def execute(self) -> None:
        p = self.data
        r = solve(Instance(p.supplies, p.demands, p.int_costs), bfs=BFS_METHOD, pivot=self._pivot)
        self.result = r
        self.objVal = r.objective / (10 ** p.cost_scale)
        self.totalIterations = r.iterations
        self.totalSolveTime = r.ms_bfs + r.ms_simplex
        # phase times in microseconds, as the reference's model statistics
        self.uv_time = r.ms_dual * 1000.0
        self.reduced_cost_time = r.ms_sweep * 1000.0
        self.pivot_time = r.ms_pivot * 1000.0
        self.cycle_discovery_time = r.ms_cycle * 1000.0
        self.resolve_time = r.ms_resolve * 1000.0
        self.adjustment_time = r.ms_adjust * 1000.0
        p.active_flows = r.active_flows
        p.totalFlowCost = self.objVal
        p.solveTime = self.totalSolveTime

    def create_flows(self) -> list:
        f = self.result.flows[:self.result.active_flows]
        self.optimal_flows[:] = [flowInformation(int(a), int(b), float(q)) for a, b, q in f]
        return self.optimal_flows


class uvModel_parallel(_Model):
    """-a parallel_uv: one pivot per reduced-cost sweep."""
    _pivot = "sequential"


class ssModel_parallel(_Model):
    """-a parallel_ss: every negative cell a candidate, the greedy
    most-negative set of tree-edge-disjoint cycles pivoted together."""
    _pivot = "parallel_ss"


class switchModel_parallel(_Model):
    """-a switch_hybrid: parallel rounds until one applies fewer than 10
    pivots, then sequential ones (switch/switch_model_parallel.cu:182-184)."""
    _pivot = "switch"
