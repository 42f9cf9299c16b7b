"""CPU: host logic of the product with no GPU -- the C ABI library loads and
exports every symbol include/flock.h declares, the generator is
deterministic, the .dat reader and the argument checks return the
documented status codes, the C++ facade compiles, the CLI reports usage
errors, and the server refuses requests over its memory budget."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

import flock_gb300 as fg
from conftest import ROOT
from golden_util import checksum

HEADER = os.path.join(ROOT, "include", "flock.h")


def declared_symbols():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(flock_[a-z_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol(flock_lib):
    syms = declared_symbols()
    assert len(syms) >= 15
    for s in syms:
        assert hasattr(flock_lib, s), s


def test_version(flock_lib):
    assert "sm_103a" in fg.version()


def test_generator_deterministic():
    a = fg.config_instance("uniform100", 0)
    b = fg.config_instance("uniform100", 0)
    assert checksum(a.supply, a.demand, a.cost) == checksum(b.supply, b.demand, b.cost)
    assert checksum(a.supply, a.demand, a.cost) == "c2b1152114b4affd"
    assert a.supply.sum() == a.demand.sum()
    assert a.cost.min() >= 1 and a.cost.max() <= 100
    e = fg.config_instance("euclid8000", 0, m=150, n=200)
    assert checksum(e.supply, e.demand, e.cost) == "65e5f43ff1f0024c"
    assert e.supply.sum() == e.demand.sum() and e.cost.min() >= 0 and e.cost.max() <= 1415


def test_generator_sizes():
    ms, ns = fg.generate_sizes(1, 2000, 10, 500)
    assert ms.min() >= 10 and ms.max() <= 500 and ns.min() >= 10 and ns.max() <= 500
    # log-uniform: median near sqrt(10*500) ~ 71
    assert 50 < np.median(ms) < 100


def test_degenerate_config_balanced():
    x = fg.config_instance("degenerate1000", 2, m=300, n=300)
    assert x.supply.sum() == x.demand.sum()
    assert x.cost.max() <= 20 and x.supply.max() <= 50


def write(tmp_path, name, text):
    p = tmp_path / name
    p.write_text(text)
    return str(p)


def test_reader_formats(tmp_path):
    p = write(tmp_path, "a.dat", "2 3\n5\t7\n4 4 4\n1.25 2 3\n4 5.5 6.75\n")
    inst, scale = fg.read_dat(p)
    assert scale == 2
    assert inst.supply.tolist() == [5, 7] and inst.demand.tolist() == [4, 4, 4]
    assert inst.cost.tolist() == [[125, 200, 300], [400, 550, 675]]
    inst0, s0 = fg.read_dat(write(tmp_path, "b.dat", "1 1 3 3 17"))
    assert s0 == 0 and inst0.cost.tolist() == [[17]]


def test_reader_errors(tmp_path):
    with pytest.raises(fg.FileNotFoundException):
        fg.read_dat(str(tmp_path / "missing.dat"))
    with pytest.raises(fg.FlockError) as ex:
        fg.read_dat(write(tmp_path, "bad.dat", "2 2\n1 1\n1 x\n1 2 3 4\n"))
    assert ex.value.status == fg.FLOCK_ERR_PARSE
    with pytest.raises(fg.FlockError) as ex:
        fg.read_dat(write(tmp_path, "short.dat", "2 2\n1 1\n1 1\n1 2 3\n"))
    assert ex.value.status == fg.FLOCK_ERR_PARSE
    with pytest.raises(fg.FlockError) as ex:
        fg.read_dat(write(tmp_path, "inexact.dat", "1 2\n2\n1 1\n1.5 2.25\n"), scale=1)
    assert ex.value.status == fg.FLOCK_ERR_INEXACT


def test_reader_reference_fixture_copy(tmp_path):
    """A fixture of the reference's tests/ folder, written back as text."""
    import json
    fx = json.load(open(os.path.join(ROOT, "tests", "golden", "reference_fixtures.json")))
    e = [x for x in fx if x["file"] == "test_TransportModel_25_25_1.dat"][0]
    txt = f"{e['m']} {e['n']}\n" + " ".join(map(str, e["supply"])) + "\n" + " ".join(map(str, e["demand"])) + "\n"
    txt += " ".join("%d.%02d" % (c // 100, c % 100) for c in e["cost"]) + "\n"
    inst, scale = fg.read_dat(write(tmp_path, "fx.dat", txt))
    assert scale <= 2
    assert (inst.cost.reshape(-1) * 10 ** (2 - scale)).tolist() == e["cost"]


def test_solve_argument_errors():
    bad = fg.Instance(np.array([3, 4], np.int32), np.array([5, 1], np.int32), np.ones((2, 2), np.int32))
    with pytest.raises(fg.FlockError) as ex:
        fg.solve(bad)
    assert ex.value.status == fg.FLOCK_ERR_UNBALANCED
    neg = fg.Instance(np.array([-1, 2], np.int32), np.array([1, 0], np.int32), np.ones((2, 2), np.int32))
    with pytest.raises(fg.FlockError) as ex:
        fg.solve(neg)
    assert ex.value.status == fg.FLOCK_ERR_ARG
    big = fg.Instance(np.array([1], np.int32), np.array([1], np.int32), np.array([[1 << 31 - 1]], np.int32))
    big.cost[0, 0] = (1 << 30) + 5
    with pytest.raises(fg.FlockError) as ex:
        fg.solve(big)
    assert ex.value.status == fg.FLOCK_ERR_RANGE


def test_cpp_facade_compiles(tmp_path):
    src = tmp_path / "use.cpp"
    src.write_text('#include "flock/algos.h"\nint main(){ProblemInstance p; std::vector<flowInformation> f(1);'
                   ' uvModel_parallel a(&p, f.data()); ssModel_parallel b(&p, f.data());'
                   ' switchModel_parallel c(&p, f.data()); (void)a; (void)b; (void)c; return 0;}\n')
    for define in [[], ["-DFLOCK_DEFAULT_BFS=FLOCK_BFS_VOGEL_DEVICE"], ["-DFLOCK_DEFAULT_BFS=FLOCK_BFS_NWC"]]:
        r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-I", os.path.join(ROOT, "include")] + define
                           + [str(src)], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr


def test_reference_main_compiles_unchanged(tmp_path):
    """The reference's own driver (src/main.cpp) compiles and links unchanged
    against the facade headers (include/flock: algos.h, instance.h, structs.h,
    logger.h, parameters.h) and the library.  Needs the reference checkout;
    the file is copied so that its own directory's headers are not found."""
    import shutil
    from conftest import REFERENCE
    src = os.path.join(REFERENCE, "src", "main.cpp")
    lib_dir = os.path.join(ROOT, "flock_gb300")
    if not os.path.exists(src):
        pytest.skip("reference checkout not present")
    if not os.path.exists(os.path.join(lib_dir, "libflock_gb300.so")):
        pytest.skip("library not built")
    shutil.copy(src, tmp_path / "main.cpp")
    r = subprocess.run(["g++", "-std=c++17", "-I", os.path.join(ROOT, "include", "flock"), str(tmp_path / "main.cpp"),
                        "-L", lib_dir, "-lflock_gb300", f"-Wl,-rpath,{lib_dir}", "-o", str(tmp_path / "ref_main")],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr


def test_facade_driver_compiles(tmp_path):
    """The committed facade driver (run on the GPU by tests/test_gpu_facade.py)
    compiles and links here."""
    lib_dir = os.path.join(ROOT, "flock_gb300")
    if not os.path.exists(os.path.join(lib_dir, "libflock_gb300.so")):
        pytest.skip("library not built")
    r = subprocess.run(["g++", "-std=c++17", "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "drivers", "facade_main.cpp"), "-L", lib_dir, "-lflock_gb300",
                        f"-Wl,-rpath,{lib_dir}", "-o", str(tmp_path / "facade_main")],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr


def test_cli_usage_errors(tmp_path):
    cli = os.path.join(ROOT, "flock_gb300", "flock")
    if not os.path.exists(cli):
        pytest.skip("CLI not built")
    r = subprocess.run([cli], capture_output=True, text=True)
    assert r.returncode == 255 and "-i" in r.stderr
    r = subprocess.run([cli, "-i", str(tmp_path / "none.dat"), "-a", "parallel_uv"], capture_output=True, text=True)
    assert r.returncode == 255 and "doesn't exist" in r.stderr
    p = write(tmp_path, "ok.dat", "1 1\n1\n1\n1\n")
    r = subprocess.run([cli, "-i", p, "-a", "nonsense"], capture_output=True, text=True)
    assert r.returncode == 254 and "Invalid Algorithm" in r.stderr


def test_server_budget_rejection():
    s = fg.Server(memory_budget_bytes=1000)
    inst = fg.config_instance("uniform100", 0)
    with pytest.raises(fg.FlockError) as ex:
        s.submit(inst)
    assert ex.value.status == fg.FLOCK_ERR_BUDGET
    s.close()


def _write_dat(path, s, d, tokens):
    with open(path, "w") as f:
        f.write(f"{len(s)} {len(d)}\n")
        f.write(" ".join(str(x) for x in s) + "\n")
        f.write(" ".join(str(x) for x in d) + "\n")
        for k in range(0, len(tokens), 997):
            f.write(" ".join(tokens[k:k + 997]) + "\n")


def test_reader_parallel_large(tmp_path):
    """A multi-megabyte file (parsed in several chunks): decimal costs read
    exactly at the smallest exact scale."""
    rng = np.random.default_rng(5)
    m, n = 700, 650
    cents = rng.integers(0, 100000, size=m * n)
    toks = [f"{c // 100}.{c % 100:02d}" for c in cents]
    s = rng.integers(1, 50, size=m)
    d = np.zeros(n, np.int64)
    d[:] = s.sum() // n
    d[-1] += s.sum() - d.sum()
    p = str(tmp_path / "big.dat")
    _write_dat(p, s, d, toks)
    assert os.path.getsize(p) > 2 << 20                # several parse chunks
    inst, scale = fg.read_dat(p)
    assert scale == 2 or (scale < 2 and np.all(cents % 10 == 0))
    np.testing.assert_array_equal(inst.cost.ravel(), cents // (10 ** (2 - scale)))
    np.testing.assert_array_equal(inst.supply, s)
    np.testing.assert_array_equal(inst.demand, d)


def test_reader_parallel_error_order(tmp_path):
    """Several bad tokens: the error of the first one (in file order) is the
    one reported, as a sequential reader would, wherever the chunks fall."""
    rng = np.random.default_rng(6)
    m, n = 600, 600
    toks = [str(x) for x in rng.integers(1, 1000, size=m * n)]
    s = np.full(m, 10)
    d = np.full(n, 10)

    def read(tokens, scale=0):
        p = str(tmp_path / "e.dat")
        _write_dat(p, s, d, tokens)
        with pytest.raises(fg.FlockError) as ex:
            fg.read_dat(p, scale=scale)
        return ex.value.status

    t = list(toks); t[200000] = "1.5"; t[300000] = "x7"
    assert read(t) == fg.FLOCK_ERR_INEXACT            # inexact comes first
    t = list(toks); t[100] = "x7"; t[300000] = "1.5"
    assert read(t) == fg.FLOCK_ERR_PARSE               # bad text comes first
    t = list(toks); t[250000] = str((1 << 30) + 1)
    assert read(t) == fg.FLOCK_ERR_RANGE
    t = list(toks[:-5]); t[1000] = "2.5"
    assert read(t) == fg.FLOCK_ERR_INEXACT             # before the missing tokens
    assert read(toks[:-5]) == fg.FLOCK_ERR_PARSE       # missing tokens


def test_binary_instance_round_trip(tmp_path):
    inst = fg.generate(0, 9, 123, 77, -1000, 1000, 1, 100)
    p = str(tmp_path / "x.fbin")
    fg.write_bin(inst, p)
    assert os.path.getsize(p) == 16 + 4 * (123 + 77 + 123 * 77)
    back = fg.read_bin(p)
    np.testing.assert_array_equal(back.supply, inst.supply)
    np.testing.assert_array_equal(back.demand, inst.demand)
    np.testing.assert_array_equal(back.cost, inst.cost)
    with open(p, "r+b") as f:
        f.truncate(100)
    with pytest.raises(fg.FlockError) as ex:
        fg.read_bin(p)
    assert ex.value.status == fg.FLOCK_ERR_PARSE


def test_parallel_loop_concurrent_callers(flock_lib):
    """The batch call's host parallel loop (a worker pool started once): every
    item runs exactly once, also with several host threads calling at once
    (a caller that finds the pool busy runs its loop alone)."""
    import threading
    f = flock_lib.flock_test_parallel_for
    f.argtypes = [ctypes.c_int32, ctypes.POINTER(ctypes.c_int32)]
    f.restype = ctypes.c_int
    assert f(-1, None) == fg.FLOCK_ERR_ARG
    assert f(0, None) == fg.FLOCK_OK
    errors = []

    def caller(seed):
        rng = np.random.default_rng(seed)
        for _ in range(150):
            n = int(rng.integers(1, 6000))
            hits = np.zeros(n, dtype=np.int32)
            rc = f(n, hits.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)))
            if rc != fg.FLOCK_OK or not (hits == 1).all():
                errors.append((seed, n, rc))

    threads = [threading.Thread(target=caller, args=(s,)) for s in range(4)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors[:3]


def test_dat_writer_round_trip(tmp_path):
    """flock_write_dat: the reference's file layout, and the reader returns the
    same integers at the same scale (negative costs and zero included)."""
    rng = np.random.default_rng(3)
    s = rng.integers(0, 50, 7).astype(np.int32)
    d = rng.integers(0, 50, 9).astype(np.int32)
    d[-1] += int(s.sum() - d.sum())
    c = rng.integers(-50000, 50000, (7, 9)).astype(np.int32)
    c[0, 0] = 0
    inst = fg.Instance(s, d, c)
    for scale in (0, 2, 3):
        p = str(tmp_path / f"x{scale}.dat")
        fg.write_dat(inst, p, scale)
        back, sc = fg.read_dat(p, scale)
        assert sc == scale
        np.testing.assert_array_equal(back.supply, s)
        np.testing.assert_array_equal(back.demand, d)
        np.testing.assert_array_equal(back.cost, c)
    p = str(tmp_path / "small.dat")
    small = fg.Instance(np.array([3, 2], np.int32), np.array([1, 4], np.int32),
                        np.array([[150, 7], [-5, 200]], np.int32))
    fg.write_dat(small, p, 2)
    assert open(p).read() == "2 2\n3\t2\t\n1\t4\t\n1.5\n0.07\n-0.05\n2.0\n"
    with pytest.raises(fg.FlockError):
        fg.write_dat(small, p, 10)


def test_dat_writer_reproduces_reference_files(tmp_path):
    """Read at scale 2 and written back, the reference's own data files come
    out byte for byte (where the reference checkout is present)."""
    from conftest import REFERENCE
    d = os.path.join(REFERENCE, "data")
    if not os.path.isdir(d):
        pytest.skip("reference data files not present")
    files = sorted(f for f in os.listdir(d) if f.endswith(".dat") and os.path.getsize(os.path.join(d, f)) < 500_000)
    assert files
    for f in files[:4]:
        inst, sc = fg.read_dat(os.path.join(d, f), 2)
        out = str(tmp_path / f)
        fg.write_dat(inst, out, 2)
        assert open(out, "rb").read() == open(os.path.join(d, f), "rb").read(), f
