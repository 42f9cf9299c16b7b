"""Independent LP optimum of a balanced transportation problem with SciPy's
HiGHS solver (test infrastructure: a cross-check of the exact optima, not a
solver of this library).  Integer data and a totally unimodular constraint
matrix: the LP optimum is integral, so it is compared exactly."""
import numpy as np


def lp_optimum(supply, demand, cost) -> int:
    from scipy.optimize import linprog
    from scipy.sparse import coo_matrix
    s = np.asarray(supply, np.int64)
    d = np.asarray(demand, np.int64)
    c = np.asarray(cost, np.int64).reshape(len(s), len(d))
    m, n = c.shape
    rows = np.concatenate([np.repeat(np.arange(m), n), m + np.tile(np.arange(n), m)])
    cols = np.concatenate([np.arange(m * n), np.arange(m * n)])
    A = coo_matrix((np.ones(2 * m * n), (rows, cols)), shape=(m + n, m * n)).tocsr()
    b = np.concatenate([s, d]).astype(np.float64)
    r = linprog(c.ravel().astype(np.float64), A_eq=A, b_eq=b, bounds=(0, None), method="highs")
    assert r.status == 0, r.message
    return int(round(r.fun))
