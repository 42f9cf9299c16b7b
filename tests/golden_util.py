"""Helpers shared by the tests and tests/golden/make_golden.py: seeded tiny
degenerate instances, float views of exact integer costs, checksums."""
import hashlib

import numpy as np


def tiny(seed, count, max_dim=8):
    """Tiny balanced instances with heavy ties and zero quantities."""
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
        out.append((s, d, c))
    return out


def float_costs(ci, scale):
    """The reference's float cost of an exact integer cost * 10^-scale."""
    return np.asarray([np.float32(k / 10.0 ** scale) for k in ci], np.float32)


def checksum(s, d, c):
    h = hashlib.sha256()
    for a in (s, d, c):
        h.update(np.ascontiguousarray(a, dtype=np.int32).tobytes())
    return h.hexdigest()[:16]
