"""Seeded synthetic distance problems of the benchmark workloads.

banded(m, n, window, ...)      random banded LDPC problem: column i has `col_weight` distinct checks
                               drawn uniformly in a window of rows centred on floor(i*m/n) (clipped to
                               the matrix); each logical row is i.i.d. Bernoulli(p_logical) over the
                               columns, resampled until it is not in the row space of H.
dense_small(seed)              m=120, n=240, window 16, one logical row (frontier <= 16 bits)
dense_scale(seed, window)      m=1000, n=2000, window 30 as specified, 4 logical rows; a wider window
                               (36-38) raises the frontier to 30-31 bits (a 1-2 GB uint8 table)
circuit_dem(seed, ...)         circuit-style detector error model: rounds x checks detectors, each
                               column flips 1-4 detectors (p = .1/.5/.3/.1) in its round or the next,
                               observable bit Bernoulli(0.05), integer weights uniform in {1,2,3}
batch_instances(seed, count)   uneven banded instances with target widths 12..26 for batching
All generators are deterministic in their seed (numpy PCG64).
"""
from __future__ import annotations

import numpy as np

from .problem import Problem


def gf2_rank(rows):
    piv = {}
    r = 0
    for v in rows:
        while v:
            t = v.bit_length() - 1
            q = piv.get(t)
            if q is None:
                piv[t] = v
                r += 1
                break
            v ^= q
    return r


def _row_space_member(hrows_basis, v):
    """True if v is in the span of the reduced basis {top bit: row}."""
    while v:
        q = hrows_basis.get(v.bit_length() - 1)
        if q is None:
            return False
        v ^= q
    return True


def _basis(rows):
    piv = {}
    for v in rows:
        while v:
            t = v.bit_length() - 1
            q = piv.get(t)
            if q is None:
                piv[t] = v
                break
            v ^= q
    return piv


def _rows_of(h, m, n):
    rows = [0] * m
    for j, c in enumerate(h):
        while c:
            low = c & -c
            rows[low.bit_length() - 1] |= 1 << j
            c ^= low
    return rows


def banded(m, n, window, col_weight=3, nobs=1, seed=0, p_logical=0.5, name=None):
    rng = np.random.default_rng(seed)
    window = min(window, m)
    h = []
    for i in range(n):
        c = (i * m) // n
        lo = min(max(0, c - window // 2), m - window)
        rows = rng.choice(window, size=col_weight, replace=False) + lo
        h.append(int(sum(1 << int(r) for r in rows)))
    basis = _basis(_rows_of(h, m, n))
    lrows = []
    if len(basis) >= n:
        raise ValueError("H has full column rank: every logical row is in its row space")
    for _ in range(nobs):
        for _attempt in range(10000):
            bits = rng.random(n) < p_logical
            v = int(sum(1 << j for j in np.flatnonzero(bits).tolist()))
            if v and not _row_space_member(basis, v):
                break
        else:
            raise ValueError("no logical row outside the row space of H was drawn")
        lrows.append(v)
    l = [0] * n
    for o, v in enumerate(lrows):
        for j in range(n):
            if (v >> j) & 1:
                l[j] |= 1 << o
    return Problem(name or "banded_m%d_n%d_w%d_s%d" % (m, n, window, seed), m, nobs, h, l,
                   [(r, 0) for r in range(m)], notes={"window": window, "seed": seed})


def dense_small(seed=0):
    """m=120 x n=240, window 16, one logical row: the CPU-runnable dense workload."""
    return banded(120, 240, 16, 3, 1, seed)


def dense_scale(seed=0, window=30):
    """m=1000 x n=2000, four logical rows taken one at a time."""
    return banded(1000, 2000, window, 3, 4, seed)


def circuit_dem(seed=0, rounds=40, checks=150, ncols=20000, p_obs=0.05, weights=(1, 2, 3), spread=6):
    """Circuit-style DEM.  A column picks a round r and a check c; its 1-4 detectors are (r or r+1,
    c + offset) with offsets within +-spread (clipped), the first one at (r, c)."""
    rng = np.random.default_rng(seed)
    m = rounds * checks
    h, l, wts = [], [], []
    seen = set()
    while len(h) < ncols:
        k = int(rng.choice(4, p=[0.1, 0.5, 0.3, 0.1])) + 1
        r = int(rng.integers(rounds))
        c = int(rng.integers(checks))
        dets = {r * checks + c}
        while len(dets) < k:
            rr = min(rounds - 1, r + int(rng.integers(2)))
            cc = min(checks - 1, max(0, c + int(rng.integers(-spread, spread + 1))))
            dets.add(rr * checks + cc)
        col = int(sum(1 << d for d in dets))
        ob = int(rng.random() < p_obs)
        if (col, ob) in seen:
            continue
        seen.add((col, ob))
        h.append(col)
        l.append(ob)
        wts.append(int(rng.choice(weights)))
    order = sorted(range(ncols), key=lambda j: (h[j] & -h[j]).bit_length())
    h = [h[j] for j in order]
    l = [l[j] for j in order]
    wts = [wts[j] for j in order]
    return Problem("dem_r%d_c%d_n%d_s%d" % (rounds, checks, ncols, seed), m, 1, h, l,
                   [(i % checks, i // checks) for i in range(m)], weights=wts,
                   notes={"rounds": rounds, "checks": checks, "seed": seed})


def batch_instances(seed=0, count=256, wmin=12, wmax=26, max_obs=12):
    """Uneven banded instances: target width w ~ U[wmin, wmax], n = 8*w*U(4,12) columns,
    m = n/2, 1..max_obs logical rows, window about w / 0.85 (the measured cut rank of these
    banded problems is 0.8-0.9 x window)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        w = int(rng.integers(wmin, wmax + 1))
        n = int(8 * w * rng.integers(4, 13))
        m = n // 2
        window = max(4, int(round(w / 0.85)))
        nobs = int(rng.integers(1, max_obs + 1))
        p = banded(m, n, window, 3, nobs, seed=int(rng.integers(1 << 31)))
        p.notes["target_width"] = w
        out.append(p)
    return out
