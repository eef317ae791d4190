"""Distance problems: columns as Python-int bitmasks over detector rows and observables.

Mirrors `cdist/problem.py:21-44` (the `Problem` record) and `cdist/problem.py:47-64`
(`dedupe`).  The distance is  d = min{|e| : XOR_j e_j h[j] = 0, XOR_j e_j l[j] != 0}.
"""
from __future__ import annotations

from dataclasses import dataclass, field


@dataclass
class Problem:
    name: str
    nrows: int
    nobs: int
    h: list            # detector bitmask of each column
    l: list            # observable bitmask of each column
    row_meta: list = field(default_factory=list)
    col_meta: list = field(default_factory=list)
    notes: dict = field(default_factory=dict)
    weights: list = None     # per-column integer weight (None: every column costs 1)

    @property
    def ncols(self):
        return len(self.h)

    def check(self, support):
        """(syndrome, logical) of a set of columns."""
        s = lg = 0
        for j in support:
            s ^= self.h[j]
            lg ^= self.l[j]
        return s, lg

    def weight_of(self, support):
        if self.weights is None:
            return len(support)
        return sum(self.weights[j] for j in support)


def dedupe(h, l, meta=None):
    """Drop all-zero columns and merge identical (h, l) columns; returns (h, l, merged meta)."""
    seen = {}
    oh, ol, om = [], [], []
    for j, (a, b) in enumerate(zip(h, l)):
        if a == 0 and b == 0:
            continue
        key = (a, b)
        if key in seen:
            if meta is not None:
                om[seen[key]].append(meta[j])
            continue
        seen[key] = len(oh)
        oh.append(a)
        ol.append(b)
        om.append([meta[j]] if meta is not None else [j])
    return oh, ol, om


def verify_witness(p: Problem, cols, obs=None):
    """True if the columns form a logical: zero syndrome, and the observable `obs` (or any) flipped."""
    s, lg = p.check(cols)
    if s != 0 or len(set(cols)) != len(cols):
        return False
    return bool((lg >> obs) & 1) if obs is not None else lg != 0
