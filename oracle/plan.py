"""Pure-Python restatement of the reference's trellis planning: TEST INFRASTRUCTURE ONLY.

The CPU arm of the benchmark and the parity tests plan with this module, so that they load no
library of the product (the product plans with its own C++ builder; the two are compared op for
op in tests/test_oracle_dense.py).

  rows_by_position   cdist/trellis.py:47-57    row r as a bitmask over column positions
  span_form          cdist/trellis.py:60-97    minimal span form: distinct starts, distinct ends
  shorten_target     cdist/trellis.py:100-122  the target row reduced by the constraint rows
  schedule           cdist/trellis.py:147-182  the op stream (expand / update / select)
  plan               cdist/trellis.py:185-193  the query  H e = 0, (mask . L) e = 1
  encoded            the op stream as int64 rows (code, a, b) for oracle/dense_port.c

The reduction steps are the reference's: the rows they produce fix which row sits on which
table bit, and the tables are compared entry for entry at checkpoints.
"""
from __future__ import annotations

import numpy as np

EXPAND, UPDATE, SELECT = 0, 1, 2


def _start(x):
    return (x & -x).bit_length() - 1


def rows_by_position(cols, order, nrows):
    rows = [0] * nrows
    for pos, j in enumerate(order):
        rest = cols[j]
        while rest:
            one = rest & -rest
            rows[one.bit_length() - 1] |= 1 << pos
            rest ^= one
    return rows


def span_form(rows):
    """Rows with pairwise distinct first and last positions spanning the same space."""
    first = {}
    for r in rows:
        while r:
            s = _start(r)
            held = first.get(s)
            if held is None:
                first[s] = r
                break
            if r.bit_length() < held.bit_length():      # the shorter row keeps the start
                first[s], held, r = r, r, held
            r ^= held
    last = {}
    for r in sorted(first.values(), key=_start, reverse=True):
        while True:
            e = r.bit_length()
            held = last.get(e)
            if held is None:
                last[e] = r
                break
            if _start(held) > _start(r):
                r ^= held                              # r loses the shared end, keeps its start
            else:
                last[e], r = r, held ^ r                # r takes the end, the sum moves on
    return list(last.values())


def shorten_target(lrow, hrows):
    """0 when the target row lies in the span of the constraint rows (infeasible query)."""
    first = {_start(r): r for r in hrows}
    last = {r.bit_length(): r for r in hrows}

    def strip_front(x):
        while x and _start(x) in first:
            x ^= first[_start(x)]
        return x
    lrow = strip_front(lrow)
    while lrow:
        held = last.get(lrow.bit_length())
        if held is None or _start(held) < _start(lrow):
            break
        lrow = strip_front(lrow ^ held)
    return lrow


class Schedule:
    """ops, peak_bits and work() of one query, as the reference's Plan holds them."""

    def __init__(self, ops, peak_bits, feasible=True):
        self.ops, self.peak_bits, self.feasible = ops, peak_bits, feasible

    def work(self):
        bits = total = 0
        for op in self.ops:
            if op[0] == "expand":
                bits += 1
            elif op[0] == "select":
                bits -= 1
            else:
                total += 1 << bits
        return total

    def encoded(self):
        out = np.zeros((len(self.ops), 3), dtype=np.int64)
        for i, op in enumerate(self.ops):
            if op[0] == "expand":
                out[i, 0] = EXPAND
            elif op[0] == "update":
                out[i] = (UPDATE, op[1], op[2] if len(op) > 2 else 1)
            else:
                out[i] = (SELECT, op[1], op[2])
        return out


def schedule(hrows, lrow, ncols):
    if lrow == 0:
        return Schedule([], 0, feasible=False)
    rows = list(hrows) + [lrow]
    opens, closes = {}, {}
    for k, r in enumerate(rows):
        opens.setdefault(_start(r), []).append(k)
        closes.setdefault(r.bit_length() - 1, []).append(k)
    live, ops, peak = [], [], 0
    for j in range(ncols):
        for k in opens.get(j, ()):
            live.append(k)
            ops.append(("expand",))
        peak = max(peak, len(live))
        mask = sum(1 << b for b, k in enumerate(live) if (rows[k] >> j) & 1)
        if mask:
            ops.append(("update", mask))
        for b in sorted((live.index(k) for k in closes.get(j, ())), reverse=True):
            ops.append(("select", b, 1 if live[b] == len(rows) - 1 else 0))
            del live[b]
    assert not live
    return Schedule(ops, peak)


def plan(h, l, obs_mask, order, nrows):
    hrows = span_form(rows_by_position(h, order, nrows))
    lrow = 0
    for pos, j in enumerate(order):
        if bin(l[j] & obs_mask).count("1") & 1:
            lrow |= 1 << pos
    return schedule(hrows, shorten_target(lrow, hrows), len(order))
