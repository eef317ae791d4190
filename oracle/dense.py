"""numpy restatement of the reference's dense Rank DP executor (test infrastructure only).

run_plan_numpy   cdist/kernel.py:72-91      (uint8, INF = 255, saturating +1)
final_value      cdist/kernel.py:18-25      (OverflowError at INF)
witness          cdist/auto.py:126-182      (traceback through the recorded tables)
brute            tests/test_dp.py:12-23
The uint16 / weighted variants restate the rule of cdist/viterbi.c:204-219
(T[s] = min(T[s], min(T[s^h] + w, INF))) with INF = 65535 for 16-bit tables; the reference
has no caller for them (parity for those rests on brute force).
"""
from __future__ import annotations

import itertools

import numpy as np

INF8 = 255
INF16 = 65535


def final_value(entry, inf=INF8):
    v = int(entry)
    if v == inf:
        raise OverflowError("the distance is at least %d, beyond the table entries" % inf)
    return v


def apply_op(T, op, inf=INF8):
    """One plan op on a numpy table; returns the new table."""
    dt = T.dtype
    if op[0] == "expand":
        return np.concatenate([T, np.full(T.size, inf, dtype=dt)])
    if op[0] == "update":
        h = int(op[1])
        w = int(op[2]) if len(op) > 2 else 1
        other = T[np.arange(T.size, dtype=np.int64) ^ h].astype(np.int64)
        other = np.where(other == inf, inf, np.minimum(other + w, inf))
        return np.minimum(T, other.astype(dt))
    _, pos, target = op
    idx = np.arange(T.size, dtype=np.int64)
    return np.ascontiguousarray(T[((idx >> pos) & 1) == target])


def run_plan_numpy(plan, dtype=np.uint8, tables=None):
    """Minimum cost of a feasible plan, None if infeasible; OverflowError at INF.
    tables: optional list that receives a copy of the table after every op."""
    if not plan.feasible:
        return None
    inf = INF8 if np.dtype(dtype) == np.uint8 else INF16
    T = np.zeros(1, dtype=dtype)
    for op in plan.ops:
        T = apply_op(T, op, inf)
        if tables is not None:
            tables.append(T.copy())
    assert T.size == 1
    return final_value(T[0], inf)


def table_after(plan, nops, dtype=np.uint8):
    """The table after the first nops ops."""
    inf = INF8 if np.dtype(dtype) == np.uint8 else INF16
    T = np.zeros(1, dtype=dtype)
    for op in plan.ops[:nops]:
        T = apply_op(T, op, inf)
    return T


def brute(h, l, obs_mask, weights=None):
    """Least weight of a column set with zero syndrome and odd overlap with obs_mask, by
    exhaustive enumeration (small problems only)."""
    n = len(h)
    best = None
    for k in range(1, n + 1):
        if weights is None and best is not None:
            break
        for sup in itertools.combinations(range(n), k):
            s = lg = 0
            for j in sup:
                s ^= h[j]
                lg ^= l[j]
            if s == 0 and bin(lg & obs_mask).count("1") & 1:
                c = k if weights is None else sum(weights[j] for j in sup)
                if best is None or c < best:
                    best = c
    return best


def witness(h, l, order, nrows, obs, make_span_form, reduce_target, lowbit, inf=INF8):
    """Columns of a minimum solution by the traceback of cdist/auto.py:126-182 (unit weights).
    The planner's reduction functions are passed in so that this stays free of package imports."""
    hrows = make_span_form(h, order, nrows)
    lrow = 0
    for pos, j in enumerate(order):
        if (l[j] >> obs) & 1:
            lrow |= 1 << pos
    lrow = reduce_target(lrow, hrows)
    if lrow == 0:
        return None
    rows = [(r, 0) for r in hrows] + [(lrow, 1)]
    start_at, end_at = {}, {}
    for idx, (r, _) in enumerate(rows):
        start_at.setdefault(lowbit(r), []).append(idx)
        end_at.setdefault(r.bit_length() - 1, []).append(idx)
    active, hist = [], []
    T = np.zeros(1, dtype=np.uint8)
    for j in range(len(order)):
        for idx in start_at.get(j, ()):
            active.append(idx)
            T = np.concatenate([T, np.full(T.size, inf, dtype=np.uint8)])
            hist.append(("expand", len(active) - 1))
        mask = sum(1 << pos for pos, idx in enumerate(active) if (rows[idx][0] >> j) & 1)
        if mask:
            other = T[np.arange(T.size, dtype=np.int64) ^ mask]
            other = np.where(other == inf, inf, other + 1).astype(np.uint8)
            hist.append(("update", mask, j, T))
            T = np.minimum(T, other)
        for pos in sorted((active.index(idx) for idx in end_at.get(j, ())), reverse=True):
            target = rows[active[pos]][1]
            T = T[((np.arange(T.size, dtype=np.int64) >> pos) & 1) == target]
            hist.append(("select", pos, target))
            active.pop(pos)
    state, value, used = 0, final_value(T[0]), []
    for step in reversed(hist):
        if step[0] == "select":
            _, pos, target = step
            state = ((state >> pos) << (pos + 1)) | (target << pos) | (state & ((1 << pos) - 1))
        elif step[0] == "update":
            _, mask, j, before = step
            if int(before[state]) != value:
                used.append(order[j])
                state ^= mask
                value -= 1
    assert value == 0
    return sorted(used)
