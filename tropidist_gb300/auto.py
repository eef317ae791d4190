"""Dense Rank DP front end (drop-in for the dense half of cdist/auto.py).

  estimate(p)          largest table and work of every logical query for the best of the
                       natural and reversed column orders (cdist/auto.py:79-102)
  dp_distance(p, ord)  exact distance, one GPU sweep per logical observable
                       (cdist/auto.py:105-123): MemoryError / TimeoutError / OverflowError as there
  dp_witness(p, ord)   columns of a minimum solution by a traceback through device-resident table
                       checkpoints (cdist/auto.py:126-182)
Column ordering heuristics (cdist/ordering.py) stay on the caller's side: pass the order.
"""
from __future__ import annotations

import math
import time

from . import kernel, trellis

# state-updates per second of the GPU executor, for predictions only (measured on GB300 with the
# fused passes; tables narrower than ~20 bits are launch-bound and slower)
RATE_GPU = 5.0e12


def predicted_seconds(work, width=30):
    rate = RATE_GPU if width >= 22 else RATE_GPU * 2.0 ** (width - 22)
    return work / max(rate, 1e9)


def profile_cost(lam):
    """(peak, log2 of the total table volume) of a cut profile (cdist/ordering.py:10-14)."""
    peak = max(lam)
    vol = sum(2.0 ** (x - peak) for x in lam)
    return peak, peak + math.log2(vol)


def best_order(p, orders=None):
    """Smallest (peak cut rank, log2 volume) among the natural order, its reverse and any given
    orders (cdist/auto.py:48-64 without the greedy heuristics)."""
    cands = [list(range(p.ncols)), list(reversed(range(p.ncols)))] + [list(o) for o in (orders or ())]
    best = None
    for c in cands:
        cost = profile_cost(trellis.cut_profile(p.h, c))
        if best is None or cost < best[0]:
            best = (cost, c)
    return best[1], best[0]


def _plans(p, order):
    """One plan per logical observable; the span form of H is shared (cdist/auto.py:67-76)."""
    hrows = trellis.minimal_span_form(trellis.rows_from_columns(p.h, order, p.nrows))
    pw = None if getattr(p, "weights", None) is None else [p.weights[j] for j in order]
    for i in range(p.nobs):
        lrow = trellis.reduce_target_row(trellis.target_row(p.l, 1 << i, order), hrows)
        yield i, trellis.make_plan(hrows, lrow, len(order), pw)


def estimate(p, order=None, max_table_bytes=None):
    """DP cost of the order (or the best of natural / reversed); nothing is allocated."""
    t0 = time.time()
    if order is None:
        order, cost = best_order(p)
    else:
        cost = profile_cost(trellis.cut_profile(p.h, order))
    out = {"order": order, "cut_rank": int(cost[0]), "queries": p.nobs}
    if max_table_bytes is not None and cost[0] > math.log2(max_table_bytes):
        out.update(peak_bits=int(cost[0]), table_bytes=1 << int(cost[0]), work=None, predicted_seconds=math.inf,
                   fits=False, estimate_seconds=time.time() - t0)
        return out
    peak, work = 0, None
    for _, plan in _plans(p, order):
        if plan.feasible:
            peak, work = plan.peak_bits + (1 if p.nobs > 1 else 0), plan.work() * p.nobs
            break
    if work is None:
        work = 0
    out.update(peak_bits=peak, table_bytes=1 << peak, work=work, predicted_seconds=predicted_seconds(work, peak),
               fits=max_table_bytes is None or (1 << peak) <= max_table_bytes, estimate_seconds=time.time() - t0)
    return out


def _dtype_for(p):
    """uint8 tables unless column weights could push a distance past 254."""
    w = getattr(p, "weights", None)
    if w is None:
        return "u8"
    return "u16" if sum(w) >= 255 else "u8"


def dp_distance(p, order, max_table_bytes=None, deadline=None, dtype=None):
    """Exact distance min over observables i of min{|e| : H e = 0, (L e)_i = 1}; None if no
    logical exists.  MemoryError if a table would exceed max_table_bytes, TimeoutError past the
    deadline (time.monotonic), OverflowError if a distance reaches the table's INF."""
    dtype = dtype or _dtype_for(p)
    eb = kernel.entry_bytes(dtype)
    best = None
    per = []
    for i, plan in _plans(p, order):
        if deadline is not None and time.monotonic() > deadline:
            raise TimeoutError("DP stopped at the time limit")
        if not plan.feasible:
            per.append(None)
            continue
        if max_table_bytes is not None and (eb << plan.peak_bits) > max_table_bytes:
            raise MemoryError("DP table of 2^%d entries exceeds the limit" % plan.peak_bits)
        v, _ = kernel.run_plan(plan, dtype=dtype)
        per.append(v)
        if v is not None and (best is None or v < best):
            best = v
    return best, per
