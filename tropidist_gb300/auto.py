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


_SIDE = {}


def _side_stream():
    """A second stream of the current device for the observables' sweeps (created once)."""
    import torch
    dev = torch.cuda.current_device()
    if dev not in _SIDE:
        _SIDE[dev] = torch.cuda.Stream(device=dev)
    return _SIDE[dev]


def dp_distance(p, order, max_table_bytes=None, deadline=None, dtype=None):
    """Exact distance min over observables i of min{|e| : H e = 0, (L e)_i = 1}; None if no
    logical exists.  MemoryError if a table would exceed max_table_bytes, TimeoutError past the
    deadline (time.monotonic), OverflowError if a distance reaches the table's INF.

    The observables' sweeps are queued on two streams in turn (each with its own pair of tables,
    while both pairs fit in half the free device memory), so that one sweep's pass boundaries
    overlap the other's passes; their final entries are copied on the device.  The host plans and
    schedules observable i + 1 while the GPU sweeps observable i, and waits once at the end."""
    import torch
    from . import device
    device.require_gpu()
    dtype = dtype or _dtype_for(p)
    eb = kernel.entry_bytes(dtype)
    inf = kernel.INF if eb == 1 else kernel.INF16
    per, slots = [], []
    main = torch.cuda.current_stream()
    lanes = [main, _side_stream()]
    bufs = [[None, None], [None, None]]
    free_bytes = torch.cuda.mem_get_info()[0]
    res = None
    nrun = 0
    for i, plan in _plans(p, order):
        if deadline is not None and time.monotonic() > deadline:
            torch.cuda.synchronize()
            raise TimeoutError("DP stopped at the time limit")
        if not plan.feasible:
            per.append(None)
            continue
        if max_table_bytes is not None and (eb << plan.peak_bits) > max_table_bytes:
            raise MemoryError("DP table of 2^%d entries exceeds the limit" % plan.peak_bits)
        need = eb << plan.peak_bits
        lane = nrun % 2 if 4 * need <= free_bytes // 2 else 0
        nrun += 1
        if bufs[lane][0] is None or bufs[lane][0].numel() < need:
            bufs[lane] = [device.empty(need), device.empty(need)]
        if res is None:
            res = torch.zeros(max(1, 2 * p.nobs), dtype=torch.uint8, device="cuda")
        st = lanes[lane]
        if lane:
            st.wait_stream(main)
        a, b = bufs[lane]
        # scheduled and launched together: the first passes run while the rest is scheduled
        cp = kernel.CompiledPlan(plan, dtype, launch=(a, b, st.cuda_stream))
        k = len(per)
        with torch.cuda.stream(st):
            res[eb * k:eb * k + eb].copy_((b if cp.final_buf else a)[:eb])
        cp.free()
        per.append(k)
        slots.append(k)
    main.wait_stream(lanes[1])
    vals = res.cpu().numpy() if res is not None else None
    best = None
    out = []
    for x in per:
        if x is None:
            out.append(None)
            continue
        raw = int(vals[eb * x]) if eb == 1 else int(vals[eb * x]) | (int(vals[eb * x + 1]) << 8)
        v = kernel.final_value(raw, inf)
        out.append(v)
        if best is None or v < best:
            best = v
    return best, out


# ---------------------------------------------------------------------- witness
def _widths(ops):
    """Table width before every op and after the last one."""
    w, out = 0, [0]
    for op in ops:
        w += 1 if op[0] == "expand" else -1 if op[0] == "select" else 0
        out.append(w)
    return out


SMALL_WITNESS_BYTES = 256 << 20      # every table of a sweep kept on the device up to this size


def _witness_small(cands, order, eb, inf):
    """dp_witness for plans whose tables all fit SMALL_WITNESS_BYTES together: per observable one
    launch that runs the sweep keeping every table and walks back on the device
    (tg_dense_witness_small); None when a plan is larger."""
    import numpy as np
    import torch
    from . import _lib, device
    L = _lib.lib()
    encs = [np.ascontiguousarray(plan.encode(), dtype=np.int64) for _, plan in cands]
    sizes = [int(L.tg_dense_witness_bytes(e.ctypes.data if len(e) else None, len(e), eb)) for e in encs]
    if any(sz < 0 or sz > SMALL_WITNESS_BYTES for sz in sizes):
        return None
    best = None
    for (i, plan), enc, sz in zip(cands, encs, sizes):
        nupd = int((enc[:, 0] == trellis.OP_UPDATE).sum()) if len(enc) else 0
        tabs = torch.empty(max(sz, 1), dtype=torch.uint8, device="cuda")
        out = torch.empty(3 + nupd, dtype=torch.int32, device="cuda")
        _lib.check(L.tg_dense_witness_small(enc.ctypes.data if len(enc) else None, len(enc), eb, tabs.data_ptr(),
                                            sz, out.data_ptr(), nupd, device.stream_ptr()))
        o = out.cpu().numpy()
        status = int(o[2 + nupd])
        if status == 1:
            raise ValueError("witness: op stream out of range")
        if status == 2:
            raise AssertionError("traceback lost the path")
        v = kernel.final_value(int(o[0]) & (0xFF if eb == 1 else 0xFFFF), inf)
        if best is None or v < best[0]:
            best = (v, i, plan, o[2:2 + int(o[1])].tolist())
    value, i, plan, ks = best
    upd_index = np.cumsum(plan.encode()[:, 0] == trellis.OP_UPDATE) - 1
    used = [order[plan.columns[int(upd_index[k])]] for k in ks]
    return {"distance": value, "witness": sorted(used), "observable": i}


def dp_witness(p, order, obs=None, dtype=None, budget_bytes=None, leaf=16):
    """Columns (problem indices) of a minimum-weight solution, with its weight and observable:
    {"distance", "witness", "observable"} (cdist/auto.py:126-182), or None if no logical exists.

    The reference keeps the table before every update and walks back through them.  Here the
    tables stay on the device: the sweep keeps canonical tables at checkpoints (as many as fit
    `budget_bytes`, default a quarter of the free device memory), and each segment between two
    checkpoints is walked back by bisection — the table at the segment's midpoint is recomputed
    from its start by a plan that begins with that table (tg_dense_plan_from), the second half is
    traced first — so only O(log segment) tables exist at once.  A leaf of at most `leaf` ops is
    recomputed with a table after every op; the walk reads two entries per update op.  Plans whose
    tables all fit SMALL_WITNESS_BYTES together take one launch per observable instead (every table
    kept, the walk back on the device)."""
    import torch
    from . import device
    dtype = dtype or _dtype_for(p)
    eb = kernel.entry_bytes(dtype)
    dt = torch.uint8 if eb == 1 else torch.int16
    inf = kernel.INF if eb == 1 else 65535
    cands = [(i, plan) for i, plan in _plans(p, order) if (obs is None or i == obs) and plan.feasible]
    if not cands:
        return None
    small = _witness_small(cands, order, eb, inf)
    if small is not None:
        return small
    best = None
    for i, plan in cands:
        v, _ = kernel.run_plan(plan, dtype=dtype)
        if v is not None and (best is None or v < best[0]):
            best = (v, i, plan)
    if best is None:
        return None
    value, i, plan = best
    ops, enc = plan.ops, plan.encode()
    n = len(ops)
    wid = _widths(ops)
    col_of = {}
    u = 0
    for k, op in enumerate(ops):
        if op[0] == "update":
            col_of[k] = order[plan.columns[u]]
            u += 1
    if budget_bytes is None:
        budget_bytes = device.free_bytes() // 4
    step = max(leaf, 1)
    while True:
        cks = list(range(step, n, step))
        if sum(eb << wid[c] for c in cks) <= budget_bytes or step >= n:
            break
        step *= 2
    cks = [c for c in range(step, n, step)]
    cp = kernel.CompiledPlan(plan, dtype, cks)
    a, b = cp.buffers()
    ck_tabs = [torch.empty(1 << wid[c], dtype=dt, device="cuda") for c in cp.ckpts]
    cp.execute(a, b, [t.view(torch.uint8) for t in ck_tabs])
    cp.free()
    tabs = {0: torch.zeros(1, dtype=dt, device="cuda")}
    for c, t in zip(cp.ckpts, ck_tabs):
        tabs[int(c)] = t
    del a, b

    def entry(t, s):
        x = int(t[s].item())
        return x & 0xFFFF if eb == 2 else x

    def run_from(t0, lo, hi, keep_all=False):
        """Tables after ops lo..hi-1 from table t0 (before op lo): the last one, or all of them."""
        sub = enc[lo:hi]
        ck = list(range(1, hi - lo)) if keep_all else []
        c2 = kernel.CompiledPlan(None, dtype, ck, w_start=wid[lo], ops=sub)
        n_a = max(1 << max(wid[lo:hi + 1]), 1)
        a2 = torch.empty(n_a, dtype=dt, device="cuda")
        b2 = torch.empty(n_a, dtype=dt, device="cuda")
        a2[:t0.numel()].copy_(t0)
        outs = [torch.empty(1 << wid[lo + k], dtype=dt, device="cuda") for k in ck]
        c2.execute(a2.view(torch.uint8), b2.view(torch.uint8), [o.view(torch.uint8) for o in outs])
        last = (b2 if c2.final_buf else a2)[:1 << wid[hi]].clone()
        c2.free()
        return (outs + [last]) if keep_all else last

    used = []

    def trace(lo, hi, t_lo, s, v):
        if hi - lo <= leaf:
            after = run_from(t_lo, lo, hi, keep_all=True) if hi - lo > 1 else []
            before = [t_lo] + after[:-1] if after else [t_lo]
            for k in range(hi - 1, lo - 1, -1):
                op, t = ops[k], before[k - lo]
                if op[0] == "select":
                    pos, tgt = op[1], op[2]
                    s = ((s >> pos) << (pos + 1)) | (tgt << pos) | (s & ((1 << pos) - 1))
                elif op[0] == "expand":
                    assert s >> wid[k] == 0, "traceback through an INF half"
                elif entry(t, s) != v:
                    mask, w = op[1], (op[2] if len(op) > 2 else 1)
                    s ^= mask
                    v -= w
                    assert entry(t, s) == v, "traceback lost the path"
                    used.append(col_of[k])
            return s, v
        mid = (lo + hi) // 2
        t_mid = run_from(t_lo, lo, mid)
        s, v = trace(mid, hi, t_mid, s, v)
        del t_mid
        return trace(lo, mid, t_lo, s, v)

    bounds = [0] + [int(c) for c in cp.ckpts] + [n]
    s, v = 0, value
    for lo, hi in reversed(list(zip(bounds, bounds[1:]))):
        s, v = trace(lo, hi, tabs[lo], s, v)
    assert s == 0 and v == 0, (s, v)
    return {"distance": value, "witness": sorted(used), "observable": i}
