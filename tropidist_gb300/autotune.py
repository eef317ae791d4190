"""Per-width autotuning of the dense Rank DP schedule.

The scheduler (libtropigpu build_dense_plan) has two knobs that set how many columns one HBM pass
fuses and how the work is laid out: the fused tile width (`dmax`, rows of a pass's tile: 2^dmax
entries) and the update span of a coset-streaming pass (3 dimensions in a thread's registers, or 4
with a lane-pair dimension), with its variant for passes that close an in-chunk row.  The best
choice depends on the table width (narrow tables are launch- and latency-bound, wide ones are
bandwidth- or ALU-bound), so `tune` times every candidate on a seeded banded plan of each width and
keeps the fastest; `apply(width)` sets the library's knobs before a plan of that width is
scheduled (the schedule is fixed when the plan is compiled, so plans compiled under different
settings can run side by side).

No counterpart in the reference, whose C kernels have no tunable fusion (cdist/viterbi.c).
"""
from __future__ import annotations

import json
import time

from . import _lib, device, kernel, synth, trellis

DEFAULT = (16, 3, 2)                     # dmax, span, span when an in-chunk row closes
CANDIDATES = [(16, 3, 2), (16, 3, 3), (16, 4, 3), (14, 3, 2)]


def set_knobs(knobs):
    dmax, span, span_sel = knobs
    L = _lib.lib()
    _lib.check(L.tg_dense_set_tuning(int(dmax), 15, 15, 14))
    _lib.check(L.tg_dense_set_stream_span(int(span), int(span_sel)))


def _probe_plan(width, seed):
    """A seeded banded plan whose frontier reaches about `width` bits (cut ~ 0.85 x window)."""
    window = max(4, int(round(width / 0.85)))
    n = 8 * width * 6
    p = synth.banded(n // 2, n, window, 3, 1, seed=seed)
    return trellis.build_plan(p.h, p.l, 1, list(range(p.ncols)), p.nrows)


def _time_plan(plan, reps=3):
    import torch
    cp = kernel.CompiledPlan(plan)
    a, b = cp.buffers()
    cp.execute(a, b)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    st = torch.cuda.current_stream()
    e0.record(st)
    for _ in range(reps):
        cp.execute(a, b)
    e1.record(st)
    torch.cuda.synchronize()
    v = cp.result(a, b)
    cp.free()
    return e0.elapsed_time(e1) / reps, v


class Tuner:
    """Width -> (dmax, span, span_sel) table, measured by `tune` or loaded from JSON."""

    def __init__(self, table=None):
        self.table = {int(k): tuple(v[:3]) for k, v in (table or {}).items()}
        self.timings = {}

    def tune(self, widths, candidates=CANDIDATES, seed=0, reps=3):
        device.require_gpu()
        for w in widths:
            plan = _probe_plan(w, seed + w)
            if not plan.feasible:
                continue
            best, rows, ref = None, [], None
            for cand in candidates:
                set_knobs(cand)
                ms, v = _time_plan(plan, reps)
                if ref is None:
                    ref = v
                if v != ref:
                    raise AssertionError("schedules disagree at width %d: %s" % (w, (cand, v, ref)))
                rows.append((cand, ms))
                if best is None or ms < best[1]:
                    best = (cand, ms)
            self.table[int(plan.peak_bits)] = best[0]
            self.timings[int(plan.peak_bits)] = rows
        set_knobs(DEFAULT)
        return self

    def knobs(self, width):
        """The knobs of the nearest tuned width at or below `width` (the default if none)."""
        ws = [w for w in self.table if w <= width]
        return self.table[max(ws)] if ws else (self.table[min(self.table)] if self.table else DEFAULT)

    def apply(self, width):
        set_knobs(self.knobs(width))

    def to_json(self):
        return json.dumps({str(w): list(k) for w, k in sorted(self.table.items())})

    def report(self):
        """{width: {"dmax": .., "span": .., "span_sel": .., "ms": {candidate: ms}}}"""
        out = {}
        for w, k in sorted(self.table.items()):
            out[w] = {"dmax": k[0], "span": k[1], "span_sel": k[2],
                      "ms": {"%d/%d/%d" % c: round(ms, 3) for c, ms in self.timings.get(w, [])}}
        return out


def compiled(plan, tuner=None, dtype="u8"):
    """CompiledPlan scheduled with the tuner's knobs for the plan's width (library defaults restored)."""
    if tuner is None:
        return kernel.CompiledPlan(plan, dtype)
    tuner.apply(plan.peak_bits)
    try:
        return kernel.CompiledPlan(plan, dtype)
    finally:
        set_knobs(DEFAULT)


def tuned_sweep_seconds(plan, tuner):
    """Wall seconds of one execution of `plan` scheduled by the tuner (test and report helper)."""
    import torch
    cp = compiled(plan, tuner)
    a, b = cp.buffers()
    t0 = time.perf_counter()
    cp.execute(a, b)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    cp.free()
    return dt
