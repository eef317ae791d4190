"""Batched exact distances: many instances' logical queries in one persistent GPU launch.

DenseBatch(plans)            schedules every feasible plan (libtropigpu tg_batch_create) and keeps a
                             device arena with two tables per plan
DenseBatch.run()             one launch of the persistent kernel; the final entry of every plan
batched_dp_distances(ps)     dp_distance over many problems at once: [(best, per_obs), ...]
The plans run in a device work queue (csrc/batch.cu): narrow plans are whole jobs of one block in
shared memory, wide plans a job per fused pass with one unit per tile.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib, auto, device, kernel


class DenseBatch:
    def __init__(self, plans):
        device.require_gpu()
        self.plans = list(plans)
        self.index = [i for i, pl in enumerate(self.plans) if pl.feasible]
        encs = [pl.encode() for i, pl in enumerate(self.plans) if pl.feasible]
        self.handle = None
        if not encs:
            return
        offs = np.zeros(len(encs) + 1, dtype=np.int64)
        for i, e in enumerate(encs):
            offs[i + 1] = offs[i] + len(e)
        self.ops = np.ascontiguousarray(np.concatenate(encs) if offs[-1] else np.zeros((1, 3), dtype=np.int64))
        self.offs = offs
        st = ctypes.c_int(0)
        self.handle = _lib.lib().tg_batch_create(len(encs), self.ops.ctypes.data, offs.ctypes.data, ctypes.byref(st))
        if not self.handle:
            _lib.check(st.value)
        info = np.zeros(4, dtype=np.int64)
        _lib.lib().tg_batch_info(self.handle, info.ctypes.data, 4)
        self.arena_bytes, self.njobs, self.units, self.nplans = (int(x) for x in info)
        self.arena = device.empty(max(1, self.arena_bytes))

    def run(self, blocks=0, window=None):
        """Final entries of every plan (None for an infeasible plan; INF = 255 is returned as is).
        window: plans in progress at once (default: the autotuned window of the widest plan)."""
        out = [None] * len(self.plans)
        if self.handle is None:
            return out
        vals = np.zeros(len(self.index), dtype=np.uint32)
        if window is None:
            window = self.default_window()
        _lib.check(_lib.lib().tg_batch_run(self.handle, self.arena.data_ptr(), int(blocks), int(window),
                                           vals.ctypes.data, device.stream_ptr()))
        for k, i in enumerate(self.index):
            out[i] = int(vals[k])
        return out

    def default_window(self):
        """Plans in progress at once: all of them (measured best on the uneven-width batches; a
        small window serialises the wide plans, whose passes then run on few blocks)."""
        return 0

    def free(self):
        if self.handle:
            _lib.lib().tg_batch_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def batched_dp_distances(problems, orders=None):
    """[(best, per_obs)] for every problem, as auto.dp_distance gives one by one; OverflowError if a
    distance reaches 255."""
    plans, owner = [], []
    for k, p in enumerate(problems):
        order = list(range(p.ncols)) if orders is None else orders[k]
        for i, plan in auto._plans(p, order):
            plans.append(plan)
            owner.append((k, i))
    vals = DenseBatch(plans).run() if plans else []
    out = [[None, [None] * p.nobs] for p in problems]
    for (k, i), v in zip(owner, vals):
        if v is None:
            continue
        v = kernel.final_value(v)
        out[k][1][i] = v
        if out[k][0] is None or v < out[k][0]:
            out[k][0] = v
    return [tuple(x) for x in out]
