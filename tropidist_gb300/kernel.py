"""Executor of a trellis Plan on the GPU (drop-in for cdist/kernel.py).

run_plan(plan) has the signature, results and errors of cdist/kernel.py:94-138: (minimum cost, or
None if the plan is infeasible; stats), OverflowError when the cost reaches INF.  The op stream is
scheduled by libtropigpu into shared-memory sweeps (narrow tables) and fused multi-column tile
passes (wide tables) over two device buffers of 2^peak_bits entries.
"""
from __future__ import annotations

import ctypes
import time

import numpy as np

from . import _lib, device

INF = 255                 # uint8 tables (cdist/kernel.py:13)
INF16 = 65535             # uint16 tables


def final_value(entry, inf=INF):
    """Minimum cost from the last table entry of a feasible plan (cdist/kernel.py:18-25)."""
    v = int(entry)
    if v == inf:
        raise OverflowError("the distance is at least %d, beyond the %d-bit entries of the dense DP"
                            % (inf, 8 if inf == INF else 16))
    return v


def entry_bytes(dtype):
    if dtype in ("u8", "uint8", np.uint8, 1):
        return 1
    if dtype in ("u16", "uint16", np.uint16, 2):
        return 2
    raise ValueError("dtype must be uint8 or uint16")


class CompiledPlan:
    """A plan scheduled into launches by the library (reusable for repeated runs)."""

    def __init__(self, plan, dtype="u8", checkpoints=(), w_start=0, ops=None, launch=None):
        """plan: a Plan (or None with `ops`, an encoded op stream); w_start > 0: the ops follow a
        table of that width, put in buffer a (canonical order) before execute, and the plan may
        end at any width (tg_dense_plan_from).  launch=(a, b, stream): schedule and run at once,
        every segment launched as soon as it is scheduled (tg_dense_plan_execute; no checkpoints,
        the plan is not executed again)."""
        self.plan = plan
        self.eb = entry_bytes(dtype)
        self.ops = np.ascontiguousarray(plan.encode() if ops is None else ops, dtype=np.int64).reshape(-1, 3)
        self.ckpts = np.ascontiguousarray(np.array(sorted(checkpoints), dtype=np.int64))
        L = _lib.lib()
        st = ctypes.c_int(0)
        if launch is not None:
            a, b, stream = launch
            entries = min(a.numel() * a.element_size(), b.numel() * b.element_size()) // self.eb
            self.handle = L.tg_dense_plan_execute(self.ops.ctypes.data if len(self.ops) else None, len(self.ops),
                                                  self.eb, a.data_ptr(), b.data_ptr(), entries,
                                                  stream if stream is not None else device.stream_ptr(),
                                                  ctypes.byref(st))
        elif w_start or ops is not None:
            self.handle = L.tg_dense_plan_from(self.ops.ctypes.data if len(self.ops) else None, len(self.ops),
                                               self.eb, int(w_start),
                                               self.ckpts.ctypes.data if len(self.ckpts) else None,
                                               len(self.ckpts), ctypes.byref(st))
        else:
            self.handle = L.tg_dense_plan(self.ops.ctypes.data, len(self.ops), self.eb,
                                          self.ckpts.ctypes.data if len(self.ckpts) else None, len(self.ckpts),
                                          ctypes.byref(st))
        if not self.handle:
            _lib.check(st.value)
        info = np.zeros(8, dtype=np.int64)
        L.tg_dense_plan_info(self.handle, info.ctypes.data, 8)
        self.peak_bits, self.nsegs, self.npasses, self.nsweeps, self.final_buf, self.nupdates = \
            (int(x) for x in info[:6])
        self.pass_bytes, self.sweep_bytes = int(info[6]), int(info[7])

    def segments(self):
        out = np.zeros((self.nsegs, 8), dtype=np.int64)
        _lib.lib().tg_dense_plan_segments(self.handle, out.ctypes.data, self.nsegs)
        return out

    def buffers(self):
        n = (1 << self.peak_bits) * self.eb
        return device.empty(n), device.empty(n)

    def execute(self, a, b, ckpt_bufs=None, stream=None):
        arr = None
        if ckpt_bufs is not None:
            arr = (ctypes.c_void_p * len(ckpt_bufs))(*[t.data_ptr() for t in ckpt_bufs])
        _lib.check(_lib.lib().tg_dense_execute(self.handle, a.data_ptr(), b.data_ptr(), arr,
                                               stream if stream is not None else device.stream_ptr()))

    def result(self, a, b, stream=None):
        v = ctypes.c_uint32(0)
        _lib.check(_lib.lib().tg_dense_result(self.handle, a.data_ptr(), b.data_ptr(), ctypes.byref(v),
                                              stream if stream is not None else device.stream_ptr()))
        return v.value

    def free(self):
        if self.handle:
            _lib.lib().tg_dense_plan_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def run_plan(plan, log=None, progress_every=0.0, dtype="u8"):
    """Run the plan on the GPU.  Returns (min cost or None if infeasible, stats); OverflowError if
    the cost reaches INF (255 for uint8 tables, 65535 for uint16)."""
    if not plan.feasible:
        return None, {"feasible": False}
    device.require_gpu()
    t0 = time.time()
    cp = CompiledPlan(plan, dtype)
    a, b = cp.buffers()
    cp.execute(a, b)
    v = cp.result(a, b)
    stats = {"seconds": time.time() - t0, "peak_bits": plan.peak_bits, "threads": _lib.lib().dp_num_threads(),
             "passes": cp.npasses, "sweeps": cp.nsweeps}
    cp.free()
    if log:
        log("  dense DP on the GPU: %d passes, %d sweeps, %.3f s" % (stats["passes"], stats["sweeps"],
                                                                    stats["seconds"]))
    return final_value(v, INF if cp.eb == 1 else INF16), stats


def table_after(plan, nops, dtype="u8"):
    """The DP table after the first nops ops of the plan, as the raw bytes of the table in a uint8
    torch tensor on the GPU (view a copy as uint16 for 16-bit tables)."""
    device.require_gpu()
    if nops == 0:
        out = device.empty(entry_bytes(dtype))
        out.zero_()
        return out
    cp = CompiledPlan(plan, dtype, checkpoints=[nops])
    a, b = cp.buffers()
    width = _width_after(plan.ops, nops)
    out = device.empty((1 << width) * cp.eb)
    cp.execute(a, b, [out])
    cp.free()
    return out


def _width_after(ops, nops):
    w = 0
    for op in ops[:nops]:
        if op[0] == "expand":
            w += 1
        elif op[0] == "select":
            w -= 1
    return w
