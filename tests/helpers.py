"""Shared helpers of the test-suite: golden fixtures, problems from fixtures, the C port."""
from __future__ import annotations

import ctypes
import functools
import hashlib
import json
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")


@functools.lru_cache(maxsize=None)
def golden(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


def unhex(xs):
    return [int(x, 16) for x in xs]


def sha(arr):
    return hashlib.sha256(np.ascontiguousarray(arr).tobytes()).hexdigest()[:16]


def ops_from_json(ops):
    return [tuple(o) for o in ops]


@functools.lru_cache(maxsize=None)
def port():
    """The C/OpenMP port of the reference's dense kernels (oracle/dense_port.c)."""
    so = os.path.join(ROOT, "oracle", "dense_port.so")
    src = os.path.join(ROOT, "oracle", "dense_port.c")
    if not os.path.exists(so) or os.path.getmtime(so) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    L = ctypes.CDLL(so)
    vp, u64, i64 = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int64
    L.port_run_plan.argtypes = [vp, i64, vp, u64]
    L.port_run_plan.restype = u64
    L.port_update.argtypes = [vp, u64, u64]
    L.port_num_threads.restype = ctypes.c_int
    return L


def port_run(plan, upto=None):
    """Run the plan's ops (or the first `upto`) with the C port; returns the final table."""
    from tropidist_gb300 import trellis
    ops = trellis.encode_ops(plan.ops[:upto] if upto is not None else plan.ops)
    buf = np.zeros(1 << max(plan.peak_bits, 0), dtype=np.uint8)
    n = port().port_run_plan(ops.ctypes.data, len(ops), buf.ctypes.data, 1)
    return buf[:n].copy()


def emulate(plan, dtype="u8", checkpoints=()):
    """Scheduled launches of the plan run by the library's host emulation: (final value, tables)."""
    from tropidist_gb300 import _lib
    from tropidist_gb300.kernel import CompiledPlan, _width_after
    cp = CompiledPlan(plan, dtype, checkpoints)
    dt = np.uint8 if cp.eb == 1 else np.uint16
    a = np.zeros(1 << cp.peak_bits, dtype=dt)
    b = np.zeros(1 << cp.peak_bits, dtype=dt)
    tabs = [np.zeros(1 << _width_after(plan.ops, k), dtype=dt) for k in cp.ckpts]
    arr = (ctypes.c_void_p * max(1, len(tabs)))(*[t.ctypes.data for t in tabs])
    _lib.check(_lib.lib().tg_debug_emulate_dense(cp.handle, a.ctypes.data, b.ctypes.data, arr))
    v = int((b if cp.final_buf else a)[0])
    info = (cp.npasses, cp.nsweeps)
    cp.free()
    return v, tabs, info
