"""Build and load libtropigpu.so, the CUDA library behind every evaluator of this package.

build() compiles tropidist_gb300/csrc/*.cu for sm_103a with nvcc (one object per translation
unit, compiled in parallel, then linked into tropidist_gb300/libtropigpu.so).  lib() loads it
with ctypes and declares the C-ABI of include/tropidist_gb300.h.  There is no fallback: if the
library cannot be built or loaded, the evaluators raise.
"""
from __future__ import annotations

import concurrent.futures
import ctypes
import glob
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
SO = os.path.join(HERE, "libtropigpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
              "-I" + os.path.join(ROOT, "include")]

_LIB = None


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False):
    """Compile every CUDA source for sm_103a and link libtropigpu.so; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    headers = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        glob.glob(os.path.join(ROOT, "include", "*.h"))
    objs, jobs = [], []
    for src in sources():
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append([_nvcc()] + ARCH + NVCC_FLAGS + ["-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
        if verbose and r.stderr:
            print(r.stderr)
        return r

    if jobs:
        with concurrent.futures.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            list(ex.map(run, jobs))
    if force or jobs or _stale(SO, objs):
        run([_nvcc()] + ARCH + ["-shared", "-o", SO] + objs + ["-lcudart", "-lpthread"])
    return SO


def _declare(L):
    c = ctypes
    vp, u64, i64, ci, u8 = c.c_void_p, c.c_uint64, c.c_int64, c.c_int, c.c_uint8
    sig = {
        "tg_version": (ci, []),
        "tg_last_error": (c.c_char_p, []),
        "tg_sm_count": (ci, []),
        "tg_set_stream": (None, [vp]),
        "dp_update": (None, [vp, u64, u64]),
        "dp_update_w": (None, [vp, u64, u64, ci]),
        "dp_expand_update": (None, [vp, u64, u64]),
        "dp_select": (u64, [vp, u64, ci, ci]),
        "dp_fill": (None, [vp, u64, u8]),
        "dp_hist": (None, [vp, u64, vp]),
        "dp_num_threads": (ci, []),
        "dp16_update": (ci, [vp, u64, u64, ci]),
        "dp16_expand_update": (ci, [vp, u64, u64, ci]),
        "dp16_select": (u64, [vp, u64, ci, ci]),
        "tg_dense_plan": (vp, [vp, i64, ci, vp, i64, c.POINTER(ci)]),
        "tg_dense_plan_from": (vp, [vp, i64, ci, ci, vp, i64, c.POINTER(ci)]),
        "tg_dense_plan_info": (ci, [vp, vp, ci]),
        "tg_dense_plan_segments": (ci, [vp, vp, i64]),
        "tg_dense_plan_free": (None, [vp]),
        "tg_dense_execute": (ci, [vp, vp, vp, vp, vp]),
        "tg_dense_result": (ci, [vp, vp, vp, c.POINTER(c.c_uint32), vp]),
        "tg_dense_execute_timed": (ci, [vp, vp, vp, vp, vp, ci]),
        "tg_dense_segment_ms": (ci, [vp, vp, i64]),
        "tg_dense_run_noalloc": (ci, [vp, i64, vp, u64, c.POINTER(c.c_uint32), vp]),
        "tg_dense_run": (ci, [vp, i64, ci, vp, vp, c.POINTER(c.c_uint32), vp]),
        "tg_dense_set_tuning": (ci, [ci, ci, ci, ci]),
        "tg_dense_set_stream_span": (ci, [ci, ci]),
        "tg_debug_emulate_dense": (ci, [vp, vp, vp, vp]),
    }
    from . import _sigs_extra
    sig.update(_sigs_extra.SIGNATURES)
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    return L


def lib():
    """The loaded library (built first if needed).  Raises if it cannot be built or loaded."""
    global _LIB
    if _LIB is None:
        path = SO
        if not os.path.exists(path) or _stale(path, sources()):
            build()
        _LIB = _declare(ctypes.CDLL(path))
    return _LIB


class TGError(RuntimeError):
    """A failure reported by libtropigpu (status code and message)."""

    def __init__(self, status, msg):
        super().__init__("libtropigpu status %d: %s" % (status, msg))
        self.status = status


def check(status):
    if status != 0:
        msg = lib().tg_last_error()
        msg = msg.decode() if msg else ""
        if status == -3:
            raise MemoryError("libtropigpu: " + msg)
        if status == -5:
            raise TimeoutError("libtropigpu: " + msg)
        raise TGError(status, msg)
    return status
