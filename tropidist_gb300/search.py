"""Completion tables of the weight-bounded search, built and probed on the GPU (drop-in for the
table part of cdist/search.py; the depth-first search itself stays with the caller).

row_hashes / column_hashes   128-bit XOR-linear syndrome hashes, seeded as cdist/search.py:83-105
Table(p, k)                  all column subsets of size <= k keyed by syndrome hash, on the device
                             (cdist/search.py:108-142; cdist/gmitm.c:61-186)
Table.lookup(...)            batched probes: least cost <= R with the same fingerprint and another
                             logical label (cdist/gmitm.c:138-163)
"""
from __future__ import annotations

import ctypes
import math
import random
import time

import numpy as np

from . import _lib, device
from .problem import Problem

DMAX = 40               # deepest threshold of the reference's search kernel (cdist/search.py:18)


def check_threshold(K):
    if K > DMAX:
        raise ValueError(f"threshold {K} exceeds the search depth {DMAX} of the kernel; nothing can be "
                         "concluded at this threshold")


def row_hashes(nrows, seed):
    """Two 64-bit random words per row from random.Random(seed) (cdist/search.py:83-85)."""
    rng = random.Random(seed)
    return ([rng.getrandbits(64) for _ in range(nrows)], [rng.getrandbits(64) for _ in range(nrows)])


def column_hashes(h, rh):
    """XOR of the row words over each column's rows: (zh, zl) uint64 arrays."""
    zh = np.zeros(len(h), dtype=np.uint64)
    zl = np.zeros(len(h), dtype=np.uint64)
    cache = {}
    for j, a in enumerate(h):
        v = cache.get(a)
        if v is None:
            x = y = 0
            m = a
            while m:
                low = m & -m
                r = low.bit_length() - 1
                x ^= rh[0][r]
                y ^= rh[1][r]
                m ^= low
            v = cache[a] = (x, y)
        zh[j], zl[j] = v
    return zh, zl


class Table:
    """All column subsets of size <= k of a problem, keyed by syndrome hash, in device memory."""

    def __init__(self, p: Problem, k, seed=12345, load=0.5, labelfree=False):
        assert labelfree or p.nobs <= 64, "more than 64 observables need a label-free table"
        device.require_gpu()
        self.problem = p
        self.k = k
        self.labelfree = labelfree
        self.wide = p.nobs > 16 and not labelfree
        self.rh = row_hashes(p.nrows, seed)
        self.zh, self.zl = column_hashes(p.h, self.rh)
        self.lg = np.zeros(p.ncols, dtype=np.uint64) if labelfree else np.array(p.l, dtype=np.uint64)
        n = p.ncols
        total = sum(math.comb(n, i) for i in range(k + 1))
        self.log2slots = max(10, math.ceil(math.log2(total / load + 1)))
        L = _lib.lib()
        st = ctypes.c_int(0)
        self.handle = L.tg_tab_create(self.log2slots, 1 if self.wide else 0, ctypes.byref(st))
        if not self.handle:
            if st.value == -3:
                raise MemoryError(f"table with 2^{self.log2slots} slots")
            _lib.check(st.value)
        t = time.time()
        _lib.check(L.tg_tab_build(self.handle, n, self.zh.ctypes.data, self.zl.ctypes.data, self.lg.ctypes.data, k))
        self.build_seconds = time.time() - t
        self.entries = int(L.tg_tab_count(self.handle))

    def hashes_for(self, h):
        """Hashes of arbitrary syndromes of this table's problem."""
        return column_hashes(h, self.rh)

    def lookup(self, zh, zl, lg, R):
        """Batched probes: per probe the least cost <= R[q] of a subset with the probe's syndrome
        hash and a logical label other than lg[q], or -1.  A label-free table stores label 0 and is
        probed with label 1, so every entry qualifies (as cdist/gmitm.c:618, 1046 do)."""
        import torch
        zh, zl = np.asarray(zh, dtype=np.uint64), np.asarray(zl, dtype=np.uint64)
        lg = np.ones(zh.size, dtype=np.uint64) if self.labelfree else np.asarray(lg, dtype=np.uint64)
        R = np.broadcast_to(np.asarray(R, dtype=np.int32), zh.shape)
        m = zh.size
        if m == 0:
            return np.zeros(0, dtype=np.int32)
        dev = [torch.from_numpy(np.ascontiguousarray(a).view(np.int64)).cuda() for a in (zh, zl, lg)]
        r = torch.from_numpy(np.array(R, dtype=np.int32)).cuda()
        out = torch.empty(m, dtype=torch.int32, device="cuda")
        _lib.check(_lib.lib().tg_tab_lookup_dev(self.handle, m, dev[0].data_ptr(), dev[1].data_ptr(),
                                                dev[2].data_ptr(), r.data_ptr(), out.data_ptr(), device.stream_ptr()))
        return out.cpu().numpy()

    def lookup_syndromes(self, syndromes, labels, R):
        """lookup() for syndromes given as row bitmasks."""
        zh, zl = self.hashes_for(list(syndromes))
        return self.lookup(zh, zl, labels, R)

    def free(self):
        if self.handle:
            _lib.lib().tg_tab_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass
