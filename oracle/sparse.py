"""numpy restatement of the reference's sparse-table backend (test infrastructure only).

NumpyTables   cdist/sparse_dp.py:300-445  (sorted unique uint64 keys, uint8 values; step, join,
                                           lookup, truncate) and _prune (:448-454)
bound         cdist/sparse_dp.py:208-217
The object plugs into tropidist_gb300.sparse_dp.Sweep / query as `backend=` so that the product's
host driver can be run with reference tables and compared with the device tables cut by cut.  The
optional column weight `w` of step() restates the unit rule with `+ w` (no reference caller).
"""
from __future__ import annotations

import numpy as np

U64 = np.uint64
INF = 255
Q = 720720


def bound(keys, tmask, hd):
    masks, weights, extra = hd
    if not len(masks):
        return np.full(keys.shape, (extra + Q - 1) // Q, dtype=np.int64)
    u = keys ^ U64(tmask)
    tot = np.full(keys.shape, extra, dtype=np.int64)
    for m, w in zip(masks, weights):
        tot += np.int64(w) * np.bitwise_count(u & U64(m)).astype(np.int64)
    return (tot + (Q - 1)) // Q


def _prune(keys, vals, cap, K, tmask, hd):
    ok = vals <= cap
    if hd is not None and keys.size:
        ok &= vals.astype(np.int64) + bound(keys, tmask, hd) <= K
    if ok.all():
        return keys, vals, None
    return keys[ok], vals[ok], ok


class NumpyTables:
    """Sparse tables as (keys, vals): keys sorted and unique (uint64), vals uint8."""
    name = "numpy"

    def __init__(self, tr=None):
        self.tr = tr

    @staticmethod
    def start():
        return np.zeros(1, dtype=U64), np.zeros(1, dtype=np.uint8)

    @staticmethod
    def size(tab):
        return tab[0].size

    @staticmethod
    def nbytes(tab):
        return tab[0].nbytes + tab[1].nbytes

    @staticmethod
    def arrays(tab):
        return tab

    @staticmethod
    def from_arrays(keys, vals):
        o = np.argsort(keys)
        return np.asarray(keys, dtype=U64)[o], np.asarray(vals, dtype=np.uint8)[o]

    @staticmethod
    def lookup(tab, s):
        keys, vals = tab
        i = int(np.searchsorted(keys, U64(s)))
        if i < keys.size and int(keys[i]) == s:
            return int(vals[i])
        return INF

    @staticmethod
    def changed_size(ch):
        return ch[0].size

    @staticmethod
    def persistent(tab):
        return tab

    @staticmethod
    def truncate(tab, below):
        keys, vals = tab
        ok = vals < below
        return keys[ok], vals[ok]

    def hist(self, tab):
        return np.bincount(tab[1], minlength=256)

    def step(self, tab, upd, sel_mask, sel_bits, cap, K, tmask, hd, keep_below=None, want_changed=False, w=1):
        keys, vals = tab
        n = keys.size
        improved = None
        if upd and n:
            src = vals < cap
            tk = keys[src] ^ U64(upd)
            tv = (vals[src].astype(np.int64) + w)
            idx = np.searchsorted(keys, tk)
            idx[idx == n] = n - 1
            hit = keys[idx] == tk
            imp = hit & (tv < vals[idx])
            if imp.any():
                vals = vals.copy()
                vals[idx[imp]] = tv[imp]
                if want_changed:
                    improved = np.zeros(n, dtype=bool)
                    improved[idx[imp]] = True
            miss = ~hit
            nk, nv = tk[miss], np.minimum(tv[miss], INF).astype(np.uint8)
        else:
            nk = np.empty(0, dtype=U64)
            nv = np.empty(0, dtype=np.uint8)
        if sel_mask:
            sm, sb = U64(sel_mask), U64(sel_bits)
            ok = (keys & sm) == sb
            keys, vals = keys[ok], vals[ok]
            if improved is not None:
                improved = improved[ok]
            ok = (nk & sm) == sb
            nk, nv = nk[ok], nv[ok]
            if sel_bits:
                keys = keys & ~sm
                nk = nk & ~sm
        keys, vals, ok = _prune(keys, vals, cap, K, tmask, hd)
        if ok is not None and improved is not None:
            improved = improved[ok]
        nk, nv, _ = _prune(nk, nv, cap, K, tmask, hd)
        changed = None
        if want_changed:
            if improved is not None and improved.any():
                ck = np.concatenate([keys[improved], nk])
                cv = np.concatenate([vals[improved], nv])
            else:
                ck, cv = nk, nv
            o = np.argsort(ck)
            changed = (ck[o], cv[o])
        if keep_below is not None and nk.size:
            ok = nv < keep_below
            nk, nv = nk[ok], nv[ok]
        if nk.size:
            o = np.argsort(nk)
            nk, nv = nk[o], nv[o]
            pos = np.searchsorted(keys, nk)
            keys = np.insert(keys, pos, nk)
            vals = np.insert(vals, pos, nv)
        return (keys, vals), changed

    @staticmethod
    def join(ch, btab, tmask):
        ck, cv = ch
        if not ck.size:
            return None
        q = ck ^ U64(tmask)
        bkeys, bvals = btab
        if not bkeys.size:
            return None
        idx = np.searchsorted(bkeys, q)
        idx[idx == bkeys.size] = bkeys.size - 1
        hit = bkeys[idx] == q
        if not hit.any():
            return None
        tot = cv[hit].astype(np.int64) + bvals[idx[hit]].astype(np.int64)
        i = int(np.argmin(tot))
        fi = int(np.flatnonzero(hit)[i])
        return int(tot[i]), int(ck[fi]), int(cv[fi]), int(q[fi])


# ---------------------------------------------------------------------- the C port as a backend
_PORT = None


def port_lib():
    """oracle/sparse_port.so (built by oracle/Makefile), with its signatures declared."""
    global _PORT
    if _PORT is None:
        import ctypes
        import os
        import subprocess
        here = os.path.dirname(os.path.abspath(__file__))
        so = os.path.join(here, "sparse_port.so")
        if not os.path.exists(so) or os.path.getmtime(so) < os.path.getmtime(os.path.join(here, "sparse_port.c")):
            subprocess.run(["make", "-s", "-C", here], check=True)
        L = ctypes.CDLL(so)
        vp, i64, u64, ci = ctypes.c_void_p, ctypes.c_int64, ctypes.c_uint64, ctypes.c_int
        L.spp_candidates.argtypes = [vp, i64, u64, ci, u64, u64, ci, ci, vp, vp, i64, u64, ci, ci, vp, vp]
        L.spp_candidates.restype = i64
        L.spp_merge.argtypes = [vp, i64, vp, i64, u64, u64, ci, ci, ci, vp, vp, i64, u64, ci, ci, vp, vp,
                                ctypes.POINTER(i64)]
        L.spp_merge.restype = i64
        L.spp_join.argtypes = [vp, i64, vp, i64, u64, ctypes.POINTER(u64), ctypes.POINTER(u64)]
        L.spp_join.restype = ci
        L.spp_hist.argtypes = [vp, i64, vp]
        _PORT = L
    return _PORT


class CPortTables:
    """The reference's C table backend (cdist/sparse_dp.py:506-605 over cdist/sparse_dp.c) restated
    over oracle/sparse_port.c: a table is one sorted array of packed states key | value << 56.
    step() returns arrays of two alternating buffers, so the table it returns is valid until the step
    after next; persistent() copies.  One object per sweep."""
    name = "c-port"
    KEYMASK = (1 << 56) - 1

    def __init__(self, tr=None):
        if tr is not None and tr.nslots > 56:
            raise ValueError("the C tables hold at most 56 row slots (this trellis needs %d)" % tr.nslots)
        self.tr = tr
        self.L = port_lib()
        self.bufs = {}
        self.flip = 0

    def _buf(self, name, n):
        b = self.bufs.get(name)
        if b is None or b.size < n:
            grow = int(1.25 * b.size) if b is not None else 0
            b = self.bufs[name] = np.empty(max(n, grow, 1024), dtype=U64)
        return b

    @staticmethod
    def start():
        return np.zeros(1, dtype=U64)

    @staticmethod
    def size(tab):
        return tab.size

    @staticmethod
    def nbytes(tab):
        return tab.nbytes

    @staticmethod
    def persistent(tab):
        return tab.copy()

    @staticmethod
    def truncate(tab, below):
        return tab[(tab >> U64(56)) < U64(below)]

    @classmethod
    def arrays(cls, tab):
        return tab & U64(cls.KEYMASK), (tab >> U64(56)).astype(np.uint8)

    @classmethod
    def from_arrays(cls, keys, vals):
        o = np.argsort(keys)
        return (np.asarray(keys, dtype=U64)[o] & U64(cls.KEYMASK)) | (np.asarray(vals).astype(U64)[o] << U64(56))

    @classmethod
    def lookup(cls, tab, s):
        keys = tab & U64(cls.KEYMASK)
        i = int(np.searchsorted(keys, U64(s)))
        if i < keys.size and int(keys[i]) == s:
            return int(tab[i] >> U64(56))
        return INF

    @staticmethod
    def changed_size(ch):
        return ch.size

    def hist(self, tab):
        h = np.zeros(256, dtype=np.int64)
        self.L.spp_hist(tab.ctypes.data, tab.size, h.ctypes.data)
        return h

    def step(self, tab, upd, sel_mask, sel_bits, cap, K, tmask, hd, keep_below=None, want_changed=False, w=1):
        import ctypes
        n = tab.size
        if hd is None:
            ncls, mp, wp, extra, use_h = 0, None, None, 0, 0
        else:
            m_arr = np.ascontiguousarray(hd[0], dtype=U64)
            w_arr = np.ascontiguousarray(hd[1], dtype=np.int64)
            extra = int(hd[2])
            ncls, use_h = m_arr.size, 1
            mp = m_arr.ctypes.data if ncls else None
            wp = w_arr.ctypes.data if ncls else None
        cand, tmp = self._buf("cand", n), self._buf("tmp", n)
        m = self.L.spp_candidates(tab.ctypes.data, n, int(upd), int(w), int(sel_mask), int(sel_bits), int(cap),
                                  ncls, mp, wp, extra, int(tmask), int(K), use_h, cand.ctypes.data, tmp.ctypes.data)
        self.flip ^= 1
        out = self._buf("out%d" % self.flip, n + m)
        ch = self._buf("changed", m) if want_changed else None
        nch = ctypes.c_int64(0)
        no = self.L.spp_merge(tab.ctypes.data, n, cand.ctypes.data, m, int(sel_mask), int(sel_bits), int(cap),
                              int(keep_below or 0), ncls, mp, wp, extra, int(tmask), int(K), use_h, out.ctypes.data,
                              ch.ctypes.data if ch is not None else None, ctypes.byref(nch))
        return out[:no], (ch[:nch.value] if want_changed else None)

    def join(self, ch, btab, tmask):
        import ctypes
        if not ch.size or not btab.size:
            return None
        fb, bb = ctypes.c_uint64(0), ctypes.c_uint64(0)
        tot = self.L.spp_join(ch.ctypes.data, ch.size, btab.ctypes.data, btab.size, int(tmask), ctypes.byref(fb),
                              ctypes.byref(bb))
        if tot < 0:
            return None
        return int(tot), fb.value & self.KEYMASK, fb.value >> 56, bb.value & self.KEYMASK
