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
