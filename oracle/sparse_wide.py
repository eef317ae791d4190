"""numpy restatement of the reference's sparse-table backend for states wider than 64 row slots:
TEST INFRASTRUCTURE ONLY.

The reference keeps a state in one machine word (at most 64 slots in numpy, 56 in C,
cdist/sparse_dp.py:97-98) and refuses wider trellises.  This module restates its table rules
(NumpyTables.step / join / lookup / truncate and _prune, cdist/sparse_dp.py:300-455) for keys of
W 64-bit words: a table is (keys uint64 [n, W], vals uint8 [n]) with distinct keys in one fixed
total order (the bytes of the key).  The column weight `w` restates the unit rule with `+ w`.
Masks and states cross the interface as Python ints; lookahead masks as uint64 [k, W] arrays.
On states of at most 64 slots it gives the same tables as oracle/sparse.NumpyTables (tested).
"""
from __future__ import annotations

import numpy as np

U64 = np.uint64
INF = 255
Q = 720720
M64 = (1 << 64) - 1


def words_of(x, W):
    """A Python int as uint64 [W] (little-endian words)."""
    x = int(x)
    return np.array([(x >> (64 * i)) & M64 for i in range(W)], dtype=U64)


def int_of(row):
    out = 0
    for i, w in enumerate(np.asarray(row, dtype=U64).tolist()):
        out |= int(w) << (64 * i)
    return out


def _void(keys):
    keys = np.ascontiguousarray(keys)
    return keys.view(np.dtype((np.void, keys.shape[1] * 8))).ravel()


def _sorted(keys, vals):
    if not len(vals):
        return keys, vals
    o = np.argsort(_void(keys), kind="stable")
    return keys[o], vals[o]


def popcount_rows(x):
    return np.bitwise_count(x).astype(np.int64).sum(axis=-1)


def bound(keys, tmask_w, hd):
    """ceil((extra + sum_c w_c |(key ^ tmask) & mask_c|) / Q) per key (cdist/sparse_dp.py:208-217)."""
    masks, weights, extra = hd
    tot = np.full(len(keys), int(extra), dtype=np.int64)
    if len(weights):
        u = keys ^ tmask_w[None, :]
        for m, w in zip(np.asarray(masks, dtype=U64).reshape(len(weights), -1), weights):
            tot += np.int64(w) * popcount_rows(u & m[None, :])
    return (tot + (Q - 1)) // Q


class WideTables:
    """Sparse tables of W-word states (see the module docstring)."""
    name = "numpy-wide"

    def __init__(self, tr=None, words=None):
        self.W = words if words is not None else max(1, (getattr(tr, "nslots", 1) + 63) // 64)

    def start(self):
        return np.zeros((1, self.W), dtype=U64), np.zeros(1, dtype=np.uint8)

    @staticmethod
    def size(tab):
        return len(tab[1])

    @staticmethod
    def nbytes(tab):
        return tab[0].nbytes + tab[1].nbytes

    @staticmethod
    def persistent(tab):
        return tab

    @staticmethod
    def changed_size(ch):
        return len(ch[1])

    @staticmethod
    def truncate(tab, below):
        ok = tab[1] < below
        return tab[0][ok], tab[1][ok]

    def arrays(self, tab):
        """(keys as Python ints, vals) in increasing key order."""
        keys = [int_of(r) for r in tab[0]]
        o = sorted(range(len(keys)), key=keys.__getitem__)
        return [keys[i] for i in o], tab[1][o] if len(o) else tab[1]

    def from_arrays(self, keys, vals):
        k = np.stack([words_of(x, self.W) for x in keys]) if len(keys) else np.zeros((0, self.W), dtype=U64)
        return _sorted(k, np.asarray(vals, dtype=np.uint8))

    def lookup(self, tab, s):
        keys, vals = tab
        if not len(vals):
            return INF
        q = _void(words_of(s, self.W)[None, :])
        v = _void(keys)
        i = int(np.searchsorted(v, q[0]))
        if i < len(v) and v[i] == q[0]:
            return int(vals[i])
        return INF

    def hist(self, tab):
        return np.bincount(tab[1], minlength=256)

    def _prune(self, keys, vals, cap, K, tmask, hd):
        ok = vals <= cap
        if hd is not None and len(vals):
            ok &= vals.astype(np.int64) + bound(keys, words_of(tmask, self.W), hd) <= K
        return ok

    def step(self, tab, upd, sel_mask, sel_bits, cap, K, tmask, hd, keep_below=None, want_changed=False, w=1):
        """T'[s] = min(T[s], T[s ^ upd] + w); the closing rows (sel_mask) must equal sel_bits and are
        cleared; values above cap and states failing the lookahead dropped; returns (table, changed)
        with changed = the new or improved states (cdist/sparse_dp.py:338-403)."""
        keys, vals = tab
        W = self.W
        um, sm, sb = words_of(upd, W), words_of(sel_mask, W), words_of(sel_bits, W)
        # candidates
        if upd and len(vals):
            src = vals < cap
            ck = keys[src] ^ um[None, :]
            cv = vals[src].astype(np.int64) + w
        else:
            ck, cv = np.zeros((0, W), dtype=U64), np.zeros(0, dtype=np.int64)
        # closing rows: filter and clear, on both the old states and the candidates
        if sel_mask:
            ok = np.all((keys & sm[None, :]) == sb[None, :], axis=1)
            keys, vals = keys[ok] & ~sm[None, :], vals[ok]
            ok = np.all((ck & sm[None, :]) == sb[None, :], axis=1)
            ck, cv = ck[ok] & ~sm[None, :], cv[ok]
        ok = self._prune(keys, vals.astype(np.int64), cap, K, tmask, hd)
        keys, vals = keys[ok], vals[ok].astype(np.int64)
        ok = self._prune(ck, cv, cap, K, tmask, hd)
        ck, cv = ck[ok], cv[ok]
        # per key the least candidate value
        if len(cv):
            o = np.lexsort((cv, _void(ck)))
            ck, cv = ck[o], cv[o]
            first = np.ones(len(cv), dtype=bool)
            vk = _void(ck)
            first[1:] = vk[1:] != vk[:-1]
            ck, cv = ck[first], cv[first]
        # against the old states: new keys, improvements
        vo = _void(keys)
        vc = _void(ck)
        pos = np.searchsorted(vo, vc) if len(vo) else np.zeros(len(vc), dtype=np.int64)
        posc = np.minimum(pos, max(len(vo) - 1, 0))
        hit = (vo[posc] == vc) if len(vo) else np.zeros(len(vc), dtype=bool)
        better = np.ones(len(cv), dtype=bool)
        better[hit] = cv[hit] < vals[posc[hit]]
        changed = None
        if want_changed:
            changed = _sorted(ck[better], np.minimum(cv[better], INF).astype(np.uint8))
        imp = hit & better
        vals = vals.copy()
        vals[posc[imp]] = cv[imp]
        nk, nv = ck[~hit], cv[~hit]
        if keep_below is not None:
            ok = nv < keep_below
            nk, nv = nk[ok], nv[ok]
        keys = np.concatenate([keys, nk])
        vals = np.concatenate([vals, nv])
        return _sorted(keys, np.minimum(vals, INF).astype(np.uint8)), changed

    def join(self, ch, btab, tmask):
        """min over changed f and backward b with key(b) = key(f) ^ tmask of f.val + b.val:
        (total, forward key, forward value, backward key) or None."""
        ck, cv = ch
        bk, bv = btab
        if not len(cv) or not len(bv):
            return None
        q = ck ^ words_of(tmask, self.W)[None, :]
        vb, vq = _void(bk), _void(q)
        pos = np.minimum(np.searchsorted(vb, vq), len(vb) - 1)
        hit = vb[pos] == vq
        if not hit.any():
            return None
        tot = cv[hit].astype(np.int64) + bv[pos[hit]].astype(np.int64)
        i = int(np.argmin(tot))
        fi = int(np.flatnonzero(hit)[i])
        return int(tot[i]), int_of(ck[fi]), int(cv[fi]), int_of(q[fi])
