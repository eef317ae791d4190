"""Device backends of the sparse Rank DP: tables of states on the GPU.

GpuTables       states of at most 56 row slots packed like the reference's C tables
                (key | value << 56, cdist/sparse_dp.c:3-4): a device array plus an open-addressing
                device index; a column step, the meet-in-the-middle join, lookups, and runs of
                steps in one library call (walk); csrc/sparse.cu
WideGpuTables   states of up to 512 row slots as W uint64 words (word-major key arrays, uint8
                values, an index keyed by a hash of the words); csrc/sparse_wide.cu.  The
                reference refuses trellises of more than 64 slots (cdist/sparse_dp.py:97-98).
Both implement the table-backend interface of cdist/sparse_dp.py:300-445 (start, size, nbytes,
arrays, from_arrays, lookup, step, changed_size, persistent, truncate, join, name); states and masks
cross it as Python ints.
"""
from __future__ import annotations

import numpy as np

from . import _lib, device

INF = 255
U64 = np.uint64
KEYMASK = (1 << 56) - 1
MAX_SLOTS = 56                  # row slots of a packed device state
MAX_WIDE_SLOTS = 512            # 8 words


class BudgetExceeded(RuntimeError):
    """A table outgrew max_states (kind "states") or a sweep passed its deadline (kind "deadline")."""

    def __init__(self, message, kind):
        super().__init__(message)
        self.kind = kind


class _Tab:
    """A device table: `arr` holds its n packed states (int64 tensor), `H` its index (2^lg slots)."""
    __slots__ = ("arr", "n", "H", "lg")

    def __init__(self, arr, n, H, lg):
        self.arr, self.n, self.H, self.lg = arr, n, H, lg

    def hptr(self):
        return self.H.data_ptr()


class _ArenaTab:
    """A table kept by a device walk inside the walk's arena (states at int64 offset a0, index at h0);
    the tensor views are made only when asked for."""
    __slots__ = ("arena", "a0", "n", "h0", "lg")

    def __init__(self, arena, a0, n, h0, lg):
        self.arena, self.a0, self.n, self.h0, self.lg = arena, a0, n, h0, lg

    @property
    def arr(self):
        return self.arena[self.a0:self.a0 + self.n]

    @property
    def H(self):
        return self.arena[self.h0:self.h0 + (1 << self.lg)]

    def hptr(self):
        return self.arena.data_ptr() + 8 * self.h0


class _Changed:
    __slots__ = ("arr", "n")

    def __init__(self, arr, n):
        self.arr, self.n = arr, n


def _lg_for(n_states):
    """Index size for up to n_states states at load <= 1/2."""
    return max(6, int(2 * max(1, n_states) - 1).bit_length() + 1)


class GpuTables:
    """Sparse tables on the GPU (packed states + device index).  Tables are immutable: a step returns
    new device buffers, so every table a sweep keeps stays valid."""
    name = "gpu"

    def __init__(self, tr):
        device.require_gpu()
        if tr.nslots > MAX_SLOTS:
            raise ValueError("the device tables hold at most %d row slots (this trellis needs %d)"
                             % (MAX_SLOTS, tr.nslots))
        self.tr = tr
        self.L = _lib.lib()
        import torch
        self.torch = torch
        self.counters = torch.zeros(4, dtype=torch.int64, device="cuda")
        self.host = torch.zeros(4, dtype=torch.int64).pin_memory()
        self.result = torch.zeros(1, dtype=torch.int64, device="cuda")

    # ------------------------------------------------------------------ helpers
    def _empty(self, n):
        return self.torch.empty(max(1, int(n)), dtype=self.torch.int64, device="cuda")

    def _read_counters(self):
        self.host.copy_(self.counters)
        self.torch.cuda.current_stream().synchronize()
        c = [int(x) for x in self.host.tolist()]
        if c[2]:
            raise RuntimeError("device table overflow (flags %d)" % c[2])
        return c

    def _build(self, arr, n, below=-1):
        lg = _lg_for(n)
        H = self._empty(1 << lg)
        kept = self._empty(n) if below >= 0 else None
        _lib.check(self.L.tg_sp_build(arr.data_ptr() if n else None, n, H.data_ptr(), lg, below,
                                      kept.data_ptr() if kept is not None else None, self.counters.data_ptr(),
                                      device.stream_ptr()))
        if below >= 0:
            m = self._read_counters()[3]
            return _Tab(kept[:m], m, H, lg)
        return _Tab(arr[:n], n, H, lg)

    # ------------------------------------------------------------------ backend interface
    def start(self):
        arr = self.torch.zeros(1, dtype=self.torch.int64, device="cuda")
        return self._build(arr, 1)

    state_bytes = 8

    @staticmethod
    def size(tab):
        return tab.n

    @staticmethod
    def nbytes(tab):
        return 8 * tab.n

    @staticmethod
    def changed_size(ch):
        return ch.n

    @staticmethod
    def persistent(tab):
        return tab

    def arrays(self, tab):
        """(keys uint64, vals uint8) of a table, sorted by key (host copies)."""
        if tab.n == 0:
            return np.zeros(0, dtype=U64), np.zeros(0, dtype=np.uint8)
        x = tab.arr[:tab.n].cpu().numpy().view(U64)
        keys = x & U64(KEYMASK)
        o = np.argsort(keys, kind="stable")
        return keys[o], (x[o] >> U64(56)).astype(np.uint8)

    def from_arrays(self, keys, vals):
        packed = (np.asarray(keys, dtype=U64) & U64(KEYMASK)) | (np.asarray(vals).astype(U64) << U64(56))
        arr = self.torch.from_numpy(packed.view(np.int64).copy()).cuda() if packed.size else self._empty(1)
        return self._build(arr, int(packed.size))

    def lookup(self, tab, s):
        if int(s) >> 56 or tab.n == 0:
            return INF
        keys = self.torch.tensor([int(s)], dtype=self.torch.int64).cuda()
        vals = self.torch.empty(1, dtype=self.torch.uint8, device="cuda")
        _lib.check(self.L.tg_sp_lookup(tab.H.data_ptr(), tab.lg, keys.data_ptr(), 1, vals.data_ptr(),
                                       device.stream_ptr()))
        return int(vals.item())

    def lookup_many(self, tab, keys):
        keys = np.asarray(keys, dtype=U64)
        if not keys.size:
            return np.zeros(0, dtype=np.uint8)
        kt = self.torch.from_numpy(keys.view(np.int64).copy()).cuda()
        vals = self.torch.empty(keys.size, dtype=self.torch.uint8, device="cuda")
        _lib.check(self.L.tg_sp_lookup(tab.H.data_ptr(), tab.lg, kt.data_ptr(), keys.size, vals.data_ptr(),
                                       device.stream_ptr()))
        return vals.cpu().numpy()

    def truncate(self, tab, below):
        return self._build(tab.arr, tab.n, below=int(below))

    def step(self, tab, upd, sel_mask, sel_bits, cap, K, tmask, hd, keep_below=None, want_changed=False, w=1):
        """One column (as cdist/sparse_dp.py:338-403): T'[s] = min(T[s], T[s ^ upd] + w), then the
        closing rows' filter and clear, values above cap and states failing the lookahead (hd)
        dropped; returns (table, changed).  New states with value >= keep_below go to changed only."""
        n = tab.n
        lg = _lg_for(2 * n)
        H = self._empty(1 << lg)
        A = self._empty(2 * n)
        ch = self._empty(n) if want_changed else None
        if hd is None:
            ncls, mp, wp, extra, use_h = 0, None, None, 0, 0
        else:
            m_arr, w_arr, extra = hd
            m_arr = np.ascontiguousarray(m_arr, dtype=U64)
            w_arr = np.ascontiguousarray(w_arr, dtype=np.int64)
            ncls, mp, wp, use_h = len(m_arr), m_arr.ctypes.data, w_arr.ctypes.data, 1
        _lib.check(self.L.tg_sp_step(tab.arr.data_ptr(), n, tab.H.data_ptr(), tab.lg, H.data_ptr(), lg, A.data_ptr(),
                                     2 * n, ch.data_ptr() if ch is not None else None, n, int(upd) & KEYMASK,
                                     int(sel_mask), int(sel_bits), int(cap),
                                     -1 if keep_below is None else int(keep_below), int(w), int(bool(want_changed)),
                                     use_h, int(K), ncls, mp, wp, int(extra), int(tmask), self.counters.data_ptr(),
                                     device.stream_ptr()))
        c = self._read_counters()
        new = _Tab(A[:c[3]], c[3], H, lg)
        changed = _Changed(ch[:c[1]], c[1]) if want_changed else None
        return new, changed

    def join(self, ch, btab, tmask):
        """Least f.value + b.value over changed forward states f and backward states b with
        key(b) = key(f) ^ tmask: (total, forward key, forward value, backward key), or None."""
        if ch is None or not ch.n or not btab.n:
            return None
        _lib.check(self.L.tg_sp_join(ch.arr.data_ptr(), ch.n, btab.H.data_ptr(), btab.lg, int(tmask),
                                     self.result.data_ptr(), device.stream_ptr()))
        r = int(self.result.item()) & 0xFFFFFFFFFFFFFFFF
        if r == 0xFFFFFFFFFFFFFFFF:
            return None
        total, fkey = r >> 56, r & KEYMASK
        bkey = fkey ^ int(tmask)
        bval = self.lookup(btab, bkey)
        return total, fkey, total - bval, bkey

    def walk(self, tab, rows, masks, weights, K, max_states=None, want_res=True):
        """Run the column steps of `rows` (int64 [m, 16] spec rows, csrc/sparse.cu tg_sp_walk) from
        `tab` in one call: (out int64 [m, 6], {step: kept table}, join results uint64 [m] or None)."""
        torch = self.torch
        m = len(rows)
        rows = np.ascontiguousarray(rows, dtype=np.int64)
        masks = np.ascontiguousarray(masks, dtype=U64)
        weights = np.ascontiguousarray(weights, dtype=np.int64)
        stride = masks.shape[1] if masks.ndim == 2 else 0
        cap = max(getattr(self, "_walk_cap", 1 << 12), 4 * tab.n)
        arena_bytes = max(getattr(self, "_arena_guess", 1 << 20), 1 << 16)
        out = np.zeros((max(1, m), 6), dtype=np.int64)
        need = np.zeros(2, dtype=np.int64)
        res = getattr(self, "_res", None)
        if res is None or res.numel() < max(1, m):
            res = self._res = torch.empty(max(1024, m), dtype=torch.int64, device="cuda")
        L = self.L
        while True:
            if max_states is not None and cap > 4 * max(max_states, 1) + 4 * tab.n:
                raise BudgetExceeded("a walk needs tables of %d states" % (cap // 2), "states")
            sb = int(L.tg_sp_walk_scratch_bytes(cap))
            if getattr(self, "_scratch", None) is None or self._scratch.numel() * 8 < sb:
                self._scratch = None
                self._scratch = torch.empty((sb + 7) // 8, dtype=torch.int64, device="cuda")
            arena = None
            if arena_bytes > (1 << 30):
                torch.cuda.empty_cache()     # earlier, smaller arenas stay cached otherwise
            arena = torch.empty((arena_bytes + 7) // 8, dtype=torch.int64, device="cuda")
            r = L.tg_sp_walk(m, rows.ctypes.data, masks.ctypes.data, weights.ctypes.data, stride, int(K),
                             tab.arr.data_ptr() if tab.n else None, tab.n, tab.hptr(), tab.lg,
                             self._scratch.data_ptr(), cap, arena.data_ptr(), arena_bytes, out.ctypes.data,
                             res.data_ptr(), need.ctypes.data, self.counters.data_ptr(), device.stream_ptr())
            if r < 0:
                _lib.check(r)
            if r == m:
                break
            if need[0]:
                cap = max(2 * cap, 2 * int(need[0]))
            if need[1]:
                # bytes for the steps done so far, extrapolated to the whole run, at most half the
                # free device memory (the retry grows it again if that was too little)
                guess = int(need[1]) * m // max(1, r + 1) + (1 << 20)
                cap_bytes = max(int(need[1]) + (1 << 20), torch.cuda.mem_get_info()[0] // 2)
                arena_bytes = max(arena_bytes + (arena_bytes >> 1), int(need[1]) + (1 << 20), min(guess, cap_bytes))
        self._walk_cap = cap
        kept, used = {}, 0
        ks = np.nonzero(out[:m, 2] >= 0)[0]
        if len(ks):
            sub = out[ks]
            for i, n, a, h, lg in zip(ks.tolist(), sub[:, 0].tolist(), sub[:, 2].tolist(), sub[:, 3].tolist(),
                                      sub[:, 4].tolist()):
                kept[i] = _ArenaTab(arena, a // 8, n, h // 8, lg)
            used = int((sub[:, 3] + 8 * (np.int64(1) << sub[:, 4])).max())
        self._arena_guess = max(1 << 16, used + (used >> 2))
        return out[:m], kept, (res[:m].cpu().numpy().view(U64) if want_res else None)

    def hist(self, tab):
        import torch
        h = torch.zeros(256, dtype=torch.int64, device="cuda")
        _lib.check(self.L.tg_sp_hist(tab.arr.data_ptr() if tab.n else None, tab.n, h.data_ptr(),
                                     device.stream_ptr()))
        return h.cpu().numpy()




# ---------------------------------------------------------------------- wide states
M64 = (1 << 64) - 1


def words_of(x, W):
    """A Python int as uint64 [W] (little-endian words)."""
    x = int(x)
    return np.array([(x >> (64 * i)) & M64 for i in range(W)], dtype=U64)


def pad_words(a, W):
    """uint64 [..., w] word rows (w <= W) as [..., W], the higher words zero (contiguous)."""
    a = np.asarray(a, dtype=U64)
    if a.shape[-1] == W:
        return np.ascontiguousarray(a)
    out = np.zeros(a.shape[:-1] + (W,), dtype=U64)
    out[..., :a.shape[-1]] = a
    return out


def ints_of(words):
    """uint64 [n, W] rows as Python ints."""
    words = np.asarray(words, dtype=U64)
    out = [0] * words.shape[0]
    for i in range(words.shape[1]):
        col = words[:, i].tolist()
        sh = 64 * i
        out = [o | (int(c) << sh) for o, c in zip(out, col)]
    return out


class _WTab:
    """A wide device table: n states, keys int64 [W * stride] (word w of state i at w * stride + i),
    vals uint8 [stride], index H (2^lg slots, value << 56 | state)."""
    __slots__ = ("keys", "vals", "n", "stride", "H", "lg")

    def __init__(self, keys, vals, n, stride, H, lg):
        self.keys, self.vals, self.n, self.stride, self.H, self.lg = keys, vals, n, stride, H, lg


class WideGpuTables:
    """Sparse tables of W-word states on the GPU (csrc/sparse_wide.cu).  Tables are immutable: a step
    returns new device buffers, so every table a sweep keeps stays valid."""
    name = "gpu-wide"

    def __init__(self, tr=None, words=None):
        device.require_gpu()
        nslots = getattr(tr, "nslots", 1) if tr is not None else 1
        if nslots > MAX_WIDE_SLOTS:
            raise ValueError("the wide device tables hold at most %d row slots (this trellis needs %d)"
                             % (MAX_WIDE_SLOTS, nslots))
        self.W = words if words is not None else max(1, (nslots + 63) // 64)
        self.L = _lib.lib()
        import torch
        self.torch = torch
        self.counters = torch.zeros(4, dtype=torch.int64, device="cuda")
        self.host = torch.zeros(4, dtype=torch.int64).pin_memory()
        self.result = torch.zeros(1, dtype=torch.int64, device="cuda")

    # ------------------------------------------------------------------ helpers
    def _i64(self, n):
        return self.torch.empty(max(1, int(n)), dtype=self.torch.int64, device="cuda")

    def _u8(self, n):
        return self.torch.empty(max(1, int(n)), dtype=self.torch.uint8, device="cuda")

    def _counts(self):
        self.host.copy_(self.counters)
        self.torch.cuda.current_stream().synchronize()
        c = [int(x) for x in self.host.tolist()]
        if c[2]:
            raise RuntimeError("wide device table overflow (flags %d)" % c[2])
        return c

    def _w(self, x):
        return words_of(x, self.W)

    def _filtered(self, keys, vals, n, stride, below):
        """A table of the states of (keys, vals) with value < below (all if below < 0)."""
        lg = _lg_for(n)
        nk, nv, H = self._i64(self.W * max(n, 1)), self._u8(n), self._i64(1 << lg)
        _lib.check(self.L.tg_spw_filter(self.W, keys.data_ptr() if n else None, vals.data_ptr() if n else None, n,
                                        stride, int(below), nk.data_ptr(), nv.data_ptr(), max(n, 1), H.data_ptr(), lg,
                                        self.counters.data_ptr(), device.stream_ptr()))
        m = self._counts()[0]
        return _WTab(nk, nv, m, max(n, 1), H, lg)

    # ------------------------------------------------------------------ backend interface
    def start(self):
        keys = self.torch.zeros(self.W, dtype=self.torch.int64, device="cuda")
        vals = self.torch.zeros(1, dtype=self.torch.uint8, device="cuda")
        return self._filtered(keys, vals, 1, 1, -1)

    @staticmethod
    def size(tab):
        return tab.n

    @property
    def state_bytes(self):
        return 8 * self.W + 1

    def nbytes(self, tab):
        return (8 * self.W + 1) * tab.n

    @staticmethod
    def changed_size(ch):
        return ch.n

    @staticmethod
    def persistent(tab):
        return tab

    def _host_words(self, tab):
        if tab.n == 0:
            return np.zeros((0, self.W), dtype=U64)
        k = tab.keys.view(self.W, tab.stride)[:, :tab.n].cpu().numpy().view(U64)
        return np.ascontiguousarray(k.T)

    def arrays(self, tab):
        """(keys as Python ints, vals uint8) in increasing key order (host copies)."""
        keys = ints_of(self._host_words(tab))
        vals = tab.vals[:tab.n].cpu().numpy() if tab.n else np.zeros(0, dtype=np.uint8)
        o = sorted(range(len(keys)), key=keys.__getitem__)
        return [keys[i] for i in o], vals[o] if len(o) else vals

    def from_arrays(self, keys, vals):
        n = len(keys)
        words = np.stack([self._w(k) for k in keys]) if n else np.zeros((1, self.W), dtype=U64)
        kt = self.torch.from_numpy(np.ascontiguousarray(words.T).view(np.int64).reshape(-1).copy()).cuda()
        vt = self.torch.from_numpy(np.asarray(vals, dtype=np.uint8).copy() if n else np.zeros(1, np.uint8)).cuda()
        return self._filtered(kt, vt, n, max(n, 1), -1)

    def lookup_many(self, tab, keys):
        m = len(keys)
        if not m or tab.n == 0:
            return np.full(m, INF, dtype=np.uint8)
        words = np.stack([self._w(k) for k in keys])
        q = self.torch.from_numpy(np.ascontiguousarray(words.T).view(np.int64).reshape(-1).copy()).cuda()
        out = self._u8(m)
        _lib.check(self.L.tg_spw_lookup(self.W, tab.H.data_ptr(), tab.lg, tab.keys.data_ptr(), tab.stride,
                                        q.data_ptr(), m, out.data_ptr(), device.stream_ptr()))
        return out[:m].cpu().numpy()

    def lookup(self, tab, s):
        if int(s) >> (64 * self.W):
            return INF
        return int(self.lookup_many(tab, [s])[0])

    def truncate(self, tab, below):
        return self._filtered(tab.keys, tab.vals, tab.n, tab.stride, int(below))

    def hist(self, tab):
        if tab.n == 0:
            return np.zeros(256, dtype=np.int64)
        return self.torch.bincount(tab.vals[:tab.n].long(), minlength=256).cpu().numpy()

    def step(self, tab, upd, sel_mask, sel_bits, cap, K, tmask, hd, keep_below=None, want_changed=False, w=1):
        """One column (the rule of cdist/sparse_dp.py:338-403 with a column weight w): returns
        (table, changed)."""
        W, n = self.W, tab.n
        ecap = max(1, 2 * n)
        lgs = _lg_for(2 * n)
        ek, ev, Hs = self._i64(W * ecap), self._u8(ecap), self._i64(1 << lgs)
        ncap = ecap
        lgn = _lg_for(2 * n)
        nk, nv, Hn = self._i64(W * ncap), self._u8(ncap), self._i64(1 << lgn)
        ccap = max(1, n)
        ck = self._i64(W * ccap) if want_changed else None
        cv = self._u8(ccap) if want_changed else None
        if hd is None:
            ncls, mp, wp, extra, use_h = 0, None, None, 0, 0
        else:
            m_arr = pad_words(np.asarray(hd[0], dtype=U64).reshape(len(hd[1]), -1), W) if len(hd[1]) \
                else np.zeros((1, W), dtype=U64)
            w_arr = np.ascontiguousarray(hd[1], dtype=np.int64) if len(hd[1]) else np.zeros(1, dtype=np.int64)
            ncls, mp, wp, extra, use_h = len(hd[1]), m_arr.ctypes.data, w_arr.ctypes.data, int(hd[2]), 1
        uw, sm, sb, tw = self._w(upd), self._w(sel_mask), self._w(sel_bits), self._w(tmask)
        _lib.check(self.L.tg_spw_step(W, tab.keys.data_ptr(), tab.vals.data_ptr(), n, tab.stride, tab.H.data_ptr(),
                                      tab.lg, ek.data_ptr(), ev.data_ptr(), ecap, Hs.data_ptr(), lgs, nk.data_ptr(),
                                      nv.data_ptr(), ncap, Hn.data_ptr(), lgn,
                                      ck.data_ptr() if ck is not None else None,
                                      cv.data_ptr() if cv is not None else None, ccap, uw.ctypes.data, sm.ctypes.data,
                                      sb.ctypes.data, int(cap), -1 if keep_below is None else int(keep_below), int(w),
                                      int(bool(want_changed)), use_h, int(K), ncls, mp, wp, extra, tw.ctypes.data,
                                      self.counters.data_ptr(), device.stream_ptr()))
        c = self._counts()
        new = _WTab(nk, nv, c[0], ncap, Hn, lgn)
        changed = _WTab(ck, cv, c[1], ccap, None, 0) if want_changed else None
        return new, changed

    def walk(self, tab, steps, words, masks, weights, K, max_states=None, want_res=True):
        """Run the column steps (int64 [m, 13] step records and uint64 [m, 5, W] words,
        csrc/sparse_wide.cu tg_spw_walk) from `tab` in one call, the table sizes kept on the device:
        (out int64 [m, 6], {step: kept table}, join results uint64 [m, 2 + W] or None)."""
        torch, L, W = self.torch, self.L, self.W
        m = len(steps)
        steps = np.ascontiguousarray(steps, dtype=np.int64)
        words = np.ascontiguousarray(words, dtype=U64)
        masks = np.ascontiguousarray(masks, dtype=U64)
        weights = np.ascontiguousarray(weights, dtype=np.int64)
        maxc = weights.shape[1] if weights.ndim == 2 else 1
        cap = max(getattr(self, "_walk_cap", 1 << 12), 2 * tab.n)
        arena_bytes = max(getattr(self, "_arena_guess", 1 << 20), 1 << 16)
        out = np.zeros((max(1, m), 6), dtype=np.int64)
        res = np.zeros((max(1, m), 2 + W), dtype=U64)
        need = np.zeros(2, dtype=np.int64)
        while True:
            if max_states is not None and cap > 4 * max(max_states, 1) + 4 * tab.n:
                raise BudgetExceeded("a walk needs tables of %d states" % (cap // 2), "states")
            sb = int(L.tg_spw_walk_scratch_bytes(W, cap, m))
            if sb < 0:
                raise ValueError("bad wide walk size")
            if getattr(self, "_scratch", None) is None or self._scratch.numel() * 8 < sb:
                self._scratch = None
                self._scratch = torch.empty((sb + 7) // 8, dtype=torch.int64, device="cuda")
            arena = None
            if arena_bytes > (1 << 30):
                torch.cuda.empty_cache()     # earlier, smaller arenas stay cached otherwise
            arena = torch.empty((arena_bytes + 7) // 8, dtype=torch.int64, device="cuda")
            r = L.tg_spw_walk(W, m, steps.ctypes.data, words.ctypes.data, masks.ctypes.data, weights.ctypes.data,
                              maxc, int(K), tab.keys.data_ptr() if tab.n else None,
                              tab.vals.data_ptr() if tab.n else None, tab.n, tab.stride, self._scratch.data_ptr(),
                              cap, arena.data_ptr(), arena_bytes, out.ctypes.data, res.ctypes.data,
                              need.ctypes.data, device.stream_ptr())
            if r < 0:
                _lib.check(r)
            if r == m:
                break
            if need[0]:
                cap = max(2 * cap, int(need[0]))
            if need[1]:
                arena_bytes = max(arena_bytes + (arena_bytes >> 1), int(need[1]) + (1 << 20))
        self._walk_cap = cap
        kept, used = {}, 0
        u8 = arena.view(torch.uint8)
        for i in np.nonzero(out[:m, 2] >= 0)[0].tolist():
            n, o, st, lg = (int(x) for x in out[i, [0, 2, 3, 4]])
            vo = o + 8 * W * st
            ho = vo + (st + 255) // 256 * 256
            kept[i] = _WTab(arena[o // 8:o // 8 + W * st], u8[vo:vo + st], n, st, arena[ho // 8:ho // 8 + (1 << lg)],
                            lg)
            used = max(used, ho + (8 << lg))
        self._arena_guess = max(1 << 16, used + (used >> 2))
        return out[:m], kept, (res[:m] if want_res else None)

    @staticmethod
    def walk_best(res):
        """The first least join total of a walk's results: (step, total, forward key) or None."""
        tot = res[:, 0]
        hit = np.nonzero(tot != U64(M64))[0]
        if not len(hit):
            return None
        k = int(hit[np.argmin(tot[hit])])
        return k, int(tot[k]), ints_of(res[k:k + 1, 2:])[0]

    def join(self, ch, btab, tmask):
        """(total, forward key, forward value, backward key) of the least f.value + b.value over
        changed f and backward b with key(b) = key(f) ^ tmask, or None."""
        if ch is None or not ch.n or not btab.n:
            return None
        tw = self._w(tmask)
        _lib.check(self.L.tg_spw_join(self.W, ch.keys.data_ptr(), ch.vals.data_ptr(), ch.n, ch.stride,
                                      btab.H.data_ptr(), btab.lg, btab.keys.data_ptr(), btab.stride, tw.ctypes.data,
                                      self.result.data_ptr(), device.stream_ptr()))
        r = int(self.result.item()) & M64
        if r == M64:
            return None
        total, i = r >> 40, r & ((1 << 40) - 1)
        fw = ch.keys.view(self.W, ch.stride)[:, i].cpu().numpy().view(U64)
        fkey = ints_of(fw[None, :])[0]
        fval = int(ch.vals[i].item())
        return int(total), fkey, fval, fkey ^ int(tmask)
