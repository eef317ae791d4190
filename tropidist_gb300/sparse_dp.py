"""Weight-truncated sparse Rank DP with device hash tables (drop-in for cdist/sparse_dp.py).

The host side keeps the reference's structure and API:
  Trellis          fixed row slots by interval colouring, per-position column / selection masks,
                   active rows and the lookahead data (cdist/sparse_dp.py:63-205)
  Sweep            one truncated sweep with checkpoints every isqrt(N) cuts, segment recomputation
                   and traceback (cdist/sparse_dp.py:621-819)
  choose_split / choose_schedule   probe sweeps and the split DP (cdist/sparse_dp.py:823-981)
  query, distance  forward / meet-in-the-middle queries, iterative deepening (cdist/sparse_dp.py:985-1151)
The tables live on the GPU: BACKENDS["gpu"] (GpuTables) stores a table as packed states
key | value << 56 in a device array plus an open-addressing device index, and runs a column step,
a join and lookups as kernels of libtropigpu (csrc/sparse.cu).  Any object with the backend
interface of cdist/sparse_dp.py:300-445 can be passed as `backend`.

Differences from the reference: the dense fallback of Sweep (`dense=`) is accepted and not used
(the device tables handle dense cuts); columns may carry integer weights (Trellis(weights=...)),
which the reference does not have.
"""
from __future__ import annotations

import ctypes
import heapq
import math
import time

import numpy as np

from . import _lib, device, trellis

INF = 255
MAX_WEIGHT = INF - 1
Q = 720720                      # lcm(1..16): lookahead weights are multiples of 1/Q (rounded down)
U64 = np.uint64
KEYMASK = (1 << 56) - 1
MAX_SLOTS = 56                  # row slots of a packed device state


def _bits(x):
    out = []
    while x:
        low = x & -x
        out.append(low.bit_length() - 1)
        x ^= low
    return out


class Trellis:
    """Minimal-span trellis of one query min{|e| : H e = 0, (L e)_obs = 1} in a column order, with
    fixed row slots so that a state means the same in both sweep directions.  Cut c separates
    positions [0, c) from [c, N).  weights: optional per-column integer weights (problem indices)."""

    def __init__(self, h, lrow, order, nrows, name="", weights=None):
        self.name = name
        self.order = list(order)
        self.N = N = len(self.order)
        self.cw = [1] * N if weights is None else [int(weights[j]) for j in self.order]
        hrows = trellis.minimal_span_form(trellis.rows_from_columns(h, self.order, nrows))
        lr = trellis.reduce_target_row(lrow, hrows)
        self.feasible = lr != 0
        if not self.feasible:
            return
        rows = list(hrows) + [lr]
        self.rows = rows
        self.target = [0] * len(hrows) + [1]
        self.L = len(rows) - 1
        self.start = [trellis.lowbit(r) for r in rows]
        self.end = [r.bit_length() - 1 for r in rows]
        # interval colouring: rows whose closed spans overlap get distinct slots; the smallest free
        # slot is reused (cdist/sparse_dp.py:85-99)
        slot = [0] * len(rows)
        free, busy, nslots = [], [], 0
        for r in sorted(range(len(rows)), key=lambda r: self.start[r]):
            while busy and busy[0][0] < self.start[r]:
                heapq.heappush(free, heapq.heappop(busy)[1])
            if free:
                s = heapq.heappop(free)
            else:
                s, nslots = nslots, nslots + 1
            slot[r] = s
            heapq.heappush(busy, (self.end[r], s))
        if nslots > 64:
            raise ValueError("trellis needs %d bits per state (at most 64 supported)" % nslots)
        self.slot, self.nslots = slot, nslots
        nr = len(rows)
        # positions of every row (CSR), and per position the slots of the rows through it
        self.row_ptr, self.row_cols = trellis.bit_positions(rows, N)
        entry_row = np.repeat(np.arange(nr, dtype=np.int64), np.diff(self.row_ptr))
        sbit = np.left_shift(np.uint64(1), np.asarray(slot, dtype=np.uint64))
        colm = np.zeros(max(1, N), dtype=U64)
        np.bitwise_or.at(colm, self.row_cols, sbit[entry_row])
        self.col = colm[:N].tolist()
        fsm, fsb, bsm, bsb = [0] * N, [0] * N, [0] * N, [0] * N
        starts_at, ends_at = [[] for _ in range(N)], [[] for _ in range(N)]
        for r in range(len(rows)):
            b = 1 << slot[r]
            fsm[self.end[r]] |= b              # a forward sweep checks a row where it ends
            bsm[self.start[r]] |= b            # a backward sweep where it starts
            if self.target[r]:
                fsb[self.end[r]] |= b
                bsb[self.start[r]] |= b
            starts_at[self.start[r]].append((slot[r], self.target[r]))
            ends_at[self.end[r]].append((slot[r], self.target[r]))
        self.fsel_mask, self.fsel_bits, self.bsel_mask, self.bsel_bits = fsm, fsb, bsm, bsb
        self.starts_at, self.ends_at = starts_at, ends_at
        # row r is active at the cuts start[r] < c <= end[r]: per cut the active rows (CSR, rows
        # ascending), their slots as a mask (slots never overlap in time) and their number
        st = np.asarray(self.start, dtype=np.int64)
        en = np.asarray(self.end, dtype=np.int64)
        ln = en - st
        tot = int(ln.sum())
        first = np.repeat(st + 1, ln)
        off = np.arange(tot, dtype=np.int64) - np.repeat(np.cumsum(ln) - ln, ln)
        cuts = first + off
        rid = np.repeat(np.arange(nr, dtype=np.int64), ln)
        o = np.lexsort((rid, cuts))
        self.act_rows = rid[o].astype(np.int32)
        self.act_ptr = np.zeros(N + 2, dtype=np.int64)
        self.act_ptr[1:] = np.cumsum(np.bincount(cuts, minlength=N + 1))[:N + 1]
        delta = np.zeros(N + 2, dtype=U64)
        np.bitwise_xor.at(delta, st + 1, sbit)
        np.bitwise_xor.at(delta, en + 1, sbit)
        act_mask = np.bitwise_xor.accumulate(delta)[:N + 1]
        self.active = act_mask.tolist()
        self.width = np.diff(self.act_ptr).tolist()
        lbit = int(sbit[self.L])         # the target row's own interval (its slot is shared over time)
        sL, eL = self.start[self.L], self.end[self.L]
        self.tmask = [lbit if sL < c <= eL else 0 for c in range(N + 1)]
        self._bd = {}

    @property
    def active_rows(self):
        """The active rows of every cut (lists, rows ascending)."""
        if getattr(self, "_active_rows", None) is None:
            rows = self.act_rows.tolist()
            ptr = self.act_ptr.tolist()
            self._active_rows = [rows[ptr[c]:ptr[c + 1]] for c in range(self.N + 1)]
        return self._active_rows

    @classmethod
    def for_query(cls, p, obs, order):
        lrow = 0
        for pos, j in enumerate(order):
            if (p.l[j] >> obs) & 1:
                lrow |= 1 << pos
        return cls(p.h, lrow, order, p.nrows, name="%s obs %d" % (getattr(p, "name", ""), obs),
                   weights=getattr(p, "weights", None))

    # ------------------------------------------------------------------ lookahead bound
    def _bound_data(self, forward):
        """Per cut: (masks, weights, extra) of the lookahead bound, computed by the library's host
        routine (tg_sp_bound_data; the same rule as _bound_data_py)."""
        N, rows = self.N, self.rows
        nr = len(rows)
        row_ptr, row_cols = self.row_ptr, self.row_cols
        # the transpose: rows through every position, rows ascending
        entry_row = np.repeat(np.arange(nr, dtype=np.int32), np.diff(row_ptr))
        o = np.argsort(row_cols, kind="stable")
        col_rows = entry_row[o]
        col_ptr = np.zeros(N + 1, dtype=np.int64)
        col_ptr[1:] = np.cumsum(np.bincount(row_cols, minlength=N))[:N]
        act_ptr, act_rows = self.act_ptr, self.act_rows
        start = np.array(self.start, dtype=np.int32)
        end = np.array(self.end, dtype=np.int32)
        slot = np.array(self.slot, dtype=np.int32)
        maxc = 48
        ncls = np.zeros(N + 1, dtype=np.int32)
        masks = np.zeros((N + 1, maxc), dtype=U64)
        wts = np.zeros((N + 1, maxc), dtype=np.int64)
        extra = np.zeros(N + 1, dtype=np.int64)
        ptr = lambda a: a.ctypes.data if a.size else None
        _lib.check(_lib.lib().tg_sp_bound_data(N, nr, ptr(row_ptr), ptr(row_cols), ptr(col_ptr), ptr(col_rows),
                                               ptr(act_ptr), ptr(act_rows), ptr(start), ptr(end), ptr(slot), self.L,
                                               int(bool(forward)), maxc, ptr(ncls), ptr(masks), ptr(wts),
                                               ptr(extra)))
        k = max(1, int(ncls.max()) if ncls.size else 1)
        return ncls, masks[:, :k].copy(), wts[:, :k].copy(), extra

    def _bound_data_py(self, forward):
        """Per cut: (masks, weights, extra) of h(s) = ceil((extra + sum_k w_k |(s ^ tmask) & mask_k|) / Q).
        Row r relevant at cut c gets weight y_r = 1 / max over remaining columns j containing r of
        |supp(j) ∩ relevant rows| (a dual solution of the covering LP), rounded down to 1/Q; the
        target row counts while it lies wholly on the remaining side (cdist/sparse_dp.py:148-192)."""
        N, rows = self.N, self.rows
        S = np.zeros((len(rows), N), dtype=np.int32)
        for r, row in enumerate(rows):
            S[r, _bits(row)] = 1
        out = []
        for c in range(N + 1):
            rel = list(self.active_rows[c])
            lone = (forward and self.start[self.L] >= c) or (not forward and self.end[self.L] < c)
            if lone:
                rel.append(self.L)
            if not rel:
                out.append(((), (), 0))
                continue
            if forward:
                lo, hi = c, max(self.end[r] for r in rel) + 1
            else:
                lo, hi = min(self.start[r] for r in rel), c
            sub = S[rel, lo:hi]
            per_col = sub.sum(axis=0)
            worst = (sub * per_col).max(axis=1)
            assert (worst >= 1).all()
            wts = Q // worst
            masks, extra = {}, 0
            for r, wr in zip(rel, wts.tolist()):
                if lone and r == self.L:
                    extra = wr
                else:
                    masks[wr] = masks.get(wr, 0) | (1 << self.slot[r])
            ks = sorted(masks)
            out.append((tuple(U64(masks[k]) for k in ks), tuple(np.int64(k) for k in ks), extra))
        return out

    def bound_raw(self, forward):
        """(ncls int32[N+1], masks uint64[N+1, k], weights int64[N+1, k], extra int64[N+1])."""
        key = ("raw", forward)
        if key not in self._bd:
            self._bd[key] = self._bound_data(forward)
        return self._bd[key]

    def bound_data(self, forward):
        """Per cut: (masks, weights, extra) tuples."""
        if forward not in self._bd:
            ncls, masks, wts, extra = self.bound_raw(forward)
            self._bd[forward] = [(tuple(masks[c, :int(ncls[c])]), tuple(wts[c, :int(ncls[c])]), int(extra[c]))
                                 for c in range(self.N + 1)]
        return self._bd[forward]

    def bound_arrays(self, forward):
        """Per cut (masks uint64, weights int64, extra), built on access."""
        key = ("arrays", forward)
        if key not in self._bd:
            self._bd[key] = _BoundView(*self.bound_raw(forward))
        return self._bd[key]


class _BoundView:
    """The lookahead data of every cut as a sequence of (masks, weights, extra), views of arrays."""

    def __init__(self, ncls, masks, weights, extra):
        self.ncls, self.masks, self.weights, self.extra = ncls, masks, weights, extra

    def __len__(self):
        return len(self.ncls)

    def __getitem__(self, c):
        k = int(self.ncls[c])
        return self.masks[c, :k], self.weights[c, :k], int(self.extra[c])


def bound(keys, tmask, hd):
    """The lookahead lower bound for an array of states (host helper, cdist/sparse_dp.py:208-217)."""
    masks, weights, extra = hd
    if not len(masks):
        return np.full(keys.shape, (extra + Q - 1) // Q, dtype=np.int64)
    u = keys ^ U64(tmask)
    tot = np.full(keys.shape, extra, dtype=np.int64)
    for m, w in zip(masks, weights):
        tot += np.int64(w) * np.bitwise_count(u & U64(m)).astype(np.int64)
    return (tot + (Q - 1)) // Q


# ---------------------------------------------------------------------- device tables
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
                # bytes for the steps done so far, extrapolated to the whole run
                arena_bytes = max(arena_bytes + (arena_bytes >> 1), int(need[1]) * m // max(1, r + 1) + (1 << 20))
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


BACKENDS = {"gpu": GpuTables}


class BudgetExceeded(RuntimeError):
    """A table outgrew max_states (kind "states") or a sweep passed its deadline (kind "deadline")."""

    def __init__(self, message, kind):
        super().__init__(message)
        self.kind = kind


def _backend(backend, tr):
    if isinstance(backend, str):
        return BACKENDS[backend](tr)
    return backend


# ---------------------------------------------------------------------- sweeps
class Sweep:
    """One direction of the truncated sweep of a trellis, with tables at checkpoints
    (cdist/sparse_dp.py:621-819).  direction +1: cuts 0 -> N from {0: 0}; -1: N -> 0.  caps: the
    largest weight kept at each cut (non-increasing in the sweep direction).  frontier (forward
    sweeps of the meet in the middle): the step out of cut p keeps weights <= caps[p] - 1 and returns
    the new or improved states of weight <= caps[p] as `changed`; where caps drops, the table before
    the drop is returned as `extra` to be joined in full."""

    def __init__(self, tr, direction, K, cap=None, use_h=True, every=None, frontier=False, backend="gpu",
                 dense=None, dense_max=1 << 30, max_states=None, deadline=None, caps=None):
        self.tr, self.direction, self.K = tr, direction, K
        self.caps = [min(int(x), K) for x in caps] if caps is not None else [min(cap, K)] * (tr.N + 1)
        if max(self.caps) > MAX_WEIGHT:
            raise ValueError("a sweep keeping weights up to %d: the tables hold at most %d (8-bit values)"
                             % (max(self.caps), MAX_WEIGHT))
        pairs = list(zip(self.caps, self.caps[1:]))
        if direction > 0:
            assert all(x >= y for x, y in pairs), "forward caps must not increase"
        else:
            assert all(x <= y for x, y in pairs), "backward caps must not decrease"
        self.use_h = use_h
        self.frontier = frontier
        self.be = _backend(backend, tr)
        self.hd = tr.bound_arrays(direction > 0) if use_h else None
        self.every = every or max(1, int(math.isqrt(tr.N)))
        self.dense = None
        self.max_states, self.deadline = max_states, deadline
        self.ckpt = {}
        self.counts = [0] * (tr.N + 1)
        self.changed_counts = [0] * (tr.N + 1)
        self.dense_cuts = 0
        self.peak = 0
        self.peak_bytes = 0
        self.steps_done = 0
        self._all = None
        # device walks: tables of at most SMALL_KEEP states are kept at every cut (within a byte
        # budget), so a meet in the middle reads them instead of recomputing segments
        self.small_tabs = {}
        self.small_bytes = 0

    RUN_STEPS = 4096            # steps per device walk of a sweep that joins nothing
    SMALL_KEEP_BYTES = 256 << 20

    def first(self):
        return (0 if self.direction > 0 else self.tr.N), self.be.start()

    def _step(self, tab, p, want_changed):
        tr, fwd = self.tr, self.direction > 0
        cut = p + 1 if fwd else p
        sm, sb = (tr.fsel_mask[p], tr.fsel_bits[p]) if fwd else (tr.bsel_mask[p], tr.bsel_bits[p])
        self.steps_done += 1
        cap, kb = self.caps[cut], None
        if self.frontier:
            cap = kb = self.caps[p]
        kw = {} if tr.cw[p] == 1 else {"w": tr.cw[p]}
        tab, ch = self.be.step(tab, tr.col[p], sm, sb, cap, self.K, tr.tmask[cut],
                               self.hd[cut] if self.hd else None, kb, want_changed, **kw)
        if self.frontier and self.caps[cut] < cap:
            return cut, self.be.truncate(tab, self.caps[cut]), ch, tab
        return cut, tab, ch, None

    # ---- device walks (GpuTables): a run of steps per library call
    def _rows(self, positions, keep, joins=None):
        """Spec rows of tg_sp_walk for the steps at `positions` (as _step), with lookahead arrays;
        keep: per step 0/1; joins: per step None or (backward table, tmask)."""
        if getattr(self, "_all", None) is None:
            self._all = self._all_rows()
        rows0, masks0, weights0 = self._all
        pos = np.asarray(positions, dtype=np.int64)
        rows = rows0[pos].copy()
        rows[:, 12] = np.asarray(keep, dtype=np.int64)
        if joins is not None:
            rows[:, 10] = 1
            ks = [k for k, j in enumerate(joins) if j is not None]
            if ks:
                rows[ks, 4] = [joins[k][0].hptr() for k in ks]
                rows[ks, 5] = [int(joins[k][1]) & KEYMASK for k in ks]
                rows[ks, 13] = [joins[k][0].lg for k in ks]
        return rows, masks0[pos], weights0[pos]

    def _all_rows(self):
        """Spec rows of every step position of this sweep (without keep / join columns)."""
        tr, fwd = self.tr, self.direction > 0
        N = tr.N
        p = np.arange(N)
        cut = p + 1 if fwd else p
        u64 = lambda xs: np.array([int(x) for x in xs], dtype=U64).view(np.int64)
        caps = np.asarray(self.caps, dtype=np.int64)
        rows = np.zeros((max(1, N), 16), dtype=np.int64)
        if N == 0:
            return rows, np.zeros((1, 1), dtype=U64), np.zeros((1, 1), dtype=np.int64)
        rows[:, 0] = u64(tr.col) & np.int64(KEYMASK)
        rows[:, 1] = u64(tr.fsel_mask if fwd else tr.bsel_mask)
        rows[:, 2] = u64(tr.fsel_bits if fwd else tr.bsel_bits)
        rows[:, 3] = u64(tr.tmask)[cut] & np.int64(KEYMASK)
        cap = caps[cut].copy()
        kb = np.full(N, -1, dtype=np.int64)
        trunc = np.full(N, -1, dtype=np.int64)
        if self.frontier:
            cap = caps[p].copy()
            kb = cap.copy()
            drop = caps[cut] < cap
            trunc[drop] = caps[cut][drop]
        rows[:, 7], rows[:, 8], rows[:, 11] = cap, kb, trunc
        rows[:, 9] = np.asarray(tr.cw, dtype=np.int64)
        if self.use_h:
            ncls, masks, wts, extra = tr.bound_raw(fwd)
            rows[:, 6] = extra[cut]
            rows[:, 14] = ncls[cut]
            rows[:, 15] = 1
            return rows, np.ascontiguousarray(masks[cut]), np.ascontiguousarray(wts[cut])
        return rows, np.zeros((N, 1), dtype=U64), np.zeros((N, 1), dtype=np.int64)

    def _positions(self, c, stop):
        return list(range(c, stop)) if self.direction > 0 else list(range(c - 1, stop - 1, -1))

    def _cut_of(self, p):
        return p + 1 if self.direction > 0 else p

    def _next_ckpt(self, c, stop):
        if self.direction > 0:
            return min(stop, (c // self.every + 1) * self.every)
        return max(stop, (c - 1) // self.every * self.every)

    def _run_walk(self, join_with=None, lower=0):
        """run() on device walks, one per checkpoint interval; join_with: the backward sweep whose
        tables the changed states of every cut are joined with (the meet in the middle).  Returns
        (last cut, best join (total, cut, forward key) or None)."""
        c0, tab = self.first()
        self.ckpt[c0] = tab
        self.counts[c0] = self.changed_counts[c0] = 1
        self.peak = 1
        best = None
        cache = {}
        if join_with is not None:
            r = self.be.join(_as_changed(self.be, tab), join_with.table(c0, cache), self.tr.tmask[c0])
            if r is not None:
                best = (r[0], c0, r[1])
        stop = self.tr.N if self.direction > 0 else 0
        ck_bytes = self.be.nbytes(tab)
        c = c0
        while c != stop and not (best is not None and best[0] <= max(lower, 0)):
            c1 = self._next_ckpt(c, stop)
            if join_with is None:           # no early stop possible: several intervals per walk
                while c1 != stop and abs(c1 - c) < self.RUN_STEPS:
                    c1 = self._next_ckpt(c1, stop)
            pos = self._positions(c, c1)
            cuts = [p + 1 for p in pos] if self.direction > 0 else pos
            small = 2 if self.small_bytes < self.SMALL_KEEP_BYTES else 0
            keep = [1 if self.is_ckpt(cut) else small for cut in cuts]
            keep[-1] = 1
            joins = None
            if join_with is not None:
                joins = [(join_with.table(cut, cache), self.tr.tmask[cut]) for cut in cuts]
            rows, masks, weights = self._rows(pos, keep, joins)
            out, kept, res = self.be.walk(tab, rows, masks, weights, self.K, self.max_states,
                                          want_res=join_with is not None)
            self.steps_done += len(pos)
            for cut, a, b in zip(cuts, out[:, 0].tolist(), out[:, 1].tolist()):
                self.counts[cut] = a
                self.changed_counts[cut] = b
            self.peak = max(self.peak, int(out[:, [0, 1, 5]].max()))
            if join_with is not None:
                ok = np.nonzero(res != U64(0xFFFFFFFFFFFFFFFF))[0]
                if len(ok):
                    k = int(ok[np.argmin(res[ok] >> U64(56))])      # the first least total
                    total = int(res[k]) >> 56
                    if best is None or total < best[0]:
                        best = (total, cuts[k], int(res[k]) & KEYMASK)
            for k, t in kept.items():
                if keep[k] == 1:
                    if k != len(pos) - 1:
                        self.ckpt[cuts[k]] = t
                        ck_bytes += self.be.nbytes(t)
                else:
                    self.small_tabs[cuts[k]] = t
                    self.small_bytes += 8 * (t.n + (1 << t.lg)) + 256
            tab = kept[len(pos) - 1]
            c = c1
            self.ckpt[c] = tab
            ck_bytes += self.be.nbytes(tab)
            self.peak_bytes = max(self.peak_bytes, ck_bytes + 8 * int(out[:, 5].max()))
            if self.max_states is not None and self.peak > self.max_states:
                raise BudgetExceeded("%d states before cut %d" % (self.peak, c), "states")
            if self.deadline is not None and time.monotonic() > self.deadline:
                raise BudgetExceeded("deadline at cut %d" % c, "deadline")
        return c, best

    def _walk(self, cut, tab, stop, want_changed=False):
        rng = range(cut, stop) if self.direction > 0 else range(cut - 1, stop - 1, -1)
        for p in rng:
            c, tab, ch, extra = self._step(tab, p, want_changed)
            yield c, tab, ch, extra

    def is_ckpt(self, c):
        return c % self.every == 0 or c == 0 or c == self.tr.N

    def run(self, on_cut=None):
        """Full sweep keeping checkpoints and per-cut counts; on_cut(cut, table, changed, extra) may
        return True to stop.  Returns the last cut reached."""
        if on_cut is None and isinstance(self.be, GpuTables):
            return self._run_walk()[0]
        c0, tab = self.first()
        self.ckpt[c0] = tab
        self.counts[c0] = self.changed_counts[c0] = 1
        self.peak = 1
        if on_cut and on_cut(c0, tab, _as_changed(self.be, tab), None):
            return c0
        stop = self.tr.N if self.direction > 0 else 0
        ck_bytes = self.be.nbytes(tab)
        for c, tab, ch, extra in self._walk(c0, tab, stop, want_changed=on_cut is not None):
            n = self.be.size(tab)
            self.counts[c] = n
            nc = self.be.changed_size(ch) if ch is not None else 0
            self.changed_counts[c] = nc
            self.peak = max(self.peak, n, nc)
            if self.is_ckpt(c):
                self.ckpt[c] = self.be.persistent(tab)
                ck_bytes += self.be.nbytes(tab)
            self.peak_bytes = max(self.peak_bytes, ck_bytes + self.be.nbytes(tab))
            if self.max_states is not None and max(n, nc) > self.max_states:
                raise BudgetExceeded("%d states at cut %d" % (max(n, nc), c), "states")
            if self.deadline is not None and time.monotonic() > self.deadline:
                raise BudgetExceeded("deadline at cut %d" % c, "deadline")
            if on_cut and on_cut(c, tab, ch, extra):
                return c
        return stop

    def segment(self, lo, hi):
        """Tables at the cuts lo..hi, recomputed from the nearest checkpoint: {cut: table}."""
        if isinstance(self.be, GpuTables):
            return self._segment_walk(lo, hi)
        out = {}
        if self.direction > 0:
            c0 = max(c for c in self.ckpt if c <= lo)
            tab = self.ckpt[c0]
            if c0 >= lo:
                out[c0] = tab
            for c, tab, _, _ in self._walk(c0, tab, hi):
                if c >= lo:
                    out[c] = self.be.persistent(tab)
        else:
            c0 = min(c for c in self.ckpt if c >= hi)
            tab = self.ckpt[c0]
            if c0 <= hi:
                out[c0] = tab
            for c, tab, _, _ in self._walk(c0, tab, lo):
                if c <= hi:
                    out[c] = self.be.persistent(tab)
        return out

    def _segment_walk(self, lo, hi):
        if self.direction > 0:
            c0 = max(c for c in self.ckpt if c <= lo)
            stop = hi
        else:
            c0 = min(c for c in self.ckpt if c >= hi)
            stop = lo
        out = {}
        tab = self.ckpt[c0]
        if lo <= c0 <= hi:
            out[c0] = tab
        pos = self._positions(c0, stop)
        if pos:
            keep = [1 if lo <= self._cut_of(p) <= hi else 0 for p in pos]
            rows, masks, weights = self._rows(pos, keep)
            _, kept, _ = self.be.walk(tab, rows, masks, weights, self.K, self.max_states, want_res=False)
            for k, p in enumerate(pos):
                if keep[k]:
                    out[self._cut_of(p)] = kept[k]
        return out

    def table(self, c, cache):
        """Table at cut c for cuts requested against the sweep's direction (cache reused between calls)."""
        t = self.small_tabs.get(c) or self.ckpt.get(c)
        if t is not None:
            return t
        if c not in cache:
            cache.clear()
            if self.direction < 0:
                cache.update(self.segment(c, min(x for x in self.ckpt if x >= c)))
            else:
                cache.update(self.segment(max(x for x in self.ckpt if x <= c), c))
        return cache[c]

    def traceback(self, cut, state, value):
        """Columns (problem indices) of a partial solution reaching `state` with weight `value` at `cut`."""
        tr = self.tr
        used = []
        s, v = int(state), int(value)
        if self.direction > 0:
            c = cut
            while c > 0:
                lo = max(0, (c - 1) // self.every * self.every)
                tabs = self.segment(lo, c - 1)
                for p in range(c - 1, lo - 1, -1):            # step p: cut p -> p + 1
                    s, v = self._undo(tabs[p], s, v, s | tr.fsel_bits[p], p, used)
                c = lo
        else:
            c = cut
            while c < tr.N:
                hi = min(tr.N, (c // self.every + 1) * self.every)
                tabs = self.segment(c + 1, hi)
                for p in range(c, hi):                          # backward step p: cut p + 1 -> p
                    s, v = self._undo(tabs[p + 1], s, v, s | tr.bsel_bits[p], p, used)
                c = hi
        assert s == 0 and v == 0, (s, v)
        return used

    def _undo(self, tab, s, v, s_mid, p, used):
        tr = self.tr
        if self.be.lookup(tab, s_mid) == v:
            return s_mid, v
        prev, w = s_mid ^ tr.col[p], tr.cw[p]
        assert tr.col[p] and self.be.lookup(tab, prev) == v - w, "traceback lost the path"
        used.append(tr.order[p])
        return prev, v - w


def _as_changed(be, tab):
    """The start table as a `changed` object of the backend (joined in full at the first cut)."""
    if isinstance(be, GpuTables):
        return _Changed(tab.arr, tab.n)
    return tab


# ---------------------------------------------------------------------- choice of the split
def weight_profile(tr, direction, cap, backend="gpu"):
    """States of each weight <= cap summed over all cuts of a sweep keeping weights <= cap."""
    sw = Sweep(tr, direction, cap, cap, use_h=False, backend=backend)
    c0, tab = sw.first()
    tot = np.zeros(cap + 1)
    tot[0] = 1
    for c, tab, _, _ in sw._walk(c0, tab, tr.N if direction > 0 else 0):
        tot += _hist(sw.be, tab)[:cap + 1]
    return tot


def _hist(be, tab):
    if hasattr(be, "hist"):
        return np.asarray(be.hist(tab), dtype=np.float64)
    return np.bincount(be.arrays(tab)[1], minlength=256).astype(np.float64)


def choose_split(tr, K, backend="gpu", probe=3, budget=2e9):
    """Split a minimising sum_{w <= a-1} F(w) + F(a-1) + 2 sum_{w <= K-a} B(w) from measured and
    extrapolated weight profiles (cdist/sparse_dp.py:839-867).  Returns (a, info)."""
    t0 = time.time()
    prof = {}
    for direction in (+1, -1):
        p = weight_profile(tr, direction, min(2, probe), backend)
        if probe > 2 and len(p) > 2 and p[1] > 0 and p[2] * p[2] / p[1] < budget:
            p = weight_profile(tr, direction, probe, backend)
        prof[direction] = p

    def extend(p, upto):
        p = list(p)
        r = p[-1] / p[-2] if len(p) > 1 and p[-2] > 0 else 1.0
        while len(p) <= upto:
            p.append(p[-1] * max(r, 1.0))
        return p

    F, B = extend(prof[+1], K), extend(prof[-1], K)
    costs = {a: sum(F[:a]) + F[a - 1] + 2 * sum(B[:K - a + 1]) for a in range(1, K + 1)}
    a = min(costs, key=costs.get)
    return a, {"forward_profile": [float(x) for x in prof[+1]], "backward_profile": [float(x) for x in prof[-1]],
               "predicted_work": {int(k): float(v) for k, v in costs.items()}, "probe_seconds": time.time() - t0}


def cut_profiles(tr, direction, cap, backend="gpu"):
    """States of each weight <= cap at every cut (array (N + 1, cap + 1))."""
    sw = Sweep(tr, direction, cap, cap, use_h=False, backend=backend)
    c0, tab = sw.first()
    out = np.zeros((tr.N + 1, cap + 1))
    out[c0, 0] = 1
    for c, tab, _, _ in sw._walk(c0, tab, tr.N if direction > 0 else 0):
        out[c] = _hist(sw.be, tab)[:cap + 1]
    return out


def probe_profiles(tr, backend="gpu", probe=3, budget=2e9):
    """Per-cut state counts of each weight in both directions, up to weight `probe` (or 2 where the
    weight-3 states, estimated from weights 1 and 2, exceed budget): ({+1: arr, -1: arr}, seconds)."""
    t0 = time.time()

    def measured(direction, cap):
        key = ("profile", direction, cap)
        if key not in tr._bd:
            tr._bd[key] = cut_profiles(tr, direction, cap, backend)
        return tr._bd[key]

    prof = {}
    for direction in (+1, -1):
        b = budget[direction] if isinstance(budget, dict) else budget
        p = measured(direction, min(2, probe))
        tot = p.sum(axis=0)
        if probe > 2 and tot[1] > 0 and tot[2] * tot[2] / tot[1] < b:
            p = measured(direction, probe)
        prof[direction] = p
    return prof, time.time() - t0


def choose_schedule(tr, K, backend="gpu", probe=3, budget=2e9, window=100):
    """A non-increasing split a(c) per cut minimising sum_c F_c(<= a-1) + F_c(a-1) + 2 B_c(<= K-a),
    F, B measured up to weight `probe` and extrapolated with the growth of the last two weights over
    a window of cuts; a DP over cuts and values of a (cdist/sparse_dp.py:906-981)."""
    prof, probe_seconds = probe_profiles(tr, backend, probe, budget)

    def wsum(x):
        cs = np.concatenate([[0.0], np.cumsum(x)])
        idx = np.arange(x.size)
        return cs[np.minimum(x.size, idx + window + 1)] - cs[np.maximum(0, idx - window)]

    def extend(p):
        top = p.shape[1] - 1
        if top >= K:
            return p[:, :K + 1]
        hi = wsum(p[:, top])
        lo = wsum(p[:, top - 1]) if top >= 1 else hi
        r = np.maximum(np.where(lo > 0, hi / np.maximum(lo, 1e-300), 1.0), 1.0)
        cols = [p[:, w] for w in range(top + 1)]
        while len(cols) <= K:
            cols.append(cols[-1] * r)
        return np.stack(cols, axis=1)

    F, B = extend(prof[+1]), extend(prof[-1])
    cF, cB = np.cumsum(F, axis=1), np.cumsum(B, axis=1)
    n = tr.N + 1
    cost = np.zeros((n, K + 1))
    for a in range(1, K + 1):
        cost[:, a] = cF[:, a - 1] + F[:, a - 1] + 2 * cB[:, K - a]
    cost[:, 0] = np.inf
    best = np.empty((n, K + 1))
    arg = np.zeros((n, K + 1), dtype=np.int64)
    best[0] = cost[0]
    for c in range(1, n):
        prev = best[c - 1]
        suf = np.minimum.accumulate(prev[::-1])[::-1]
        sarg = np.empty(K + 1, dtype=np.int64)
        m, ai = np.inf, K
        for a in range(K, -1, -1):
            if prev[a] < m:
                m, ai = prev[a], a
            sarg[a] = ai
        best[c] = cost[c] + suf
        arg[c] = sarg
    a = int(np.argmin(best[n - 1]))
    sched = [0] * n
    for c in range(n - 1, -1, -1):
        sched[c] = a
        if c:
            a = int(arg[c, a])
    idx = np.arange(n)
    av = np.array(sched)
    fwd = cF[idx, av - 1] + F[idx, av - 1]
    bwd = cB[idx, K - av]
    every = max(1, int(math.isqrt(tr.N)))
    ck = (idx % every == 0) | (idx == 0) | (idx == n - 1)
    seg = np.add.reduceat(bwd, np.arange(0, n, every)).max()
    states = bwd[ck].sum() + seg + cF[idx, av - 1][ck].sum() + 4 * max(fwd.max(), bwd.max())
    uniform = {a: float(cost[:, a].sum()) for a in range(1, K + 1)}
    return sched, {"predicted_work": float(best[n - 1].min()), "uniform_predicted_work": uniform,
                   "predicted_peak_states": float(max(fwd.max(), bwd.max())),
                   "predicted_mean_states": float((fwd.sum() + bwd.sum()) / (2 * n)),
                   "predicted_bytes": float(8 * states), "schedule": _runs(sched),
                   "forward_profile": prof[+1].sum(axis=0).tolist(),
                   "backward_profile": prof[-1].sum(axis=0).tolist(), "probe_seconds": probe_seconds}


# ---------------------------------------------------------------------- one query at one threshold
def query(tr, K, mode="mitm", split=None, use_h=True, witness=True, lower=0, every=None, backend="gpu",
          dense=None, dense_max=1 << 30, log=None, max_states=None, deadline=None):
    """Least weight of a solution of the trellis' query if it is <= K (else None), with per-cut
    statistics and a witness (cdist/sparse_dp.py:985-1095).  mode "forward": one sweep keeping
    weights <= K.  mode "mitm": a backward sweep keeping weights <= K - a(c), then a forward sweep
    keeping weights <= a(c) - 1 whose new or improved states are joined with the backward table at
    every cut (and the whole table where a drops).  split: int, "auto", "schedule" or a list of
    N + 1 non-increasing values (default K // 2 + 1)."""
    t0 = time.time()
    bname = backend if isinstance(backend, str) else backend.name
    rec = {"K": K, "mode": mode, "use_h": bool(use_h), "value": None, "witness": None, "width": max(tr.width),
           "backend": bname}

    def new_be():
        return BACKENDS[backend](tr) if isinstance(backend, str) else backend.__class__(tr)

    be = new_be()
    if mode == "forward":
        fw = Sweep(tr, +1, K, K, use_h, every, backend=be, max_states=max_states, deadline=deadline)
        fw.run()
        tab = fw.ckpt[tr.N]
        rec.update(forward_counts=fw.counts, peak_states=fw.peak, peak_table_bytes=fw.peak_bytes,
                   sweep_seconds=time.time() - t0, steps=fw.steps_done, dense_cuts=fw.dense_cuts)
        v = be.lookup(tab, 0)
        if v != INF:
            rec["value"] = v
            if witness:
                t1 = time.time()
                rec["witness"] = sorted(fw.traceback(tr.N, 0, v))
                rec["traceback_seconds"] = time.time() - t1
        rec["seconds"] = time.time() - t0
        return rec
    predicted = None
    if split == "auto":
        split, rec["split_choice"] = choose_split(tr, K, backend=new_be() if isinstance(backend, str) else backend)
        predicted = rec["split_choice"]["predicted_work"][split]
    elif split == "schedule":
        split, rec["split_choice"] = choose_schedule(tr, K, backend=new_be() if isinstance(backend, str) else backend)
        predicted = rec["split_choice"]["predicted_work"]
    if split is None:
        split = K // 2 + 1
    sched = [max(1, min(int(x), K)) for x in split] if isinstance(split, (list, tuple)) else \
        [max(1, min(int(split), K))] * (tr.N + 1)
    assert len(sched) == tr.N + 1 and all(x >= y for x, y in zip(sched, sched[1:])), "split must not increase"
    bw = Sweep(tr, -1, K, use_h=use_h, every=every, backend=be, max_states=max_states, deadline=deadline,
               caps=[K - x for x in sched])
    fw = Sweep(tr, +1, K, use_h=use_h, every=bw.every, frontier=True, backend=new_be(), max_states=max_states,
               deadline=deadline, caps=sched)
    if log:
        log("K=%d split a=%s: backward sweep (weights <= %s)%s" % (
            K, _runs(sched), _runs([K - x for x in sched]), "" if predicted is None else
            ", predicted work %.3g" % predicted))
    bw.run()
    t1 = time.time()
    best = [None]
    cache = {}
    joins = [0]

    def join(c, tab, ch, extra):
        for part in (ch, extra):
            if part is None:
                continue
            if not isinstance(part, _Changed) and isinstance(fw.be, GpuTables):
                part = _Changed(part.arr, part.n)
            if not fw.be.changed_size(part):
                continue
            joins[0] += fw.be.changed_size(part)
            r = fw.be.join(part, bw.table(c, cache), tr.tmask[c])
            if r is not None and (best[0] is None or r[0] < best[0][0]):
                best[0] = (r[0], c) + tuple(r[1:])
        return best[0] is not None and best[0][0] <= max(lower, 0)

    if isinstance(fw.be, GpuTables) and isinstance(bw.be, GpuTables):
        # device walks: the joins of every cut run inside the walk calls
        _, b = fw._run_walk(join_with=bw, lower=lower)
        joins[0] = int(sum(fw.changed_counts))
        if b is not None:
            total, c, fkey = b
            bkey = fkey ^ (int(tr.tmask[c]) & KEYMASK)
            bval = bw.be.lookup(bw.table(c, cache), bkey)
            best[0] = (total, c, fkey, total - bval, bkey)
    else:
        fw.run(on_cut=join)
    cache.clear()
    rec.update(forward_counts=fw.counts, backward_counts=bw.counts, changed_counts=fw.changed_counts,
               peak_states=max(fw.peak, bw.peak), peak_table_bytes=fw.peak_bytes + bw.peak_bytes,
               backward_seconds=t1 - t0, forward_seconds=time.time() - t1,
               split=sched[0] if len(set(sched)) == 1 else _runs(sched), split_values=sched, joined=joins[0],
               steps=fw.steps_done + bw.steps_done, dense_cuts=bw.dense_cuts)
    if best[0] is not None and best[0][0] <= K:
        value, c, sl, fl, sr = best[0]
        rec["value"], rec["join_cut"] = value, c
        if witness:
            t2 = time.time()
            cols = fw.traceback(c, sl, fl) + bw.traceback(c, sr, value - fl)
            rec["witness"] = sorted(cols)
            rec["traceback_seconds"] = time.time() - t2
    rec["seconds"] = time.time() - t0
    return rec


def _runs(x):
    """A per-cut list as 'value' or 'value@cut,value@cut,...' where it changes."""
    out = [(v, c) for c, v in enumerate(x) if c == 0 or v != x[c - 1]]
    return str(out[0][0]) if len(out) == 1 else ",".join("%d@%d" % vc for vc in out)


# ---------------------------------------------------------------------- distance
def default_order(p):
    from . import auto
    return auto.best_order(p)[0]


def plan_trellises(p, order=None):
    """Host planning of distance(): the order and every observable's trellis with its lookahead
    data (no GPU; picklable, so it can run in a worker process)."""
    order = default_order(p) if order is None else order
    trs = [Trellis.for_query(p, i, order) for i in range(p.nobs)]
    # the lookahead data of both directions of every trellis: the library's routine releases the
    # interpreter, so the directions run side by side
    jobs = [(t, fwd) for t in trs if t.feasible for fwd in (True, False)]
    if len(jobs) > 1:
        from concurrent.futures import ThreadPoolExecutor
        with ThreadPoolExecutor(min(len(jobs), 8)) as ex:
            list(ex.map(lambda j: j[0].bound_raw(j[1]), jobs))
    else:
        for t, fwd in jobs:
            t.bound_raw(fwd)
    return trs


def distance(p, order=None, start=1, kmax=64, mode="mitm", use_h=True, witness=True, log=None, every=None,
             backend="gpu", dense=None, split=None, trellises=None):
    """Exact distance by iterative deepening of K from `start` (a lower bound): a dict with the
    distance (None if none <= kmax), a checked witness and one record per (threshold, observable)
    (cdist/sparse_dp.py:1110-1151).  trellises: the result of plan_trellises, if planned ahead."""
    t0 = time.time()
    if trellises is not None:
        trs = trellises
    else:
        order = default_order(p) if order is None else order
        trs = [Trellis.for_query(p, i, order) for i in range(p.nobs)]
    out = {"distance": None, "witness": None, "runs": [], "lower_bound": start,
           "order_cut_rank": max((max(t.width) for t in trs if t.feasible), default=0)}
    for K in range(start, kmax + 1):
        best = None
        for i, tr in enumerate(trs):
            if not tr.feasible:
                continue
            r = query(tr, K, mode=mode, use_h=use_h, witness=witness, lower=K, every=every, backend=backend,
                      dense=dense, split=split(K) if callable(split) else split)
            r["obs"] = i
            out["runs"].append(summary(r))
            if log:
                log("  K=%d obs %d: value %s peak %d states %.2fs" % (K, i, r["value"], r["peak_states"], r["seconds"]))
            if r["value"] is not None and (best is None or r["value"] < best["value"]):
                best = r
                if r["value"] <= K:
                    break
        if best is not None:
            out["distance"] = best["value"]
            if witness:
                cols = best["witness"]
                s = lg = 0
                for j in cols:
                    s ^= p.h[j]
                    lg ^= p.l[j]
                wt = len(cols) if getattr(p, "weights", None) is None else sum(p.weights[j] for j in cols)
                assert s == 0 and lg != 0 and wt == best["value"] and len(cols) == len(set(cols)), \
                    "witness check failed"
                out["witness"] = cols
            break
        out["lower_bound"] = K + 1
    out["seconds"] = time.time() - t0
    return out


def summary(r):
    """A query record without the per-cut arrays (their totals instead)."""
    out = {k: v for k, v in r.items() if not k.endswith("_counts") and k not in ("witness", "split_values")}
    for k in ("forward_counts", "backward_counts", "changed_counts"):
        if k in r:
            out[k.replace("_counts", "_states_total")] = int(sum(r[k]))
    return out
