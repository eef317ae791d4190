"""Weight-truncated sparse Rank DP on device tables (drop-in for cdist/sparse_dp.py).

The public names and records are the reference's: Trellis, Sweep, query, distance, summary,
choose_split, choose_schedule, BACKENDS, BudgetExceeded (cdist/sparse_dp.py:63-1160), so a caller
of the reference's sparse DP can switch to this module; the tables live on the GPU
(tropidist_gb300/sparse_tables.py).

How a query runs here.
  Trellis    the query's rows in minimal span form with a fixed slot per row (interval colouring,
             the slot assignment of cdist/sparse_dp.py:85-99, so a state means the same in both
             directions and the tables equal the reference's as sets), per position the column's
             slot mask and the closing rows, per cut the active rows, the target row's slot and the
             lookahead classes (a C++ routine of the library).  States may be wider than one
             machine word (up to 512 slots): the reference stops at 64.
  Sweep      one direction of the truncated sweep.  A sweep advances in *legs*: runs of consecutive
             steps that the backend executes in one call where it can (GpuTables.walk: a whole
             checkpoint interval or several on the device, the tables it keeps copied into an
             arena) and one step per call otherwise.  It keeps its tables at every isqrt(N)-th cut
             (checkpoints) and every small table (at most 1024 states, within a byte budget), and
             recomputes any other table from the checkpoint before it in its own direction.
  query      forward mode: one sweep keeping weights <= K, the value is the final table's state 0.
             Meet in the middle: a backward sweep keeping weights <= K - a(c), then a forward
             sweep keeping weights <= a(c) - 1 whose new or improved states (and, where a(c)
             drops, the whole table before the drop) are joined at every cut with the backward
             table of that cut: the least total over all cuts is the value; the witness comes from
             the two tracebacks.
  distance   iterative deepening of the threshold over the observables.
The split a(c) only affects the speed: by default K // 2 + 1 everywhere; "auto" picks one value
and "schedule" one per cut from weight profiles measured by cheap sweeps (a cost model of states
stepped, written for this implementation).
"""
from __future__ import annotations

import heapq
import math
import time

import numpy as np

from . import _lib, trellis
from .sparse_tables import (INF, KEYMASK, M64, MAX_SLOTS, MAX_WIDE_SLOTS, BudgetExceeded, GpuTables,
                            WideGpuTables, _Changed, pad_words, words_of)

MAX_WEIGHT = INF - 1
Q = 720720                      # lcm(1..16): lookahead weights are multiples of 1/Q (rounded down)
U64 = np.uint64

BACKENDS = {"gpu": GpuTables, "gpu-wide": WideGpuTables}


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
        if nslots > MAX_WIDE_SLOTS:
            raise ValueError("trellis needs %d bits per state (at most %d supported)" % (nslots, MAX_WIDE_SLOTS))
        self.slot, self.nslots = slot, nslots
        self.words = max(1, (nslots + 63) // 64)     # uint64 words of a state
        nr = len(rows)
        # positions of every row (CSR), and per position the slots of the rows through it
        self.row_ptr, self.row_cols = trellis.bit_positions(rows, N)
        entry_row = np.repeat(np.arange(nr, dtype=np.int64), np.diff(self.row_ptr))
        if self.words == 1:
            sbit = np.left_shift(np.uint64(1), np.asarray(slot, dtype=np.uint64))
            colm = np.zeros(max(1, N), dtype=U64)
            np.bitwise_or.at(colm, self.row_cols, sbit[entry_row])
            self.col = colm[:N].tolist()
        else:                                          # masks beyond one word: Python ints
            col = [0] * N
            ptr = self.row_ptr.tolist()
            cols = self.row_cols.tolist()
            for r in range(nr):
                b = 1 << slot[r]
                for q in range(ptr[r], ptr[r + 1]):
                    col[cols[q]] |= b
            self.col = col
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
        if self.words == 1:
            delta = np.zeros(N + 2, dtype=U64)
            np.bitwise_xor.at(delta, st + 1, sbit)
            np.bitwise_xor.at(delta, en + 1, sbit)
            act_mask = np.bitwise_xor.accumulate(delta)[:N + 1]
            self.active = act_mask.tolist()
        else:
            delta = [0] * (N + 2)
            for r in range(nr):
                b = 1 << slot[r]
                delta[self.start[r] + 1] ^= b
                delta[self.end[r] + 1] ^= b
            acc, active = 0, []
            for c in range(N + 1):
                acc ^= delta[c]
                active.append(acc)
            self.active = active
        self.width = np.diff(self.act_ptr).tolist()
        lbit = 1 << slot[self.L]         # the target row's own interval (its slot is shared over time)
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
        maxc, W = 48, self.words
        ncls = np.zeros(N + 1, dtype=np.int32)
        masks = np.zeros((N + 1, maxc, W), dtype=U64)
        wts = np.zeros((N + 1, maxc), dtype=np.int64)
        extra = np.zeros(N + 1, dtype=np.int64)
        ptr = lambda a: a.ctypes.data if a.size else None
        _lib.check(_lib.lib().tg_sp_bound_data_wide(N, nr, ptr(row_ptr), ptr(row_cols), ptr(col_ptr), ptr(col_rows),
                                                    ptr(act_ptr), ptr(act_rows), ptr(start), ptr(end), ptr(slot),
                                                    self.L, int(bool(forward)), maxc, W, ptr(ncls), ptr(masks),
                                                    ptr(wts), ptr(extra)))
        k = max(1, int(ncls.max()) if ncls.size else 1)
        masks = masks[:, :k, 0] if W == 1 else masks[:, :k, :]
        return ncls, masks.copy(), wts[:, :k].copy(), extra

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
            wrap = U64 if self.words == 1 else int
            out.append((tuple(wrap(masks[k]) for k in ks), tuple(np.int64(k) for k in ks), extra))
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


def _backend(backend, tr):
    """A backend object: a name of BACKENDS ("gpu" takes the wide tables when the states need more
    than 56 slots) or an object with the table-backend interface."""
    if not isinstance(backend, str):
        return backend
    if backend == "gpu" and tr.nslots > MAX_SLOTS:
        backend = "gpu-wide"
    return BACKENDS[backend](tr)


def _fresh(backend, tr):
    """Another backend object of the same kind (one per sweep: a backend may reuse its buffers)."""
    return _backend(backend, tr) if isinstance(backend, str) else backend.__class__(tr)


def _as_changed(be, tab):
    """The start table as a `changed` object of the backend (joined in full at the first cut)."""
    if isinstance(be, GpuTables):
        return _Changed(tab.arr, tab.n)
    return tab


def _values(be, tab, keys):
    """The values of several states in one table (one device round trip where the backend can)."""
    if hasattr(be, "lookup_many"):
        return [int(x) for x in be.lookup_many(tab, keys)]
    return [be.lookup(tab, k) for k in keys]


# ---------------------------------------------------------------------- sweeps
class Sweep:
    """One direction of the truncated sweep of a trellis.  direction +1 runs cuts 0 -> N from the
    table {0: 0} at cut 0, -1 runs N -> 0.  The table at cut c keeps weights <= caps[c] (cap for all
    cuts, or a per-cut list that does not grow in the sweep direction; at most 254, the 8-bit
    values).  use_h: drop states whose weight plus the lookahead bound exceeds K.  frontier (forward
    sweep of a meet in the middle): the step out of cut p keeps weights <= caps[p] - 1 and reports
    its new or improved states of weight <= caps[p] as `changed`; where caps drops, the table before
    the drop is reported as `extra`.  max_states / deadline (time.monotonic) raise BudgetExceeded.
    dense / dense_max are accepted for the reference's signature; the device tables need no dense
    form.  After run(): ckpt (cut -> table), counts and changed_counts per cut, peak (the most
    states of one table or changed set), peak_bytes, steps_done."""

    RUN_STEPS = 4096                # steps per device leg of a sweep that joins nothing ...
    LEG_ARENA_BYTES = 4 << 30       # ... while the tables a leg keeps took at most this many bytes
    SMALL_STATES = 1024             # tables this small are kept at every cut ...
    SMALL_KEEP_BYTES = 256 << 20    # ... within this many bytes

    def __init__(self, tr, direction, K, cap=None, use_h=True, every=None, frontier=False, backend="gpu",
                 dense=None, dense_max=1 << 30, max_states=None, deadline=None, caps=None):
        self.tr, self.direction, self.K = tr, direction, K
        if caps is None:
            caps = [cap] * (tr.N + 1)
        self.caps = [min(int(x), K) for x in caps]
        if max(self.caps) > MAX_WEIGHT:
            raise ValueError("a sweep keeping weights up to %d: the tables hold at most %d (8-bit values)"
                             % (max(self.caps), MAX_WEIGHT))
        later = self.caps[1:] if direction > 0 else self.caps[:-1]
        earlier = self.caps[:-1] if direction > 0 else self.caps[1:]
        assert all(b <= a for a, b in zip(earlier, later)), "caps must not grow in the sweep direction"
        self.use_h, self.frontier = use_h, frontier
        self.be = _backend(backend, tr)
        self.on_device = isinstance(self.be, GpuTables)
        self.legs = self.on_device or isinstance(self.be, WideGpuTables)    # steps run as device walks
        self.hd = tr.bound_arrays(direction > 0) if use_h else None
        self.every = every or max(1, int(math.isqrt(tr.N)))
        self.max_states, self.deadline = max_states, deadline
        self.ckpt = {}
        self.small_tabs, self.small_bytes = {}, 0
        self.counts = [0] * (tr.N + 1)
        self.changed_counts = [0] * (tr.N + 1)
        self.peak = self.peak_bytes = self.steps_done = self.dense_cuts = 0
        self._held_bytes = 0
        self._spec = None

    # ------------------------------------------------------------------ geometry
    def start_cut(self):
        return 0 if self.direction > 0 else self.tr.N

    def end_cut(self):
        return self.tr.N if self.direction > 0 else 0

    def first(self):
        return self.start_cut(), self.be.start()

    def is_ckpt(self, c):
        return c % self.every == 0 or c == 0 or c == self.tr.N

    def _positions(self, c, stop):
        """The step positions that take the table from cut c to cut stop."""
        return list(range(c, stop)) if self.direction > 0 else list(range(c - 1, stop - 1, -1))

    def _cut_of(self, p):
        return p + 1 if self.direction > 0 else p

    def _next_ckpt(self, c, stop):
        if self.direction > 0:
            return min(stop, (c // self.every + 1) * self.every)
        return max(stop, (c - 1) // self.every * self.every)

    def _from_ckpt(self, c):
        """The checkpoint from which the table at cut c is recomputed (at or before c in the sweep
        direction)."""
        if self.direction > 0:
            return max(x for x in self.ckpt if x <= c)
        return min(x for x in self.ckpt if x >= c)

    # ------------------------------------------------------------------ one step
    def _step(self, tab, p, want_changed):
        """The step at position p: (new cut, table, changed, extra)."""
        tr, fwd = self.tr, self.direction > 0
        cut = self._cut_of(p)
        sm, sb = (tr.fsel_mask[p], tr.fsel_bits[p]) if fwd else (tr.bsel_mask[p], tr.bsel_bits[p])
        cap, kb = (self.caps[p], self.caps[p]) if self.frontier else (self.caps[cut], None)
        kw = {} if tr.cw[p] == 1 else {"w": tr.cw[p]}
        self.steps_done += 1
        tab, ch = self.be.step(tab, tr.col[p], sm, sb, cap, self.K, tr.tmask[cut],
                               self.hd[cut] if self.hd else None, kb, want_changed, **kw)
        if self.frontier and self.caps[cut] < cap:
            return cut, self.be.truncate(tab, self.caps[cut]), ch, tab
        return cut, tab, ch, None

    def _note(self, c, tab, ch):
        """Per-cut bookkeeping of a step's result: counts, peaks, the tables kept, budgets."""
        n = self.be.size(tab)
        nc = self.be.changed_size(ch) if ch is not None else 0
        self.counts[c], self.changed_counts[c] = n, nc
        self.peak = max(self.peak, n, nc)
        if self.is_ckpt(c):
            self.ckpt[c] = self.be.persistent(tab)
            self._held_bytes += self.be.nbytes(tab)
        self.peak_bytes = max(self.peak_bytes, self._held_bytes + self.be.nbytes(tab))
        if self.max_states is not None and max(n, nc) > self.max_states:
            raise BudgetExceeded("%d states at cut %d" % (max(n, nc), c), "states")
        if self.deadline is not None and time.monotonic() > self.deadline:
            raise BudgetExceeded("deadline at cut %d" % c, "deadline")

    def _begin(self):
        c0, tab = self.first()
        self.ckpt[c0] = tab
        self.counts[c0] = self.changed_counts[c0] = 1
        self.peak = 1
        self._held_bytes = self.be.nbytes(tab)
        return c0, tab

    # ------------------------------------------------------------------ whole sweeps
    def run(self, on_cut=None):
        """The whole sweep, keeping checkpoints and per-cut counts; on_cut(cut, table, changed,
        extra) may return True to stop.  Returns the last cut reached."""
        if on_cut is None and self.legs:
            return self._device_legs()[0]
        c, tab = self._begin()
        if on_cut and on_cut(c, tab, _as_changed(self.be, tab), None):
            return c
        for p in self._positions(c, self.end_cut()):
            c, tab, ch, extra = self._step(tab, p, on_cut is not None)
            self._note(c, tab, ch)
            if on_cut and on_cut(c, tab, ch, extra):
                return c
        return c

    def meet(self, back, lower=0):
        """The forward (frontier) sweep of a meet in the middle against the finished backward sweep
        `back`: the least (total, cut, forward state, forward value, backward state) over every
        cut's joins, or None; it stops early once a total <= lower is found."""
        if self.legs and back.legs:
            return self._device_meet(back, lower)
        tr = self.tr
        best = [None]
        store = _TablesAt(back)

        def join(c, part):
            if part is None or not self.be.changed_size(part):
                return
            self.joined += self.be.changed_size(part)
            r = self.be.join(part, store.at(c), tr.tmask[c])
            if r is not None and (best[0] is None or r[0] < best[0][0]):
                best[0] = (r[0], c) + tuple(r[1:])

        c, tab = self._begin()
        self.joined = 0
        join(c, _as_changed(self.be, tab))
        for p in self._positions(c, self.end_cut()):
            if best[0] is not None and best[0][0] <= max(lower, 0):
                break
            c, tab, ch, extra = self._step(tab, p, True)
            self._note(c, tab, ch)
            join(c, ch)
            if extra is not None:
                join(c, extra if not isinstance(self.be, GpuTables) else _Changed(extra.arr, extra.n))
        return best[0]

    # ------------------------------------------------------------------ device legs (walks)
    def _device_meet(self, back, lower):
        store = _TablesAt(back)
        _, b = self._device_legs(join_with=store, lower=lower)
        self.joined = int(sum(self.changed_counts))
        if b is None:
            return None
        total, c, fkey = b
        bkey = fkey ^ (int(self.tr.tmask[c]) & KEYMASK if self.on_device else int(self.tr.tmask[c]))
        bval = back.be.lookup(store.at(c), bkey)
        return total, c, fkey, total - bval, bkey

    def _device_legs(self, join_with=None, lower=0):
        """The sweep as device legs (one per checkpoint interval when joining, else up to RUN_STEPS
        steps); join_with: a _TablesAt of the backward sweep.  Returns (last cut, best join
        (total, cut, forward key) or None)."""
        c, tab = self._begin()
        best = None
        if join_with is not None:
            r = self.be.join(_as_changed(self.be, tab), join_with.at(c), self.tr.tmask[c])
            if r is not None:
                best = (r[0], c, r[1])
        stop = self.end_cut()
        while c != stop and not (best is not None and best[0] <= max(lower, 0)):
            c1 = self._next_ckpt(c, stop)
            if join_with is None:
                # one checkpoint interval per leg once the kept tables are large (a leg's kept
                # tables share one arena allocation)
                big = getattr(self.be, "_arena_guess", 0) > self.LEG_ARENA_BYTES
                while c1 != stop and abs(c1 - c) < self.RUN_STEPS and not big:
                    c1 = self._next_ckpt(c1, stop)
            pos = self._positions(c, c1)
            cuts = [self._cut_of(p) for p in pos]
            small = 2 if self.small_bytes < self.SMALL_KEEP_BYTES else 0
            keep = [1 if self.is_ckpt(x) else small for x in cuts]
            keep[-1] = 1
            joins = None                 # the last leg's backward tables are not held while the next are built
            joins = None if join_with is None else [(join_with.at(x), self.tr.tmask[x]) for x in cuts]
            out, kept, res = self.be.walk(tab, *self._rows(pos, keep, joins), self.K, self.max_states,
                                          want_res=join_with is not None)
            self.steps_done += len(pos)
            for x, a, b in zip(cuts, out[:, 0].tolist(), out[:, 1].tolist()):
                self.counts[x], self.changed_counts[x] = a, b
            self.peak = max(self.peak, int(out[:, [0, 1]].max()))
            if join_with is not None:
                r = self._walk_best(res)
                if r is not None and (best is None or r[1] < best[0]):
                    best = (r[1], cuts[r[0]], r[2])
            for k, t in kept.items():
                if keep[k] == 1 and k != len(pos) - 1:
                    self.ckpt[cuts[k]] = t
                    self._held_bytes += self.be.nbytes(t)
                elif keep[k] == 2:
                    self.small_tabs[cuts[k]] = t
                    self.small_bytes += self.be.nbytes(t) + 8 * (1 << t.lg) + 256
            tab = kept[len(pos) - 1]
            c = c1
            self.ckpt[c] = tab
            self._held_bytes += self.be.nbytes(tab)
            self.peak_bytes = max(self.peak_bytes, self._held_bytes + self.be.state_bytes * int(out[:, 5].max()))
            if self.max_states is not None and self.peak > self.max_states:
                raise BudgetExceeded("%d states before cut %d" % (self.peak, c), "states")
            if self.deadline is not None and time.monotonic() > self.deadline:
                raise BudgetExceeded("deadline at cut %d" % c, "deadline")
        return c, best

    def _walk_best(self, res):
        """The first least join total of a walk: (step, total, forward key) or None."""
        if not self.on_device:
            return self.be.walk_best(res)
        hit = np.nonzero(res != U64(0xFFFFFFFFFFFFFFFF))[0]
        if not len(hit):
            return None
        k = int(hit[np.argmin(res[hit] >> U64(56))])
        return k, int(res[k]) >> 56, int(res[k]) & KEYMASK

    def _rows(self, positions, keep, joins=None):
        """Spec rows of tg_sp_walk for the steps at `positions` (as _step), with lookahead arrays;
        keep: per step 0/1; joins: per step None or (backward table, tmask)."""
        if not self.on_device:
            return self._wide_rows(positions, keep, joins)
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

    def _wide_rows(self, positions, keep, joins=None):
        """Step records of tg_spw_walk (multi-word states) for the steps at `positions`:
        (steps int64 [m, 13], words uint64 [m, 5, W], lookahead masks, weights)."""
        if getattr(self, "_all", None) is None:
            self._all = self._all_wide()
        steps0, words0, masks0, weights0 = self._all
        pos = np.asarray(positions, dtype=np.int64)
        steps, words = steps0[pos].copy(), words0[pos].copy()
        steps[:, 4] = np.asarray(keep, dtype=np.int64)
        if joins is not None:
            W = self.be.W
            for k, j in enumerate(joins):
                if j is None:
                    continue
                t, tmask = j
                steps[k, 5] = 1
                steps[k, 9], steps[k, 10] = t.keys.data_ptr(), t.H.data_ptr()
                steps[k, 11], steps[k, 12] = t.lg, t.stride
                words[k, 4] = words_of(tmask, W)
        return steps, words, masks0[pos], weights0[pos]

    def _all_wide(self):
        """Step records of every step position of this sweep for tg_spw_walk (without keep / join)."""
        tr, fwd, W = self.tr, self.direction > 0, self.be.W
        N = tr.N
        steps = np.zeros((max(1, N), 13), dtype=np.int64)
        words = np.zeros((max(1, N), 5, W), dtype=U64)
        if N == 0:
            return steps, words, np.zeros((1, 1, W), dtype=U64), np.zeros((1, 1), dtype=np.int64)
        p = np.arange(N)
        cut = p + 1 if fwd else p
        caps = np.asarray(self.caps, dtype=np.int64)
        cap = caps[cut].copy()
        kb = np.full(N, -1, dtype=np.int64)
        trunc = np.full(N, -1, dtype=np.int64)
        if self.frontier:
            cap = caps[p].copy()
            kb = cap.copy()
            drop = caps[cut] < cap
            trunc[drop] = caps[cut][drop]
        steps[:, 0], steps[:, 1], steps[:, 3] = cap, kb, trunc
        steps[:, 2] = np.asarray(tr.cw, dtype=np.int64)

        def wv(xs):
            xs = [int(x) for x in xs]
            return np.array([[(x >> (64 * i)) & M64 for i in range(W)] for x in xs], dtype=U64).reshape(len(xs), W)
        sm, sb = (tr.fsel_mask, tr.fsel_bits) if fwd else (tr.bsel_mask, tr.bsel_bits)
        words[:, 0], words[:, 1], words[:, 2] = wv(tr.col), wv(sm), wv(sb)
        words[:, 3] = words[:, 4] = wv(tr.tmask)[cut]
        if self.use_h:
            ncls, masks, wts, extra = tr.bound_raw(fwd)
            masks = np.asarray(masks, dtype=U64)
            if masks.ndim == 2:
                masks = masks[:, :, None]
            steps[:, 6], steps[:, 7], steps[:, 8] = ncls[cut], 1, extra[cut]
            return steps, words, pad_words(masks[cut], W), np.ascontiguousarray(wts[cut])
        return steps, words, np.zeros((N, 1, W), dtype=U64), np.zeros((N, 1), dtype=np.int64)

    # ------------------------------------------------------------------ recomputed tables
    def tables(self, lo, hi):
        """The tables at the cuts lo..hi (lo <= hi), recomputed from the checkpoint before them in
        the sweep direction: {cut: table}."""
        fwd = self.direction > 0
        c0 = self._from_ckpt(lo if fwd else hi)
        stop = hi if fwd else lo
        out = {}
        tab = self.ckpt[c0]
        if lo <= c0 <= hi:
            out[c0] = tab
        pos = self._positions(c0, stop)
        if not pos:
            return out
        if self.legs:
            keep = [1 if lo <= self._cut_of(p) <= hi else 0 for p in pos]
            _, kept, _ = self.be.walk(tab, *self._rows(pos, keep), self.K, self.max_states, want_res=False)
            for k, p in enumerate(pos):
                if keep[k]:
                    out[self._cut_of(p)] = kept[k]
            return out
        for p in pos:
            c, tab, _, _ = self._step(tab, p, False)
            if lo <= c <= hi:
                out[c] = self.be.persistent(tab)
        return out

    segment = tables

    def traceback(self, cut, state, value):
        """Columns (problem indices) of a partial solution that reaches `state` with weight `value`
        at `cut`: walking back to the sweep's start one checkpoint interval at a time, a step used
        its column unless the table before it already holds the state (closing rows restored) with
        the same weight."""
        tr, fwd = self.tr, self.direction > 0
        sel = tr.fsel_bits if fwd else tr.bsel_bits
        used, s, v = [], int(state), int(value)
        c = cut
        while c != self.start_cut():
            if fwd:
                lo = self._from_ckpt(c - 1)
                tabs = self.tables(lo, c - 1)
                steps = [(p, tabs[p]) for p in range(c - 1, lo - 1, -1)]
                c = lo
            else:
                hi = self._from_ckpt(c + 1)
                tabs = self.tables(c + 1, hi)
                steps = [(p, tabs[p + 1]) for p in range(c, hi)]
                c = hi
            for p, before in steps:
                mid = s | sel[p]
                without, with_col = _values(self.be, before, [mid, mid ^ tr.col[p]])
                if without == v:
                    s = mid
                    continue
                assert tr.col[p] and with_col == v - tr.cw[p], "traceback lost the path"
                used.append(tr.order[p])
                s, v = mid ^ tr.col[p], v - tr.cw[p]
        assert s == 0 and v == 0, (s, v)
        return used


class _TablesAt:
    """The tables of a finished sweep at the cuts that the opposite sweep asks for, in that sweep's
    order: kept tables directly, any other from one recomputed checkpoint interval (cached)."""

    def __init__(self, sweep):
        self.sweep = sweep
        self.span, self.cache = None, {}

    def at(self, c):
        sw = self.sweep
        t = sw.small_tabs.get(c)
        if t is None:
            t = sw.ckpt.get(c)
        if t is not None:
            return t
        if c not in self.cache:
            base = sw._from_ckpt(c)
            self.cache = {}              # the interval held so far is released before the next one is built
            self.cache = sw.tables(min(c, base), max(c, base)) if sw.direction < 0 else sw.tables(base, c)
        return self.cache[c]


# ---------------------------------------------------------------------- choice of the split
def _hist(be, tab):
    if hasattr(be, "hist"):
        return np.asarray(be.hist(tab), dtype=np.float64)
    return np.bincount(np.asarray(be.arrays(tab)[1], dtype=np.uint8), minlength=256).astype(np.float64)


def weight_profiles(tr, cap, backend="gpu"):
    """Per direction (+1, -1) and cut, the number of states of each weight <= cap in a sweep that
    keeps weights <= cap without the lookahead: {direction: array (N + 1, cap + 1)}."""
    out = {}
    for d in (+1, -1):
        sw = Sweep(tr, d, cap, cap, use_h=False, backend=_fresh(backend, tr))
        prof = np.zeros((tr.N + 1, cap + 1))
        c, tab = sw.first()
        prof[c, 0] = 1
        for p in sw._positions(c, sw.end_cut()):
            c, tab, _, _ = sw._step(tab, p, False)
            prof[c] = _hist(sw.be, tab)[:cap + 1]
        out[d] = prof
    return out


def _measured_profiles(tr, backend, probe, budget):
    """Weight profiles up to `probe`, or up to 2 where the states of weight 3, guessed from the
    growth between weights 1 and 2, would pass `budget` (cached on the trellis)."""
    t0 = time.time()
    key = ("profiles", 2)
    if key not in tr._bd:
        tr._bd[key] = weight_profiles(tr, 2, backend)
    prof = tr._bd[key]
    if probe > 2:
        tot = {d: prof[d].sum(axis=0) for d in prof}
        guess = max((t[2] * t[2] / t[1]) if t[1] > 0 else 0.0 for t in tot.values())
        if guess < budget:
            key = ("profiles", probe)
            if key not in tr._bd:
                tr._bd[key] = weight_profiles(tr, probe, backend)
            prof = tr._bd[key]
    return prof, time.time() - t0


def _extend(prof, K, window):
    """Per-cut profiles extended to weight K: beyond the measured weights each cut grows by the
    ratio of its last two weights, both summed over a window of neighbouring cuts (at least 1)."""
    n, top = prof.shape[0], prof.shape[1] - 1
    if top >= K:
        return prof[:, :K + 1]
    kernel = np.ones(2 * window + 1)
    hi = np.convolve(prof[:, top], kernel, mode="same")
    lo = np.convolve(prof[:, top - 1], kernel, mode="same") if top >= 1 else hi
    growth = np.where(lo > 0, hi / np.where(lo > 0, lo, 1.0), 1.0)
    growth = np.maximum(growth, 1.0)
    extra = prof[:, top:top + 1] * growth[:, None] ** np.arange(1, K - top + 1)[None, :]
    return np.concatenate([prof, extra], axis=1)


def _split_costs(tr, K, backend, probe, budget, window):
    """cost[c, a]: states stepped at cut c with the split a (a = 1..K): the forward sweep's table
    (weights < a) and its changed states (weight a, at most), the backward table (weights <= K - a)
    twice (swept, then recomputed for the joins)."""
    prof, secs = _measured_profiles(tr, backend, probe, budget)
    F = np.cumsum(_extend(prof[+1], K, window), axis=1)
    B = np.cumsum(_extend(prof[-1], K, window), axis=1)
    cost = np.full((tr.N + 1, K + 1), np.inf)
    for a in range(1, K + 1):
        cost[:, a] = F[:, a] + 2 * B[:, K - a]
    return cost, prof, secs


def choose_split(tr, K, backend="gpu", probe=3, budget=2e9, window=100):
    """One split a for every cut (the reference's choose_split, cdist/sparse_dp.py:839-867, with
    this module's cost model): (a, info)."""
    cost, prof, secs = _split_costs(tr, K, backend, probe, budget, window)
    total = cost.sum(axis=0)
    a = int(np.argmin(total))
    return a, {"predicted_work": {int(x): float(total[x]) for x in range(1, K + 1)},
               "forward_profile": prof[+1].sum(axis=0).tolist(),
               "backward_profile": prof[-1].sum(axis=0).tolist(), "probe_seconds": secs}


def choose_schedule(tr, K, backend="gpu", probe=3, budget=2e9, window=100):
    """A split a(c) per cut, not increasing with c, minimising the summed cost (the reference's
    choose_schedule, cdist/sparse_dp.py:906-981, with this module's cost model): a dynamic
    programme over the cuts, best[c][a] = cost[c][a] + min over a' >= a of best[c - 1][a'].
    Returns (schedule, info)."""
    cost, prof, secs = _split_costs(tr, K, backend, probe, budget, window)
    n = tr.N + 1
    idx = np.arange(K + 1)
    best = cost[0].copy()
    choice = np.zeros((n, K + 1), dtype=np.int16)       # the a' taken at c - 1 for each a at c
    for c in range(1, n):
        rev = best[::-1]
        run_min = np.minimum.accumulate(rev)
        at = np.maximum.accumulate(np.where(rev == run_min, idx, 0))
        choice[c] = (K - at)[::-1]
        best = cost[c] + run_min[::-1]
    a = int(np.argmin(best))
    sched = [0] * n
    for c in range(n - 1, -1, -1):
        sched[c] = a
        a = int(choice[c, a])
    uniform = cost.sum(axis=0)
    return sched, {"predicted_work": float(best.min()),
                   "uniform_predicted_work": {int(x): float(uniform[x]) for x in range(1, K + 1)},
                   "schedule": _runs(sched), "forward_profile": prof[+1].sum(axis=0).tolist(),
                   "backward_profile": prof[-1].sum(axis=0).tolist(), "probe_seconds": secs}


def _runs(values):
    """A per-cut list as 'v' when constant, else 'v@cut,...' at every change."""
    marks = [(c, v) for c, v in enumerate(values) if c == 0 or v != values[c - 1]]
    if len(marks) == 1:
        return str(marks[0][1])
    return ",".join("%d@%d" % (v, c) for c, v in marks)


def _schedule(tr, K, split, backend):
    """The split per cut, the predicted work (or None) and the record of the choice."""
    info = None
    predicted = None
    if split == "auto":
        split, info = choose_split(tr, K, backend=backend)
        predicted = info["predicted_work"][split]
    elif split == "schedule":
        split, info = choose_schedule(tr, K, backend=backend)
        predicted = info["predicted_work"]
    if split is None:
        split = K // 2 + 1
    if isinstance(split, (list, tuple)):
        sched = [max(1, min(int(x), K)) for x in split]
    else:
        sched = [max(1, min(int(split), K))] * (tr.N + 1)
    assert len(sched) == tr.N + 1 and all(b <= a for a, b in zip(sched, sched[1:])), "split must not increase"
    return sched, predicted, info


# ---------------------------------------------------------------------- one query at one threshold
def query(tr, K, mode="mitm", split=None, use_h=True, witness=True, lower=0, every=None, backend="gpu",
          dense=None, dense_max=1 << 30, log=None, max_states=None, deadline=None):
    """The least weight of a solution of the trellis' query when it is <= K (else value None),
    with per-cut statistics and a witness (the reference's query, cdist/sparse_dp.py:985-1095).
    mode "forward": one sweep keeping weights <= K.  mode "mitm": a backward sweep keeping weights
    <= K - a(c), then a forward frontier sweep keeping weights <= a(c) - 1, joined at every cut;
    split: None (K // 2 + 1), an int, "auto", "schedule" or N + 1 non-increasing values.  lower: a
    known lower bound (a join reaching it ends the forward sweep)."""
    t0 = time.time()
    rec = {"K": K, "mode": mode, "use_h": bool(use_h), "value": None, "witness": None, "width": max(tr.width),
           "backend": backend if isinstance(backend, str) else backend.name}
    budget = dict(max_states=max_states, deadline=deadline)
    if mode == "forward":
        sw = Sweep(tr, +1, K, K, use_h, every, backend=_fresh(backend, tr), **budget)
        sw.run()
        rec.update(forward_counts=sw.counts, peak_states=sw.peak, peak_table_bytes=sw.peak_bytes,
                   sweep_seconds=time.time() - t0, steps=sw.steps_done, dense_cuts=0)
        v = sw.be.lookup(sw.ckpt[tr.N], 0)
        if v != INF:
            rec["value"] = v
            if witness:
                t1 = time.time()
                rec["witness"] = sorted(sw.traceback(tr.N, 0, v))
                rec["traceback_seconds"] = time.time() - t1
        rec["seconds"] = time.time() - t0
        return rec
    sched, predicted, choice = _schedule(tr, K, split, backend)
    if choice is not None:
        rec["split_choice"] = choice
    back = Sweep(tr, -1, K, use_h=use_h, every=every, backend=_fresh(backend, tr), caps=[K - a for a in sched],
                 **budget)
    ahead = Sweep(tr, +1, K, use_h=use_h, every=back.every, frontier=True, backend=_fresh(backend, tr), caps=sched,
                  **budget)
    if log:
        log("K=%d split %s: backward sweep (weights <= %s)%s" % (
            K, _runs(sched), _runs([K - a for a in sched]),
            "" if predicted is None else ", predicted work %.3g" % predicted))
    back.run()
    t1 = time.time()
    best = ahead.meet(back, lower)
    rec.update(forward_counts=ahead.counts, backward_counts=back.counts, changed_counts=ahead.changed_counts,
               peak_states=max(ahead.peak, back.peak), peak_table_bytes=ahead.peak_bytes + back.peak_bytes,
               backward_seconds=t1 - t0, forward_seconds=time.time() - t1,
               split=sched[0] if len(set(sched)) == 1 else _runs(sched), split_values=sched,
               joined=ahead.joined, steps=ahead.steps_done + back.steps_done, dense_cuts=0)
    if best is not None and best[0] <= K:
        value, c, f_state, f_value, b_state = best
        rec["value"], rec["join_cut"] = value, c
        if witness:
            t2 = time.time()
            cols = ahead.traceback(c, f_state, f_value) + back.traceback(c, b_state, value - f_value)
            rec["witness"] = sorted(cols)
            rec["traceback_seconds"] = time.time() - t2
    rec["seconds"] = time.time() - t0
    return rec


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


def _check_witness(p, cols, value):
    syndrome = logical = 0
    for j in cols:
        syndrome ^= p.h[j]
        logical ^= p.l[j]
    weights = getattr(p, "weights", None)
    weight = len(cols) if weights is None else sum(weights[j] for j in cols)
    assert syndrome == 0 and logical != 0 and weight == value and len(set(cols)) == len(cols), \
        "witness check failed"


def distance(p, order=None, start=1, kmax=64, mode="mitm", use_h=True, witness=True, log=None, every=None,
             backend="gpu", dense=None, split=None, trellises=None):
    """Exact distance by raising the threshold K from `start` (a known lower bound): at each K
    every observable's query runs with lower = K, and the first one that meets at weight <= K gives
    the distance (every smaller K failed for all of them).  Returns the distance (None if above
    kmax), a witness checked against H and L, the lower bound proved, and one summary per query run
    (the reference's distance, cdist/sparse_dp.py:1110-1151).  trellises: plan_trellises' result."""
    t0 = time.time()
    if trellises is None:
        order = default_order(p) if order is None else order
        trellises = [Trellis.for_query(p, i, order) for i in range(p.nobs)]
    live = [(i, t) for i, t in enumerate(trellises) if t.feasible]
    out = {"distance": None, "witness": None, "runs": [], "lower_bound": start,
           "order_cut_rank": max((max(t.width) for _, t in live), default=0)}
    for K in range(start, kmax + 1):
        hit = None
        for i, tr in live:
            r = query(tr, K, mode=mode, use_h=use_h, witness=witness, lower=K, every=every, backend=backend,
                      dense=dense, split=split(K) if callable(split) else split)
            r["obs"] = i
            out["runs"].append(summary(r))
            if log:
                log("  K=%d obs %d: value %s peak %d states %.2fs" % (K, i, r["value"], r["peak_states"],
                                                                      r["seconds"]))
            if r["value"] is not None:
                hit = r
                break
        if hit is not None:
            out["distance"] = hit["value"]
            if witness:
                _check_witness(p, hit["witness"], hit["value"])
                out["witness"] = hit["witness"]
            break
        out["lower_bound"] = K + 1
    out["seconds"] = time.time() - t0
    return out


def summary(r):
    """A query record with its per-cut lists replaced by their totals (`<name>_states_total`)."""
    per_cut = ("forward_counts", "backward_counts", "changed_counts")
    out = {k: v for k, v in r.items() if k not in per_cut and k not in ("witness", "split_values")}
    for k in per_cut:
        if k in r:
            out[k[:-len("_counts")] + "_states_total"] = int(sum(r[k]))
    return out
