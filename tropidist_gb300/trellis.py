"""Host planning of the dense Rank DP: the minimal-span trellis of one query and its op stream.

For a column order, the state at cut i is the vector of partial parities of the rows that are
"active" there (started, not yet ended) once the rows are in minimal span form (distinct starts,
distinct ends).  The sweep over the columns is a stream of three ops on a table of 2^width
entries:

  ("expand",)              a row starts: the table doubles, the new row is its top bit and the
                           upper half starts at infinity
  ("update", mask[, w])    a column: T[s] = min(T[s], T[s ^ mask] + w)   (w = 1 unless given)
  ("select", pos, target)  a row ends: keep the entries whose bit `pos` equals `target` and
                           remove that bit (the table halves)

The reduction steps follow the reference planner exactly, because the state encoding (which
row sits at which bit) has to be identical for the DP tables to be identical entry for entry:
  rank_profile / cut_profile      cdist/trellis.py:20-44
  rows_from_columns               cdist/trellis.py:47-57
  minimal_span_form               cdist/trellis.py:60-97
  reduce_target_row               cdist/trellis.py:100-122
  Plan / make_plan / build_plan   cdist/trellis.py:125-193
Weighted columns (the optional third field of an update) have no counterpart in the reference.
"""
from __future__ import annotations


import numpy as np

OP_EXPAND, OP_UPDATE, OP_SELECT = 0, 1, 2


def lowbit(x):
    """Index of the lowest set bit (-1 for 0)."""
    return (x & -x).bit_length() - 1


def bit_positions(values, nbits=None):
    """Set-bit positions of many nonnegative ints at once: (ptr int64 [n + 1], pos int32), positions
    ascending within each value (one byte scan instead of a big-int loop per bit)."""
    n = len(values)
    if nbits is None:
        nbits = max((v.bit_length() for v in values), default=0)
    nb = max(1, (nbits + 7) // 8)
    B = np.frombuffer(b"".join(v.to_bytes(nb, "little") for v in values), dtype=np.uint8).reshape(n, nb)
    r, k = np.nonzero(B)
    U = np.unpackbits(B[r, k][:, None], axis=1, bitorder="little")
    i, b = np.nonzero(U)
    which = r[i]
    pos = (k[i].astype(np.int64) * 8 + b).astype(np.int32)
    ptr = np.zeros(n + 1, dtype=np.int64)
    ptr[1:] = np.cumsum(np.bincount(which, minlength=n))
    return ptr, pos


_CSR = [None, None]     # key of the last column list given to rank_profile, its (nrows, col_ptr, col_rows)


def _columns_csr(cols):
    key = (len(cols), hash(tuple(cols)))
    if _CSR[0] != key:
        ptr, pos = bit_positions(cols)
        nrows = int(pos.max()) + 1 if pos.size else 0
        _CSR[0], _CSR[1] = key, (nrows, ptr, pos)
    return _CSR[1]


def rank_profile(cols, order):
    """r[i] = GF(2) rank of the first i columns of `order`, for i = 0..N (cdist/trellis.py:20-36),
    by the library's host routine (word-parallel bitsets; rank_profile_py restates it in Python)."""
    from . import _lib
    nrows, col_ptr, col_rows = _columns_csr(cols)
    order_a = np.ascontiguousarray(np.asarray(order, dtype=np.int32))
    out = np.zeros(len(order) + 1, dtype=np.int32)
    _lib.check(_lib.lib().tg_rank_profile(len(order), nrows, col_ptr.ctypes.data,
                                          col_rows.ctypes.data if col_rows.size else None,
                                          order_a.ctypes.data if order_a.size else None, out.ctypes.data))
    return out.tolist()


def rank_profile_py(cols, order):
    """Python restatement of rank_profile (cdist/trellis.py:20-36)."""
    pivots = {}
    rank = 0
    out = [0]
    for j in order:
        v = cols[j]
        while v:
            top = v.bit_length() - 1
            p = pivots.get(top)
            if p is None:
                pivots[top] = v
                rank += 1
                break
            v ^= p
        out.append(rank)
    return out


def cut_profile(cols, order):
    """Cut rank lambda_i = rank(past) + rank(future) - rank(all) for cuts i = 0..N."""
    fwd = rank_profile(cols, order)
    bwd = rank_profile(cols, list(reversed(order)))[::-1]
    tot = fwd[-1]
    return [a + b - tot for a, b in zip(fwd, bwd)]


def rows_from_columns(cols, order, nrows):
    """Row r as a bitmask over column positions of `order`."""
    rows = [0] * nrows
    for pos, j in enumerate(order):
        v = cols[j]
        while v:
            low = v & -v
            rows[low.bit_length() - 1] |= 1 << pos
            v ^= low
    return rows


def minimal_span_form(rows):
    """Row-reduce to distinct starts and distinct ends; dependent rows vanish.

    Starts: a row meeting a stored row with the same start is reduced by whichever of the two
    ends earlier (that one is stored).  Ends: rows are visited latest start first; a row meeting a
    stored row with the same end is reduced by it when the stored row starts later, otherwise it
    replaces the stored row and the difference carries on.
    """
    start_of = {}
    for row in rows:
        cur = row
        while cur:
            s = lowbit(cur)
            held = start_of.get(s)
            if held is None:
                start_of[s] = cur
                break
            if cur.bit_length() < held.bit_length():
                start_of[s] = cur
                cur, held = held, cur
            cur ^= held
    end_of = {}
    for row in sorted(start_of.values(), key=lowbit, reverse=True):
        cur = row
        while True:
            e = cur.bit_length()
            held = end_of.get(e)
            if held is None:
                end_of[e] = cur
                break
            if lowbit(held) > lowbit(cur):
                cur ^= held
            else:
                end_of[e] = cur
                cur ^= held
    out = list(end_of.values())
    assert len({lowbit(r) for r in out}) == len(out) and len({r.bit_length() for r in out}) == len(out)
    return out


def reduce_target_row(lrow, hrows):
    """Shorten the span of the target-1 row with the constraint rows; 0 means the query is
    infeasible (the observable is a combination of the checks)."""
    starts = {lowbit(r): r for r in hrows}
    ends = {r.bit_length(): r for r in hrows}

    def strip_start(x):
        while x:
            q = starts.get(lowbit(x))
            if q is None:
                break
            x ^= q
        return x

    lrow = strip_start(lrow)
    while lrow:
        q = ends.get(lrow.bit_length())
        if q is None or lowbit(q) < lowbit(lrow):
            break
        lrow = strip_start(lrow ^ q)
    return lrow


class Plan:
    """Op stream of one query: ops ("expand",) | ("update", mask[, w]) | ("select", pos, target),
    peak_bits (log2 of the largest table), widths (active rows after each column), columns (the
    position in the order of each update op).  A plan built by the C++ planner holds the encoded
    stream and makes the tuples only when `ops` is read."""

    def __init__(self, ops, peak_bits, widths, ncols, feasible=True, columns=None, enc=None):
        self._ops = ops
        self._enc = enc
        self.peak_bits = peak_bits
        self.widths = widths
        self.ncols = ncols
        self.feasible = feasible
        self.columns = [] if columns is None else columns

    @property
    def ops(self):
        if self._ops is None:
            self._ops = decode_ops(self._enc)
        return self._ops

    def work(self):
        """Table entries touched by the update ops (the state-update count)."""
        if self._enc is not None and self.peak_bits < 48:
            code = self._enc[:, 0]
            delta = (code == OP_EXPAND).astype(np.int64) - (code == OP_SELECT).astype(np.int64)
            before = np.cumsum(delta) - delta
            return int(np.sum(np.left_shift(np.int64(1), before[code == OP_UPDATE])))
        return plan_work(self.ops)

    def encode(self):
        """The op stream as an int64 array of (code, a, b) rows for the C-ABI:
        expand (0, 0, 0); update (1, mask, w); select (2, pos, target)."""
        if self._enc is None:
            self._enc = encode_ops(self._ops)
        return self._enc


def decode_ops(enc):
    out = []
    for code, a, b in enc.tolist():
        if code == OP_EXPAND:
            out.append(("expand",))
        elif code == OP_UPDATE:
            out.append(("update", a) if b == 1 else ("update", a, b))
        else:
            out.append(("select", a, b))
    return out


def plan_work(ops):
    tot = 0
    bits = 0
    for op in ops:
        if op[0] == "expand":
            bits += 1
        elif op[0] == "select":
            bits -= 1
        else:
            tot += 1 << bits
    return tot


def encode_ops(ops):
    out = np.zeros((len(ops), 3), dtype=np.int64)
    for i, op in enumerate(ops):
        if op[0] == "expand":
            out[i, 0] = OP_EXPAND
        elif op[0] == "update":
            mask = int(op[1])
            if mask >> 63:
                raise ValueError("update masks are limited to 63 bits")
            out[i] = (OP_UPDATE, mask, int(op[2]) if len(op) > 2 else 1)
        else:
            out[i] = (OP_SELECT, int(op[1]), int(op[2]))
    return out


def make_plan(hrows, lrow, ncols, weights=None):
    """Op stream of the sweep for constraint rows (target 0) and one target-1 row
    (cdist/trellis.py:147-182), built by the library's C++ planner (tg_make_plan) from the rows as
    bitsets.  weights: optional per-position column weight."""
    if lrow == 0:
        return Plan([], 0, [], ncols, feasible=False)
    import ctypes
    from . import _lib
    rows = list(hrows) + [lrow]
    words = max(1, (ncols + 63) // 64)
    nb = 8 * words
    buf = b"".join(r.to_bytes(nb, "little") for r in rows)
    bits = np.frombuffer(buf, dtype=np.uint64)
    w = None if weights is None else np.ascontiguousarray(weights, dtype=np.int64)
    widths = np.zeros(max(1, ncols), dtype=np.int32)
    out = np.zeros(3, dtype=np.int64)
    cap = 2 * len(rows) + ncols + 16
    L = _lib.lib()
    while True:
        ops = np.zeros((cap, 3), dtype=np.int64)
        cols = np.zeros(cap, dtype=np.int32)
        r = L.tg_make_plan(len(rows), ncols, words, bits.ctypes.data, w.ctypes.data if w is not None else None,
                           ops.ctypes.data, cap, widths.ctypes.data, cols.ctypes.data, out.ctypes.data)
        if r == -4:
            raise ValueError("update masks are limited to 63 bits")
        if r < 0:
            _lib.check(r)
        if r == 0:
            break
        cap = r
    n, nupd, peak = (int(x) for x in out)
    return Plan(None, peak, widths[:ncols].tolist(), ncols, columns=cols[:nupd].tolist(), enc=ops[:n])


def make_plan_py(hrows, lrow, ncols, weights=None):
    """The same op stream built in Python (the cross-check of the C++ planner)."""
    if lrow == 0:
        return Plan([], 0, [], ncols, feasible=False)
    rows = list(hrows) + [lrow]
    target = [0] * len(hrows) + [1]
    begins, finishes = {}, {}
    for idx, r in enumerate(rows):
        begins.setdefault(lowbit(r), []).append(idx)
        finishes.setdefault(r.bit_length() - 1, []).append(idx)
    active = []
    ops, widths, columns = [], [], []
    peak = 0
    for j in range(ncols):
        for idx in begins.get(j, ()):
            active.append(idx)
            ops.append(("expand",))
        peak = max(peak, len(active))
        mask = 0
        for pos, idx in enumerate(active):
            if (rows[idx] >> j) & 1:
                mask |= 1 << pos
        if mask:      # a column touching no active row is a free zero-syndrome fault
            w = 1 if weights is None else int(weights[j])
            ops.append(("update", mask) if w == 1 else ("update", mask, w))
            columns.append(j)
        for pos in sorted((active.index(idx) for idx in finishes.get(j, ())), reverse=True):
            ops.append(("select", pos, target[active[pos]]))
            active.pop(pos)
        widths.append(len(active))
    assert not active
    return Plan(ops, peak, widths, ncols, columns=columns)


def target_row(l, obs_mask, order):
    """Bitmask over positions of the columns whose logical part has odd overlap with obs_mask."""
    lrow = 0
    for pos, j in enumerate(order):
        if bin(l[j] & obs_mask).count("1") & 1:
            lrow |= 1 << pos
    return lrow


def build_plan(h, l, obs_mask, order, nrows, weights=None):
    """Plan of the query  H e = 0, (obs_mask . L) e = 1  in the given column order
    (cdist/trellis.py:185-193).  weights: optional per-column weights (problem indices)."""
    hrows = minimal_span_form(rows_from_columns(h, order, nrows))
    lrow = reduce_target_row(target_row(l, obs_mask, order), hrows)
    pw = None if weights is None else [weights[j] for j in order]
    return make_plan(hrows, lrow, len(order), pw)
