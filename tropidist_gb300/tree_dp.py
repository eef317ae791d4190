"""Exact min-plus DP on a binary tree of columns, executed on the GPU (drop-in for cdist/tree_dp.py).

CompiledTreeDP(columns, tree).run(target) -> (least Hamming weight of e with M e = target, or None
when the system has no solution; stats), as cdist/tree_dp.py:255-501.  Columns are nonnegative
Python ints (bit masks over the rows); a tree is a column index or a pair of trees whose leaves are
range(len(columns)) once each; None is the empty tree.

The mathematics is the reference's (cdist/tree_dp.py:3-29): with a particular solution e0 and
e = e0 + x, M x = 0, the table of a node S holds, for every interface state M_S x_S in
im(M_S) & im(M_rest), the least sum over j in S of (x_j xor e0_j); a join combines the
compatible child pairs, 2^J of them with J = dim(parent interface) + dim(left & right interfaces).

Compilation (host, exact GF(2) elimination on Python ints) gives every node's interface basis and
every join's generator maps.  Execution is on the device: leaves are initialised from the target's
representative in one launch, and the joins run grouped by height (every join of one height in one
launch; long runs of tiny heights in a single-block launch) over uint32 tables in one device arena
(tropidist_gb300/csrc/tree.cu).  There is no CPU executor: without the library or a GPU, run()
raises.

tree_min_distance_for_mask / preflight_tree_dp: the logical-query front ends of
cdist/tree_dp.py:508-546.
"""
from __future__ import annotations

import ctypes
import sys
import time
from dataclasses import dataclass

import numpy as np

DEFAULT_MEMORY_BYTES = 256 << 20       # cdist/tree_dp.py:40-41: the same limits, the same accounting
DEFAULT_JOIN_WORK = 100_000_000
DEVICE_INDEX_BITS = 32                 # device tables are indexed by uint32 states


class TreeDPResourceError(RuntimeError):
    """Compilation, dense memory, candidate-pair work, or time limit exceeded."""

    def __init__(self, message, profile=None):
        super().__init__(message)
        self.profile = profile


# ---------------------------------------------------------------- GF(2) elimination on Python ints
class _Eliminator:
    """Row echelon form keyed by leading bit; optionally tracks which inputs combine to each row."""

    def __init__(self, track=False, dependencies=True):
        self.rows = {}          # leading bit -> (vector, combination of inputs)
        self.track = track
        self.keep = track and dependencies
        self.dependencies = []  # combinations of inputs that sum to zero
        self.count = 0

    def add(self, v):
        comb = (1 << self.count) if self.track else 0
        self.count += 1
        while v:
            top = v.bit_length() - 1
            row = self.rows.get(top)
            if row is None:
                self.rows[top] = (v, comb)
                return True
            v ^= row[0]
            comb ^= row[1]
        if self.keep:
            self.dependencies.append(comb)
        return False

    def express(self, v):
        """Combination of inputs summing to v, or None if v is outside their span."""
        comb = 0
        while v:
            row = self.rows.get(v.bit_length() - 1)
            if row is None:
                return None
            v ^= row[0]
            comb ^= row[1]
        return comb

    def rank(self):
        return len(self.rows)


def _span_basis(vectors):
    e = _Eliminator()
    for v in vectors:
        e.add(v)
    return tuple(v for v, _ in e.rows.values())


def _combine(vectors, bits):
    out = 0
    i = 0
    while bits:
        if bits & 1:
            out ^= vectors[i]
        bits >>= 1
        i += 1
    return out


def _extend_basis(first, basis):
    """A basis of span(basis) that starts with the independent vectors `first` (inside that span)."""
    e = _Eliminator()
    out = []
    for v in tuple(first) + tuple(basis):
        if e.add(v):
            out.append(v)
    assert len(out) == len(basis)
    return tuple(out)


def _intersect(a, b):
    """Basis of span(a) & span(b) for independent a and b: the a-part of every dependency of a + b."""
    e = _Eliminator(track=True)
    for v in tuple(a) + tuple(b):
        e.add(v)
    lo = (1 << len(a)) - 1
    return tuple(_combine(a, d & lo) for d in e.dependencies)


# ---------------------------------------------------------------- tree structure
@dataclass(frozen=True)
class TreeNode:
    leaf: int | None
    left: int | None = None
    right: int | None = None


@dataclass(frozen=True)
class TreeJoin:
    left_rank: int
    right_rank: int
    parent_rank: int
    parent_maps: tuple
    free_maps: tuple

    @property
    def join_dimension(self):
        return self.parent_rank + len(self.free_maps)

    @property
    def work(self):
        return 1 << self.join_dimension


def _flatten(tree, ncols):
    """Post-order node list (children before parents, left subtree first) without recursion, with
    the reference's validation (cdist/tree_dp.py:146-173)."""
    if ncols == 0:
        if tree is not None:
            raise ValueError("the empty problem requires tree=None")
        return ()
    nodes, seen, built = [], set(), []
    todo = [(tree, 0)]
    visits = 0
    while todo:
        item, state = todo.pop()
        if state == 1:
            r, l = built.pop(), built.pop()
            built.append(len(nodes))
            nodes.append(TreeNode(None, l, r))
            continue
        visits += 1
        if visits > 2 * ncols - 1:
            raise ValueError("tree has too many nodes, repeated leaves, or a cycle")
        if isinstance(item, int) and not isinstance(item, bool):
            if item < 0 or item >= ncols or item in seen:
                raise ValueError("tree leaves must be each column index exactly once")
            seen.add(item)
            built.append(len(nodes))
            nodes.append(TreeNode(item))
        elif isinstance(item, (tuple, list)) and len(item) == 2:
            todo.append((item, 1))
            todo.append((item[1], 0))
            todo.append((item[0], 0))
        else:
            raise ValueError("each tree node must be an integer leaf or a binary pair")
    if len(seen) != ncols or len(built) != 1:
        raise ValueError("tree leaves must be each column index exactly once")
    return tuple(nodes)


def _deep_size(obj):
    """Recursive sys.getsizeof of a Python object graph, shared objects once."""
    total, seen, todo = 0, set(), [obj]
    while todo:
        x = todo.pop()
        if id(x) in seen:
            continue
        seen.add(id(x))
        total += sys.getsizeof(x)
        if isinstance(x, dict):
            todo.extend(x.keys())
            todo.extend(x.values())
        elif isinstance(x, (tuple, list, set, frozenset)):
            todo.extend(x)
        elif hasattr(x, "__dict__"):
            todo.append(vars(x))
    return total


def cost_dtype(ncols):
    """The reference's table dtype: the narrowest unsigned type holding ncols + 1."""
    for dt in (np.uint8, np.uint16, np.uint32, np.uint64):
        if ncols + 1 <= np.iinfo(dt).max:
            return np.dtype(dt)
    raise ValueError("number of columns exceeds supported exact integer range")


class _Arena:
    """First-fit placement of the device tables (offsets in uint32 entries, 32-byte aligned)."""

    def __init__(self):
        self.free = []          # sorted (offset, size)
        self.top = 0
        self.peak = 0
        self.live = 0
        self.peak_live = 0

    @staticmethod
    def _round(n):
        return (n + 7) & ~7

    def alloc(self, n):
        self.live += n
        self.peak_live = max(self.peak_live, self.live)
        n = self._round(n)
        for i, (o, s) in enumerate(self.free):
            if s >= n:
                if s == n:
                    del self.free[i]
                else:
                    self.free[i] = (o + n, s - n)
                return o
        o = self.top
        self.top += n
        self.peak = max(self.peak, self.top)
        return o

    def release(self, o, n):
        self.live -= n
        n = self._round(n)
        import bisect
        i = bisect.bisect_left(self.free, (o, 0))
        self.free.insert(i, (o, n))
        # merge with the neighbours, then give a block at the top back
        if i + 1 < len(self.free) and self.free[i][0] + self.free[i][1] == self.free[i + 1][0]:
            self.free[i] = (self.free[i][0], self.free[i][1] + self.free[i + 1][1])
            del self.free[i + 1]
        if i > 0 and self.free[i - 1][0] + self.free[i - 1][1] == self.free[i][0]:
            self.free[i - 1] = (self.free[i - 1][0], self.free[i - 1][1] + self.free[i][1])
            del self.free[i]
            i -= 1
        if self.free and self.free[-1][0] + self.free[-1][1] == self.top:
            self.top = self.free[-1][0]
            del self.free[-1]


# ---------------------------------------------------------------- compiled tree
class CompiledTreeDP:
    """A binary tree realization of M, reusable for any target (cdist/tree_dp.py:236-406).

    max_compile_bytes bounds the reference's conservative estimate of the basis storage before any
    basis is built; max_compile_seconds is checked between nodes.  Nothing exponential in size is
    allocated until run()."""

    def __init__(self, columns, tree, *, max_compile_bytes=DEFAULT_MEMORY_BYTES, max_compile_seconds=60.0):
        t0 = time.monotonic()
        self.columns = tuple(columns)
        for v in self.columns:
            if not isinstance(v, int) or isinstance(v, bool) or v < 0:
                raise ValueError("columns must be nonnegative Python integers")
        self.ncols = len(self.columns)
        self.nodes = _flatten(tree, self.ncols)
        self.root = len(self.nodes) - 1
        dt = cost_dtype(self.ncols)
        self.dtype, self.itemsize, self.infinity = dt.name, dt.itemsize, self.ncols + 1

        def check_time():
            if max_compile_seconds is not None and time.monotonic() - t0 > max_compile_seconds:
                raise TreeDPResourceError("tree compilation exceeded max_compile_seconds")

        # storage bound before building anything: at most min(rank, leaves below) vectors per node
        # in four per-node collections, plus elimination workspace (cdist/tree_dp.py:270-291)
        rank_bound = min(self.ncols, max((v.bit_length() for v in self.columns), default=0))
        below = []
        for nd in self.nodes:
            below.append(1 if nd.leaf is not None else below[nd.left] + below[nd.right])
        vec_b = sys.getsizeof(1 << rank_bound) + 8
        amb_b = max((sys.getsizeof(v) for v in self.columns), default=28) + 8
        self.compile_storage_bound_bytes = (
            _deep_size(self.columns) + _deep_size(self.nodes)
            + sum(min(rank_bound, c) for c in below) * (4 * amb_b + 2 * vec_b)
            + len(self.nodes) * rank_bound * (amb_b + vec_b)
            + 16 * (rank_bound + 1) ** 2 + len(self.nodes) * 512 + 16384)
        if max_compile_bytes is not None and self.compile_storage_bound_bytes > max_compile_bytes:
            raise TreeDPResourceError(
                "conservative compilation bound %d bytes exceeds max_compile_bytes=%d"
                % (self.compile_storage_bound_bytes, max_compile_bytes),
                {"compile_storage_bound_bytes": self.compile_storage_bound_bytes})

        self.solver = _Eliminator(track=True, dependencies=False)
        for v in self.columns:
            self.solver.add(v)
        self.matrix_rank = self.solver.rank()

        # column span of every subtree (bottom up), of everything outside it (top down), and the
        # interface: their intersection
        space, space_rank = {}, []
        for i, nd in enumerate(self.nodes):
            check_time()
            space[i] = (_span_basis((self.columns[nd.leaf],)) if nd.leaf is not None
                        else _span_basis(space[nd.left] + space[nd.right]))
            space_rank.append(len(space[i]))
        outside = {self.root: ()} if self.nodes else {}
        interfaces = [()] * len(self.nodes)
        outside_rank = [0] * len(self.nodes)
        for i in range(len(self.nodes) - 1, -1, -1):
            check_time()
            nd = self.nodes[i]
            comp = outside.pop(i)
            outside_rank[i] = len(comp)
            interfaces[i] = _intersect(space.pop(i), comp)
            if nd.leaf is None:
                outside[nd.left] = _span_basis(comp + space[nd.right])
                outside[nd.right] = _span_basis(comp + space[nd.left])
        # a child's table may be indexed in any basis of its interface; both children of a join take
        # the basis of their common part first (in the same order), so the join's kernel generators
        # become pairs of unit vectors (e_k, e_k): the pairs of one parent then read aligned blocks
        # of 2^F entries of each child table
        for i, nd in enumerate(self.nodes):
            if nd.leaf is None:
                common = _intersect(interfaces[nd.left], interfaces[nd.right])
                interfaces[nd.left] = _extend_basis(common, interfaces[nd.left])
                interfaces[nd.right] = _extend_basis(common, interfaces[nd.right])
        self.interfaces = tuple(interfaces)

        # generator maps of every join; the stack schedule of the reference's executor (its arena
        # accounting, reported by preflight)
        self.joins, self.execution_children = {}, {}
        peaks = []
        for i, nd in enumerate(self.nodes):
            check_time()
            prank = len(interfaces[i])
            if nd.leaf is not None:
                peaks.append(1 << prank)
                continue
            il, ir = interfaces[nd.left], interfaces[nd.right]
            e = _Eliminator(track=True)
            for v in il + ir:
                e.add(v)
            pmaps = [e.express(v) for v in interfaces[i]]
            if any(m is None for m in pmaps):
                raise AssertionError("parent interface must be contained in the child sum")
            nf = len(e.dependencies)
            if e.dependencies != [(1 << k) | (1 << (len(il) + k)) for k in range(nf)]:
                raise AssertionError("kernel generators must be the common basis vectors")
            # parent generators modulo the kernel: no left coordinate among the common ones
            low = (1 << nf) - 1
            pmaps = tuple(m ^ (m & low) ^ ((m & low) << len(il)) for m in pmaps)
            jn = TreeJoin(len(il), len(ir), prank, pmaps, tuple(e.dependencies))
            if jn.join_dimension != space_rank[nd.left] + space_rank[nd.right] + outside_rank[i] - self.matrix_rank:
                raise AssertionError("compatible-pair dimension identity failed")
            self.joins[i] = jn
            ls, rs, ps = 1 << len(il), 1 << len(ir), 1 << prank
            here = ls + rs + ps
            lr = max(peaks[nd.left], ls + peaks[nd.right], here)
            rl = max(peaks[nd.right], rs + peaks[nd.left], here)
            if lr <= rl:
                self.execution_children[i] = (nd.left, nd.right)
                peaks.append(lr)
            else:
                self.execution_children[i] = (nd.right, nd.left)
                peaks.append(rl)
        order, todo = [], ([(self.root, False)] if self.nodes else [])
        while todo:
            i, done = todo.pop()
            if done or self.nodes[i].leaf is not None:
                order.append(i)
            else:
                a, b = self.execution_children[i]
                todo.extend(((i, True), (b, False), (a, False)))
        self.order = tuple(order)
        self.peak_live_entries = peaks[self.root] if self.nodes else 0
        self._device = {}
        self.compilation_seconds = time.monotonic() - t0
        self.compiled_metadata_bytes = _deep_size({k: v for k, v in vars(self).items() if k != "_device"})

    # ------------------------------------------------------------ accounting
    def preflight(self, *, max_memory_bytes=DEFAULT_MEMORY_BYTES, max_join_work=DEFAULT_JOIN_WORK,
                  max_table_bits=None):
        """Table sizes and candidate-pair counts, with the reference's limits and accounting
        (cdist/tree_dp.py:371-406) plus the device figures of this executor."""
        base = self._device.get("profile")
        if base is None:
            base = self._device["profile"] = self._profile()
        max_rank, max_join, work = base["max_interface_rank"], base["max_join_dimension"], base["join_work"]
        table_bytes, peak = base["peak_live_table_bytes"], base["peak_dense_bytes"]
        why = []
        if max_rank >= 63 or max_join >= 63:
            why.append("table or join index requires at least 63 bits")
        if table_bytes > np.iinfo(np.intp).max:
            why.append("arena exceeds the platform array index range")
        if max_table_bits is not None and max_rank > max_table_bits:
            why.append("interface rank %d exceeds max_table_bits=%d" % (max_rank, max_table_bits))
        if max_memory_bytes is not None and peak > max_memory_bytes:
            why.append("dense workspace %d bytes exceeds max_memory_bytes=%d" % (peak, max_memory_bytes))
        if max_join_work is not None and work > max_join_work:
            why.append("join work %d exceeds max_join_work=%d" % (work, max_join_work))
        return dict(base, allowed=not why, rejection_reasons=why)

    def _profile(self):
        """The target- and limit-independent part of preflight (computed once)."""
        ranks = [len(v) for v in self.interfaces]
        max_rank = max(ranks, default=0)
        max_join = max((j.join_dimension for j in self.joins.values()), default=0)
        work = sum(j.work for j in self.joins.values())
        table_bytes = self.peak_live_entries * self.itemsize
        scratch = 2 * max_join * 8
        peak = table_bytes + scratch
        dev = self._layout() if max_rank < 63 else None
        return {
            "ncols": self.ncols, "matrix_rank": self.matrix_rank,
            "dtype": self.dtype, "dtype_bytes": self.itemsize, "infinity": self.infinity,
            "edge_state_dimensions": ranks, "max_interface_rank": max_rank,
            "max_join_dimension": max_join, "join_work": work,
            "join_profiles": [dict(node=i, left_rank=j.left_rank, right_rank=j.right_rank,
                                   parent_rank=j.parent_rank, kernel_rank=len(j.free_maps),
                                   join_dimension=j.join_dimension, work=j.work,
                                   child_parent_table_bytes=self.itemsize * ((1 << j.left_rank) + (1 << j.right_rank)
                                                                             + (1 << j.parent_rank)))
                              for i, j in self.joins.items()],
            "largest_table_bytes": (1 << max_rank) * self.itemsize if self.nodes else 0,
            "peak_live_table_bytes": table_bytes, "arena_bytes": table_bytes,
            "scratch_bytes": scratch, "peak_dense_bytes": peak,
            "compiled_metadata_bytes": self.compiled_metadata_bytes,
            "compile_storage_bound_bytes": self.compile_storage_bound_bytes,
            "compilation_seconds": self.compilation_seconds,
            "memory_scope": "reference accounting (stack-ordered arena of the table dtype); the device "
                            "arena is reported as device_arena_bytes",
            "threads": 1,
            "device_dtype": "uint32",
            "device_arena_bytes": 4 * dev["arena"] if dev else None,
            "device_peak_live_table_bytes": 4 * dev["peak_live"] if dev else None,
            "device_heights": dev["heights"] if dev else None,
        }

    def _layout(self):
        """Heights, arena offsets and descriptor rows of the device executor (target independent)."""
        if "layout" in self._device:
            return self._device["layout"]
        n = len(self.nodes)
        height = [0] * n
        for i, nd in enumerate(self.nodes):
            if nd.leaf is None:
                height[i] = 1 + max(height[nd.left], height[nd.right])
        H = max(height, default=0)
        by_h = [[] for _ in range(H + 1)]
        for i in range(n):
            by_h[height[i]].append(i)
        size = [1 << len(v) for v in self.interfaces]
        A = _Arena()
        off = [0] * n
        for i in by_h[0]:
            off[i] = A.alloc(size[i])
        for h in range(1, H + 1):
            for i in by_h[h]:
                off[i] = A.alloc(size[i])
            for i in by_h[h]:
                nd = self.nodes[i]
                A.release(off[nd.left], size[nd.left])
                A.release(off[nd.right], size[nd.right])
        leaves = np.array([[off[i], size[i], self.nodes[i].leaf, 1 if self.columns[self.nodes[i].leaf] else 0]
                           for i in by_h[0]], dtype=np.int64).reshape(-1, 4)
        rows, maps, grows, gmaps = [], [], [], []
        for h in range(1, H + 1):
            for i in by_h[h]:
                nd, jn = self.nodes[i], self.joins[i]
                g = gemm_form(jn)
                if g is not None and g["F"] >= 2 and 6 <= g["mb"] <= 21 and 6 <= g["nb"] <= 21 and g["kb"] <= 16:
                    grows.append([len(rows), g["F"], g["mb"], g["nb"], g["kb"], len(gmaps)])
                    for k in ("DL", "DR", "DT", "PA", "PB", "PT"):
                        gmaps.extend(g[k])
                rows.append([off[nd.left], off[nd.right], off[i], jn.parent_rank, len(jn.free_maps), h,
                             len(maps) // 2, 0])
                lo = (1 << jn.left_rank) - 1
                for gen in jn.parent_maps + jn.free_maps:
                    maps.append(gen & lo)
                    maps.append(gen >> jn.left_rank)
        lay = {"heights": H, "arena": max(A.peak, 1), "peak_live": A.peak_live,
               "leaves": leaves, "joins": np.array(rows, dtype=np.int64).reshape(-1, 8),
               "maps": np.array(maps, dtype=np.uint64), "root": off[self.root] if n else 0,
               "gemm": np.array(grows, dtype=np.int64).reshape(-1, 6), "gmaps": np.array(gmaps, dtype=np.uint32)}
        self._device["layout"] = lay
        return lay

    def device_plan(self, small_pairs=-1, rbits=-1, gemm=True):
        """The library's plan handle for this tree (built once per setting); gemm: run the joins that
        have the block-product form as min-plus block products."""
        from . import _lib
        key = ("plan", small_pairs, rbits, gemm)
        if key in self._device:
            return self._device[key]
        lay = self._layout()
        ranks = [len(v) for v in self.interfaces]
        if max(ranks, default=0) > DEVICE_INDEX_BITS:
            raise TreeDPResourceError("interface rank %d exceeds the %d-bit state index of the device tables"
                                      % (max(ranks), DEVICE_INDEX_BITS))
        maps = np.ascontiguousarray(lay["maps"].astype(np.uint32))
        lv, jr = np.ascontiguousarray(lay["leaves"]), np.ascontiguousarray(lay["joins"])
        gr = np.ascontiguousarray(lay["gemm"] if gemm else lay["gemm"][:0])
        gm = np.ascontiguousarray(lay["gmaps"])
        st = ctypes.c_int(0)
        h = _lib.lib().tg_tree_plan(lv.ctypes.data if len(lv) else None, len(lv),
                                    jr.ctypes.data if len(jr) else None, len(jr),
                                    maps.ctypes.data if len(maps) else None, len(maps) // 2,
                                    gr.ctypes.data if len(gr) else None, len(gr),
                                    gm.ctypes.data if len(gm) else None, len(gm),
                                    int(lay["arena"]), int(lay["root"]), self.ncols, int(small_pairs), int(rbits),
                                    ctypes.byref(st))
        if not h:
            _lib.check(st.value)
        self._device[key] = h
        return h

    def device_info(self, small_pairs=-1, rbits=-1, gemm=True):
        from . import _lib
        info = np.zeros(9, dtype=np.int64)
        _lib.check(_lib.lib().tg_tree_plan_info(self.device_plan(small_pairs, rbits, gemm), info.ctypes.data, 9))
        keys = ("heights", "steps", "launches", "pairs", "arena_entries", "leaves", "joins", "single_block_steps",
                "block_product_joins")
        return dict(zip(keys, (int(x) for x in info)))

    def free(self):
        """Release the library's plan handles (the host layout and profile stay)."""
        from . import _lib
        plans = [k for k in self._device if isinstance(k, tuple) and k[0] == "plan"]
        for k in plans:
            if self._device[k]:
                _lib.lib().tg_tree_plan_free(self._device[k])
            del self._device[k]

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    # ------------------------------------------------------------ execution
    def representative(self, target):
        """Column mask of a particular solution of M e = target, or None."""
        return self.solver.express(target)

    def run(self, target=0, *, max_memory_bytes=DEFAULT_MEMORY_BYTES, max_join_work=DEFAULT_JOIN_WORK,
            max_table_bits=None, max_seconds=60.0, backend="gpu", arena=None, small_pairs=-1, rbits=-1, gemm=True):
        """(exact minimum weight or None, stats), as cdist/tree_dp.py:409-501.  backend: "gpu" (or
        "c", the reference's name of its compiled executor); arena: an optional device buffer of at
        least device_arena_bytes, reused across calls."""
        if not isinstance(target, int) or isinstance(target, bool) or target < 0:
            raise ValueError("target must be a nonnegative Python integer")
        if backend not in ("gpu", "c"):
            raise ValueError("backend must be 'gpu' (or 'c'); this package has no Python executor")
        prof = self.preflight(max_memory_bytes=max_memory_bytes, max_join_work=max_join_work,
                              max_table_bits=max_table_bits)
        rep = self.representative(target)
        if rep is None:
            return None, dict(prof, feasible=False, seconds=0.0, join_work_done=0, allocated_dense_bytes=0,
                              backend="gpu")
        if not prof["allowed"]:
            raise TreeDPResourceError("; ".join(prof["rejection_reasons"]), prof)
        if not self.nodes:
            return 0, dict(prof, feasible=True, seconds=0.0, join_work_done=0, allocated_dense_bytes=0, backend="gpu")
        t0 = time.monotonic()
        if max_seconds is not None and time.monotonic() - t0 > max_seconds:
            raise TreeDPResourceError("tree DP exceeded max_seconds; no exact result returned", prof)
        from . import _lib, device
        device.require_gpu()
        plan = self.device_plan(small_pairs, rbits, gemm)
        need = prof["device_arena_bytes"]
        if arena is None or arena.numel() * arena.element_size() < need:
            try:
                arena = device.empty(need)
            except RuntimeError as e:       # torch's out-of-memory error
                raise TreeDPResourceError("device arena of %d bytes: %s" % (need, e), prof)
        words = np.zeros(max(1, (self.ncols + 63) // 64), dtype=np.uint64)
        x, k = rep, 0
        while x:
            words[k] = x & 0xFFFFFFFFFFFFFFFF
            x >>= 64
            k += 1
        val = ctypes.c_uint32(0)
        _lib.check(_lib.lib().tg_tree_run(plan, arena.data_ptr(), words.ctypes.data, self.infinity,
                                          ctypes.byref(val), device.stream_ptr()))
        secs = time.monotonic() - t0
        if max_seconds is not None and secs > max_seconds:
            raise TreeDPResourceError("tree DP exceeded max_seconds; no exact result returned", prof)
        if val.value >= self.infinity:
            raise AssertionError("a consistent affine system must have a finite root cost")
        return int(val.value), dict(prof, feasible=True, seconds=secs, join_work_done=prof["join_work"],
                                    allocated_dense_bytes=need, observed_peak_live_table_bytes=
                                    prof["device_peak_live_table_bytes"], backend="gpu")


def _augmented(h_cols, l_cols, mask):
    if len(h_cols) != len(l_cols):
        raise ValueError("H and L must have the same number of columns")
    if not isinstance(mask, int) or isinstance(mask, bool) or mask < 0:
        raise ValueError("observable mask must be a nonnegative Python integer")
    for v in l_cols:
        if not isinstance(v, int) or isinstance(v, bool) or v < 0:
            raise ValueError("logical columns must be nonnegative Python integers")
    for v in h_cols:
        if not isinstance(v, int) or isinstance(v, bool) or v < 0:
            raise ValueError("detector columns must be nonnegative Python integers")
    nrows = max((v.bit_length() for v in h_cols), default=0)
    cols = tuple(h | ((bin(l & mask).count("1") & 1) << nrows) for h, l in zip(h_cols, l_cols))
    return cols, nrows


def tree_min_distance_for_mask(h_cols, l_cols, mask, tree, *, max_compile_bytes=DEFAULT_MEMORY_BYTES,
                               max_compile_seconds=60.0, **limits):
    """Least weight of e with H e = 0 and parity(mask & L e) = 1 on the given tree
    (cdist/tree_dp.py:508-527): the target row is appended below H's rows."""
    cols, nrows = _augmented(h_cols, l_cols, mask)
    prog = CompiledTreeDP(cols, tree, max_compile_bytes=max_compile_bytes, max_compile_seconds=max_compile_seconds)
    d, info = prog.run(1 << nrows, **limits)
    info["observable_mask"] = mask
    prog.free()
    return d, info


def preflight_tree_dp(h_cols, l_cols, mask, tree, *, max_compile_bytes=DEFAULT_MEMORY_BYTES,
                      max_compile_seconds=60.0, **limits):
    """Resources and feasibility of a logical query without running it (cdist/tree_dp.py:530-546)."""
    cols, nrows = _augmented(h_cols, l_cols, mask)
    prog = CompiledTreeDP(cols, tree, max_compile_bytes=max_compile_bytes, max_compile_seconds=max_compile_seconds)
    return dict(prog.preflight(**limits), feasible=prog.representative(1 << nrows) is not None,
                observable_mask=mask)


def gemm_form(join):
    """The block-product form of a join, or None.

    With the kernel generators (e_k, e_k), parent p reads left entries (a(p) << F) | f and right
    entries (b(p) << F) | (f ^ d(p)) for f < 2^F, where a, b, d are linear in p.  When p -> (a, b)
    is onto (every left block meets every right block), p = PA a ^ PB b ^ PT t with t in the kernel of
    that map, and d = DL a ^ DR b ^ DT t; with f' = f ^ DL a the parent's value is
        min over f' of L[(a << F) | (f' ^ DL a)] + R[(b << F) | (f' ^ DR b ^ DT t)]
    a min-plus product of 2^mb left rows and 2^nb right rows of length 2^F, once per t.
    Returns dict(F, mb, nb, kb, DL, DR, DT, PA, PB, PT) (lists of ints, one per bit)."""
    F = len(join.free_maps)
    lr, rr, P = join.left_rank, join.right_rank, join.parent_rank
    mb, nb = lr - F, rr - F
    low = (1 << F) - 1
    # per parent generator: its (a | b << mb) block coordinates and its d
    ab, dd = [], []
    for m in join.parent_maps:
        left, right = m & ((1 << lr) - 1), m >> lr
        if left & low:
            return None
        ab.append((left >> F) | ((right >> F) << mb))
        dd.append(right & low)
    e = _Eliminator(track=True)
    for v in ab:
        e.add(v)
    if e.rank() != mb + nb:
        return None
    PA = [e.express(1 << i) for i in range(mb)]
    PB = [e.express(1 << (mb + j)) for j in range(nb)]
    PT = list(e.dependencies)
    d_of = lambda comb: _combine(dd, comb)
    return {"F": F, "mb": mb, "nb": nb, "kb": len(PT), "PA": PA, "PB": PB, "PT": PT,
            "DL": [d_of(c) for c in PA], "DR": [d_of(c) for c in PB], "DT": [d_of(c) for c in PT]}
