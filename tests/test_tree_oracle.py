"""Tree DP: compilation and the CPU oracle against the reference's own results (tests/golden/
tree_dp.json, written by tests/golden/make_golden.py from cdist/tree_dp.py) and brute force; the
resource checks and input validation of cdist/tree_dp.py (tests/test_tree_dp.py:140-190)."""
import json
import os
import random
from itertools import product

import pytest

from helpers import ROOT
from oracle import tree as ot
from tropidist_gb300 import tree_dp as td

GOLD = json.load(open(os.path.join(ROOT, "tests", "golden", "tree_dp.json")))
KEYS = ("edge_state_dimensions", "max_join_dimension", "join_work", "peak_live_table_bytes",
        "largest_table_bytes", "dtype", "infinity", "matrix_rank")


def tup(t):
    return tuple(tup(x) for x in t) if isinstance(t, list) else t


def balanced(xs):
    if not xs:
        return None
    if len(xs) == 1:
        return xs[0]
    m = len(xs) // 2
    return balanced(xs[:m]), balanced(xs[m:])


def comb(xs):
    if not xs:
        return None
    t = xs[0]
    for x in xs[1:]:
        t = (t, x)
    return t


def test_all_small_matrices_all_targets_oracle():
    solved = 0
    for n in range(5):
        tree = balanced(list(range(n)))
        for cols in product(range(4), repeat=n):
            want = ot.brute_affine(cols)
            prog = td.CompiledTreeDP(cols, tree)
            for t in range(8):
                assert ot.run(prog, t) == want.get(t), (cols, t)
                solved += 1
    assert solved == 2728


@pytest.mark.parametrize("case", range(len(GOLD["affine"])))
def test_compile_and_oracle_match_reference(case):
    c = GOLD["affine"][case]
    prog = td.CompiledTreeDP(c["columns"], tup(c["tree"]))
    pf = prog.preflight()
    for k in KEYS:
        assert pf[k] == c["profile"][k], k
    for t, d in zip(c["targets"], c["distances"]):
        assert ot.run(prog, t) == d


def test_logical_queries_match_reference():
    for c in GOLD["logical"]:
        cols, nrows = td._augmented(c["h"], c["l"], c["mask"])
        prog = td.CompiledTreeDP(cols, tup(c["tree"]))
        assert ot.run(prog, 1 << nrows) == c["distance"]
        assert [len(v) for v in prog.interfaces] == c["edge_state_dimensions"]
        assert ot.brute_logical(c["h"], c["l"], c["mask"]) == c["distance"]


def test_distances_beyond_255():
    for c in GOLD["chains"]:
        n = c["ncols"]
        h = [1] + [(1 << (j - 1)) | (1 << j) for j in range(1, n - 1)] + [1 << (n - 2)]
        cols, nrows = td._augmented(h, [1] + [0] * (n - 1), 1)
        prog = td.CompiledTreeDP(cols, balanced(list(range(n))))
        assert prog.dtype == c["dtype"] and prog.infinity == c["infinity"]
        assert ot.run(prog, 1 << nrows) == c["distance"] == n


def test_large_profiles_match_reference():
    for c in GOLD["large"]:
        prog = td.CompiledTreeDP(c["columns"], tup(c["tree"]))
        pf = prog.preflight(max_join_work=None, max_memory_bytes=None)
        for k in KEYS:
            assert pf[k] == c["profile"][k], k
        if pf["max_join_dimension"] <= 20:
            for t, d in zip(c["targets"], c["distances"]):
                assert ot.run(prog, t) == d


def test_join_dimension_identity_and_interfaces_are_cut_ranks():
    rng = random.Random(5)
    for trial in range(40):
        n, m = rng.randrange(2, 12), rng.randrange(1, 7)
        cols = [rng.randrange(1 << m) for _ in range(n)]
        order = list(range(n))
        rng.shuffle(order)
        prog = td.CompiledTreeDP(cols, comb(order) if trial % 2 else balanced(order))

        def rank(sub):
            e = td._Eliminator()
            for j in sub:
                e.add(cols[j])
            return e.rank()
        sup = []
        for i, nd in enumerate(prog.nodes):
            s = {nd.leaf} if nd.leaf is not None else sup[nd.left] | sup[nd.right]
            sup.append(s)
            rest = set(range(n)) - s
            # dim(im M_S & im M_rest) = rank S + rank rest - rank M
            assert len(prog.interfaces[i]) == rank(s) + rank(rest) - rank(range(n))


def test_device_layout_keeps_live_tables_apart():
    rng = random.Random(9)
    for trial in range(30):
        n, m = rng.randrange(1, 30), rng.randrange(1, 10)
        cols = [rng.randrange(1 << m) for _ in range(n)]
        order = list(range(n))
        rng.shuffle(order)
        prog = td.CompiledTreeDP(cols, (comb, balanced)[trial % 2](order))
        lay = prog._layout()
        size = [1 << len(v) for v in prog.interfaces]
        rows = {}
        for off, sz, col, nz in lay["leaves"]:
            rows[("leaf", int(col))] = (int(off), int(sz))
        # every join's parent must not overlap a table that is live at its height
        height = {}
        for i, nd in enumerate(prog.nodes):
            height[i] = 0 if nd.leaf is not None else 1 + max(height[nd.left], height[nd.right])
        parent = {}
        for i, nd in enumerate(prog.nodes):
            if nd.leaf is None:
                parent[nd.left] = i
                parent[nd.right] = i
        offs = {}
        leaf_off = {int(c): int(o) for o, _, c, _ in lay["leaves"]}
        j = 0
        joins_by_h = sorted((height[i], i) for i in range(len(prog.nodes)) if prog.nodes[i].leaf is None)
        for (h, i), r in zip(joins_by_h, lay["joins"]):
            offs[i] = int(r[2])
            assert r[5] == h
        for i, nd in enumerate(prog.nodes):
            if nd.leaf is not None:
                offs[i] = leaf_off[nd.leaf]
        # live interval of node i: [height[i], height[parent[i]]] (the root to the end)
        H = max(height.values())
        for h in range(H + 1):
            live = [i for i in range(len(prog.nodes))
                    if height[i] <= h and (i == prog.root or height[parent[i]] >= h)]
            spans = sorted((offs[i], offs[i] + size[i]) for i in live)
            for (a0, a1), (b0, b1) in zip(spans, spans[1:]):
                assert a1 <= b0, (trial, h)
            assert all(b <= lay["arena"] for _, b in spans)


def test_preflight_rejects_before_any_device_work():
    prog = td.CompiledTreeDP([1, 2, 3, 1, 2, 3], ((0, (1, 2)), (3, (4, 5))))
    pf = prog.preflight()
    assert pf["join_work"] > 1
    for kw in (dict(max_memory_bytes=pf["peak_dense_bytes"] - 1), dict(max_join_work=pf["join_work"] - 1),
               dict(max_table_bits=0), dict(max_seconds=-1)):
        with pytest.raises(td.TreeDPResourceError):
            prog.run(**kw)
    with pytest.raises(td.TreeDPResourceError):
        td.CompiledTreeDP([1, 2], (0, 1), max_compile_bytes=1)
    assert not td.preflight_tree_dp([1], [0], 1, 0)["feasible"]


def test_empty_and_malformed_inputs():
    prog = td.CompiledTreeDP([], None)
    assert prog.run(0)[0] == 0
    assert prog.run(1)[0] is None
    for tree in ((0, 0), (0, 2), (0,), (False, 1), 0, None):
        with pytest.raises(ValueError):
            td.CompiledTreeDP([1, 2], tree)
    cycle = [0, None]
    cycle[1] = cycle
    with pytest.raises(ValueError):
        td.CompiledTreeDP([1, 2], cycle)
    for col in (-1, True, 1.0):
        with pytest.raises(ValueError):
            td.CompiledTreeDP([col], 0)
    for t in (-1, True, 1.0):
        with pytest.raises(ValueError):
            td.CompiledTreeDP([1], 0).run(t)
    with pytest.raises(ValueError):
        td.CompiledTreeDP([1], 0).run(1, backend="python")


def test_deep_comb_compiles_without_recursion():
    prog = td.CompiledTreeDP([0] * 1300, comb(list(range(1300))))
    assert prog.preflight()["max_interface_rank"] == 0
    assert prog._layout()["heights"] == 1299


def test_free_keeps_host_layout_and_profile():
    prog = td.CompiledTreeDP([1, 2, 3, 1, 2, 3], ((0, (1, 2)), (3, (4, 5))))
    a = prog.preflight()
    prog._layout()
    prog.free()
    b = prog.preflight()
    assert a == b and "layout" in prog._device and "profile" in prog._device
