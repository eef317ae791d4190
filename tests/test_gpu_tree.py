"""Tree DP on the GPU against the reference's results (tests/golden/tree_dp.json), brute force and
the numpy oracle of the join; every device path (single-block heights, the join kernel with owned
and shared parents, inner and outer Gray walks) is forced on small cases; the per-call entry points
tree_join_u* / tree_move against the oracle join."""
import ctypes
import json
import os
import random
from itertools import product

import numpy as np
import pytest

from helpers import ROOT
from oracle import tree as ot

pytestmark = pytest.mark.gpu

GOLD = json.load(open(os.path.join(ROOT, "tests", "golden", "tree_dp.json")))
# (small_pairs, rbits): default; all heights in the join kernel with 1 pair per thread (every
# parent shared by threads: fill + atomics), 2 pairs, the inner walk only, and all pairs of a parent
# in one thread (outer Gray loop)
SETTINGS = [(-1, -1), (0, 0), (0, 1), (0, 6), (0, 62)]


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
    t = xs[0]
    for x in xs[1:]:
        t = (t, x)
    return t


@pytest.fixture(scope="module")
def td():
    import torch
    assert torch.cuda.is_available()
    from tropidist_gb300 import tree_dp
    return tree_dp


def test_all_small_matrices_all_targets(td):
    solved = 0
    for n in range(5):
        tree = balanced(list(range(n)))
        for cols in product(range(4), repeat=n):
            want = ot.brute_affine(cols)
            prog = td.CompiledTreeDP(cols, tree)
            for t in range(8):
                got, st = prog.run(t)
                assert got == want.get(t), (cols, t)
                solved += 1
            prog.free()
    assert solved == 2728


@pytest.mark.parametrize("setting", SETTINGS)
def test_reference_cases_every_path(td, setting):
    sp, rb = setting
    for c in GOLD["affine"]:
        prog = td.CompiledTreeDP(c["columns"], tup(c["tree"]))
        for t, d in zip(c["targets"], c["distances"]):
            assert prog.run(t, small_pairs=sp, rbits=rb)[0] == d, (c["columns"], t, setting)
        prog.free()
    for c in GOLD["large"]:
        prog = td.CompiledTreeDP(c["columns"], tup(c["tree"]))
        for t, d in zip(c["targets"], c["distances"]):
            got = prog.run(t, max_join_work=None, max_memory_bytes=None, max_seconds=None,
                           small_pairs=sp, rbits=rb)[0]
            assert got == d, (t, setting)
        prog.free()


def test_logical_queries_and_distances_beyond_255(td):
    for c in GOLD["logical"]:
        d, st = td.tree_min_distance_for_mask(c["h"], c["l"], c["mask"], tup(c["tree"]))
        assert d == c["distance"]
        assert st["edge_state_dimensions"] == c["edge_state_dimensions"]
    for c in GOLD["chains"]:
        n = c["ncols"]
        h = [1] + [(1 << (j - 1)) | (1 << j) for j in range(1, n - 1)] + [1 << (n - 2)]
        d, st = td.tree_min_distance_for_mask(h, [1] + [0] * (n - 1), 1, balanced(list(range(n))))
        assert d == c["distance"] == n
        assert st["dtype"] == c["dtype"] and st["infinity"] == c["infinity"]


def test_random_trees_against_oracle_every_path(td):
    rng = random.Random(77)
    for trial in range(24):
        m, n = rng.randint(6, 14), rng.randint(12, 40)
        cols = [sum(1 << r for r in rng.sample(range(m), rng.randint(1, 3))) for _ in range(n)]
        order = list(range(n))
        rng.shuffle(order)
        prog = td.CompiledTreeDP(cols, (balanced, comb)[trial % 2](order))
        if prog.preflight()["max_join_dimension"] > 20:
            continue
        for t in [0] + [rng.randrange(1 << m) for _ in range(2)]:
            want = ot.run(prog, t)
            for sp, rb in SETTINGS:
                got = prog.run(t, max_join_work=None, small_pairs=sp, rbits=rb)[0]
                assert got == want, (trial, t, sp, rb)
        prog.free()


def test_deep_comb_and_parent_larger_than_children(td):
    prog = td.CompiledTreeDP([0] * 1300, comb(list(range(1300))))
    assert prog.run()[0] == 0
    info = prog.device_info()
    assert info["heights"] == 1299 and info["launches"] <= 4     # one single-block launch
    cols = [1 << j for j in range(8)] * 2
    prog = td.CompiledTreeDP(cols, balanced(list(range(16))))
    assert prog.preflight()["largest_table_bytes"] == 256
    for t in (0, 1, 3, 17, 127, 128, 255):
        for sp, rb in SETTINGS:
            assert prog.run(t, small_pairs=sp, rbits=rb)[0] == bin(t).count("1")


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("dtype", [np.uint8, np.uint16, np.uint32, np.uint64])
def test_per_call_join_matches_oracle(dtype):
    import torch
    from tropidist_gb300 import _lib
    L = _lib.lib()
    rng = np.random.default_rng(3)
    P, F, lr, rr = 4, 5, 6, 7
    J = P + F
    lm = rng.integers(0, 1 << lr, J).astype(np.uint64)
    rm = rng.integers(0, 1 << rr, J).astype(np.uint64)
    inf = 40
    left = rng.integers(0, inf + 1, 1 << lr).astype(dtype)
    right = rng.integers(0, inf + 1, 1 << rr).astype(dtype)
    want = ot.join(left.astype(np.int64), right.astype(np.int64), [int(x) for x in lm], [int(x) for x in rm], P, inf)
    tdt = {np.uint8: torch.uint8, np.uint16: torch.uint16, np.uint32: torch.uint32, np.uint64: torch.uint64}[dtype]
    dl, dr = _dev(left.view(np.uint8)), _dev(right.view(np.uint8))
    out = torch.full((1 << P,), inf, dtype=tdt, device="cuda")
    fn = getattr(L, "tree_join_u%d" % (8 * np.dtype(dtype).itemsize))
    # in chunks, as the reference's executor calls it (cdist/tree_dp.py:480-488)
    for b in range(0, 1 << J, 77):
        e = min(b + 77, 1 << J)
        assert fn(dl.data_ptr(), dr.data_ptr(), out.data_ptr(), lm.ctypes.data, rm.ctypes.data, P, J, b, e, inf) == 0
    torch.cuda.synchronize()
    got = out.view(torch.uint8).cpu().numpy().view(dtype).astype(np.int64)
    assert np.array_equal(got, want)


def test_tree_move_overlapping():
    import torch
    from tropidist_gb300 import _lib
    L = _lib.lib()
    base = np.arange(5000, dtype=np.uint32)
    for src, dst, nbytes in ((4000, 0, 4000), (100, 40, 8000), (0, 3000, 6000), (12, 4, 9000), (0, 10000, 100)):
        buf = _dev(base.view(np.uint8))
        want = base.view(np.uint8).copy()
        want[dst:dst + nbytes] = base.view(np.uint8)[src:src + nbytes].copy()
        assert L.tree_move(buf.data_ptr() + dst, buf.data_ptr() + src, nbytes) == 0
        torch.cuda.synchronize()
        assert np.array_equal(buf.cpu().numpy(), want), (src, dst, nbytes)


def test_block_product_joins(td):
    """Joins whose kernel generators are unit pairs and whose parents cover every pair of child
    blocks run as min-plus block products (k_tree_gemm): against the oracle where it is affordable,
    against the per-pair kernel elsewhere, on several targets each."""
    from tropidist_gb300 import synth
    rng = random.Random(12)
    seen = 0
    # chunks of 32 (F >= 5), 16 (F = 4), 8 (F = 3) and 4 (F = 2) entries per staging step: these
    # trees run block products with F = 3 .. 9 and 2 (70 x 140, seeds 1 and 5)
    for (m, n, win, seed), check in (((60, 120, 12, 3), "oracle"), ((80, 160, 10, 2), "oracle"),
                                     ((80, 160, 12, 1), "oracle"), ((70, 140, 11, 1), "oracle"),
                                     ((70, 140, 11, 5), "oracle"), ((120, 240, 12, 7), "device"),
                                     ((90, 180, 11, 4), "device")):
        p = synth.banded(m, n, win, 3, 1, seed=seed)
        prog = td.CompiledTreeDP(p.h, balanced(list(range(n))))
        info = prog.device_info()
        assert info["block_product_joins"] >= 1
        seen += info["block_product_joins"]
        lim = dict(max_join_work=None, max_memory_bytes=None, max_seconds=None)
        for t in [rng.randrange(1 << m) for _ in range(4)]:
            got = prog.run(t, **lim)[0]
            want = ot.run(prog, t) if check == "oracle" else prog.run(t, gemm=False, **lim)[0]
            assert got == want, ((m, n, seed), t)
        prog.free()
    assert seen >= 14
