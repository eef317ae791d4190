"""Sparse Rank DP on device tables, against the reference's outputs and the numpy oracle."""
import itertools
import random

import numpy as np
import pytest

from helpers import golden, sha, unhex
from oracle.sparse import NumpyTables
from test_sparse_oracle import brute, check_witness

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def gpu():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")


def _problem(case):
    from tropidist_gb300.problem import Problem
    return Problem("rand", case["m"], case["k"], case["h"], case["l"])


def test_device_tables_at_every_cut_match_reference():
    from tropidist_gb300 import sparse_dp
    from tropidist_gb300.problem import Problem
    for case in golden("sparse_tables.json"):
        p = Problem("t", case["nrows"], 1, unhex(case["h"]), unhex(case["l"]))
        tr = sparse_dp.Trellis.for_query(p, 0, list(range(p.ncols)))
        sw = sparse_dp.Sweep(tr, +1 if case["forward"] else -1, case["K"], case["K"], use_h=case["use_h"], every=1,
                             backend="gpu")
        sw.run()
        assert sw.counts == case["counts"]
        for c, (n, hk, hv) in case["tables"].items():
            keys, vals = sw.be.arrays(sw.ckpt[int(c)])
            assert keys.size == n and sha(keys) == hk and sha(vals) == hv, c


def test_query_values_match_reference():
    from tropidist_gb300 import sparse_dp
    checked = 0
    for case in golden("sparse_random.json"):
        if not case["feasible"]:
            continue
        p = _problem(case)
        tr = sparse_dp.Trellis.for_query(p, case["obs"], case["order"])
        for run in case["runs"][::3]:
            r = sparse_dp.query(tr, run["K"], mode=run["mode"], split=run["split"], use_h=run["use_h"], backend="gpu")
            assert r["value"] == run["value"], run
            assert r["peak_states"] == run["peak_states"], run
            if run["value"] is not None:
                check_witness(p, r["witness"], run["value"], case["obs"])
            checked += 1
    assert checked > 300


def test_frontier_sweeps_match_oracle_cut_by_cut():
    """Meet-in-the-middle forward sweeps (frontier, falling caps, lookahead): every table and every
    changed set equal the oracle's, on seeded banded problems."""
    from tropidist_gb300 import sparse_dp, synth
    rng = random.Random(4)
    for seed in range(3):
        p = synth.dense_small(seed)
        tr = sparse_dp.Trellis.for_query(p, 0, list(range(p.ncols)))
        K = 6
        caps = sorted((rng.randint(1, K) for _ in range(tr.N + 1)), reverse=True)
        out = {}
        for name in ("gpu", "numpy"):
            be = "gpu" if name == "gpu" else NumpyTables(tr)
            sw = sparse_dp.Sweep(tr, +1, K, use_h=True, every=1, frontier=True, backend=be, caps=caps)
            rec = []

            def on_cut(c, tab, ch, extra, sw=sw, rec=rec):
                tk, tv = sw.be.arrays(tab)
                if ch is not None and name == "gpu" and hasattr(ch, "arr"):
                    x = ch.arr[:ch.n].cpu().numpy().view(np.uint64)
                    ck = np.sort(x & np.uint64((1 << 56) - 1))
                    cv = (x[np.argsort(x & np.uint64((1 << 56) - 1))] >> np.uint64(56)).astype(np.uint8)
                elif ch is not None:
                    ck, cv = ch
                else:
                    ck = cv = np.zeros(0)
                rec.append((c, sha(tk), sha(tv), sha(np.asarray(ck, dtype=np.uint64)), sha(np.asarray(cv, dtype=np.uint8))))
                return False

            sw.run(on_cut=on_cut)
            out[name] = rec
        assert out["gpu"] == out["numpy"]


def test_distance_matches_brute_force():
    from tropidist_gb300 import sparse_dp
    from tropidist_gb300.problem import Problem
    rng = random.Random(5)
    for _ in range(30):
        n, m, k = rng.randint(2, 12), rng.randint(1, 7), rng.randint(1, 2)
        dens = rng.choice([0.2, 0.35, 0.5])
        h = [sum(1 << r for r in range(m) if rng.random() < dens) for _ in range(n)]
        l = [sum(1 << r for r in range(k) if rng.random() < 0.4) for _ in range(n)]
        p = Problem("rand", m, k, h, l)
        truth = [brute(p, i) for i in range(k)]
        truth = min((t for t in truth if t is not None), default=None)
        order = list(range(n))
        rng.shuffle(order)
        for mode in ("forward", "mitm"):
            r = sparse_dp.distance(p, order=order, mode=mode, kmax=n + 1)
            assert r["distance"] == truth
            if truth is not None:
                check_witness(p, r["witness"], truth)


def test_eight_bit_boundary():
    """cdist's dp_boundary_check / dp_overflow_check (tests/test_false_bounds.py:205-231): a forward
    sweep keeps weights up to K: 254 is exact, 255 is refused; a meet in the middle holds 255."""
    from tropidist_gb300 import sparse_dp
    from tropidist_gb300.problem import Problem

    def chain(n):
        h = [1] + [(1 << (j - 1)) | (1 << j) for j in range(1, n - 1)] + [1 << (n - 2)]
        return Problem("chain", n - 1, 1, h, [1] + [0] * (n - 1))

    tr = sparse_dp.Trellis.for_query(chain(254), 0, list(range(254)))
    r = sparse_dp.query(tr, 254, mode="forward", use_h=False)
    assert r["value"] == 254 and r["witness"] == list(range(254))
    tr = sparse_dp.Trellis.for_query(chain(255), 0, list(range(255)))
    with pytest.raises(ValueError):
        sparse_dp.query(tr, 255, mode="forward", use_h=False)
    r = sparse_dp.query(tr, 255, mode="mitm", use_h=False)
    assert r["value"] == 255 and r["witness"] == list(range(255))
    tr = sparse_dp.Trellis.for_query(chain(510), 0, list(range(510)))
    with pytest.raises(ValueError):
        sparse_dp.query(tr, 510, mode="mitm", use_h=False, witness=False)


def test_weighted_columns():
    from tropidist_gb300 import sparse_dp
    from tropidist_gb300.problem import Problem
    rng = random.Random(17)
    for _ in range(25):
        n, m = rng.randint(2, 10), rng.randint(1, 6)
        h = [sum(1 << r for r in range(m) if rng.random() < 0.35) for _ in range(n)]
        l = [rng.randrange(0, 2) for _ in range(n)]
        wts = [rng.randint(1, 3) for _ in range(n)]
        p = Problem("w", m, 1, h, l, weights=wts)
        order = list(range(n))
        rng.shuffle(order)
        tr = sparse_dp.Trellis.for_query(p, 0, order)
        truth = brute(p, 0, wts)
        if not tr.feasible:
            continue
        for mode in ("forward", "mitm"):
            r = sparse_dp.query(tr, sum(wts) + 1, mode=mode)
            assert r["value"] == truth
            if truth is not None:
                assert sum(wts[j] for j in r["witness"]) == truth


def test_known_codes_by_sparse_mitm():
    from tropidist_gb300 import sparse_dp
    from tropidist_gb300.problem import Problem
    for case in golden("codes.json")[:2]:
        p = Problem(case["name"], case["nrows"], case["nobs"], unhex(case["h"]), unhex(case["l"]))
        d = case["distance"]
        r = sparse_dp.distance(p, order=case["order"], mode="mitm", start=d - 1)
        assert r["distance"] == d and r["lower_bound"] == d
        check_witness(p, r["witness"], d)
