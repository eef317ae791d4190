"""The weight-bounded search (tg_search) with its probes answered by the oracle's completion table:
against the reference's own search (tests/golden/search.json, written by tests/golden/make_golden.py
from cdist/search.py), brute force, and known code distances (tests/golden/codes.json)."""
import itertools
import json
import os
import random

import numpy as np
import pytest

from helpers import ROOT
from oracle import table as otab
from tropidist_gb300 import search
from tropidist_gb300.problem import Problem

GOLD = json.load(open(os.path.join(ROOT, "tests", "golden", "search.json")))
CODES = json.load(open(os.path.join(ROOT, "tests", "golden", "codes.json")))


def oracle_probe(p, k, seed=12345):
    zh, zl = search.column_hashes(p.h, search.row_hashes(p.nrows, seed))
    wide = p.nobs > 16
    tab = otab.entries(zh, zl, np.array(p.l, dtype=np.uint64), k, wide=wide)

    def probe(pzh, pzl, plg, R):
        return [otab.lookup(tab, a, b, c, wide=wide) for a, b, c in zip(pzl, plg, R)]
    return probe


def problem(m, n, nobs, h, l, name="p"):
    return Problem(name, m, nobs, list(h), list(l), [(i, 0) for i in range(m)])


def brute(h, l):
    for w in range(1, len(h) + 1):
        for cols in itertools.combinations(range(len(h)), w):
            x = g = 0
            for j in cols:
                x ^= h[j]
                g ^= l[j]
            if x == 0 and g != 0:
                return w
    return None


@pytest.mark.parametrize("case", range(len(GOLD)))
def test_reference_search_distances(case):
    c = GOLD[case]
    p = problem(c["m"], c["n"], c["nobs"], c["h"], c["l"])
    r = search.distance(p, k_table=c["k_table"], kmax=c["kmax"], probe=oracle_probe(p, c["k_table"]), wave=64)
    assert r["distance"] == c["distance"]
    assert r["lower_bound"] == c["lower_bound"]
    for s in r["solutions"]:
        syn, lg = p.check(list(s))
        assert syn == 0 and lg != 0 and len(s) == r["distance"]


def test_brute_force_every_table_depth_and_wave():
    rng = random.Random(5)
    for t in range(120):
        m, n, nobs = rng.randint(1, 10), rng.randint(1, 13), rng.randint(1, 3)
        h = [rng.randrange(1 << m) for _ in range(n)]
        l = [rng.randrange(1 << nobs) for _ in range(n)]
        p = problem(m, n, nobs, h, l)
        k = t % 3
        r = search.distance(p, k_table=k, kmax=n, probe=oracle_probe(p, k), wave=1 + t % 9)
        assert r["distance"] == brute(h, l), t
        if r["distance"] is not None:
            (s,) = r["solutions"]
            syn, lg = p.check(list(s))
            assert syn == 0 and lg != 0 and len(s) == r["distance"]


@pytest.mark.parametrize("name", ["bb72_Z", "surface_d9_Z"])
def test_known_code_distances(name):
    c = next(x for x in CODES if x["name"] == name)
    h = [int(x, 16) if isinstance(x, str) else int(x) for x in c["h"]]
    l = [int(x, 16) if isinstance(x, str) else int(x) for x in c["l"]]
    p = problem(c["nrows"], len(h), c["nobs"], h, l, name)
    r = search.distance(p, k_table=2, kmax=c["distance"], probe=oracle_probe(p, 2))
    assert r["distance"] == c["distance"]
    assert [x["status"] for x in r["runs"]] == ["exhausted"] * (c["distance"] - 1) + ["found"]


def test_unsupported_modes_raise():
    p = problem(2, 3, 1, [1, 2, 3], [1, 0, 0])
    with pytest.raises(NotImplementedError):
        search.distance(p, enum_all=True, probe=oracle_probe(p, 2))
    with pytest.raises(NotImplementedError):
        search.distance(p, labelfree=True, probe=oracle_probe(p, 2))


def test_time_limit_start_and_orders():
    c = next(x for x in CODES if x["name"] == "bb72_Z")
    h = [int(x, 16) if isinstance(x, str) else int(x) for x in c["h"]]
    l = [int(x, 16) if isinstance(x, str) else int(x) for x in c["l"]]
    p = problem(c["nrows"], len(h), c["nobs"], h, l, "bb72")
    probe = oracle_probe(p, 2)
    # a certified lower bound as the start skips the thresholds below it
    r = search.distance(p, k_table=2, kmax=6, start=5, probe=probe)
    assert r["distance"] == 6 and [x["K"] for x in r["runs"]] == [5, 6]
    # any rank order and the anchors in any order give the same distance
    rng = random.Random(3)
    rank = list(range(p.ncols))
    rng.shuffle(rank)
    anchors = sorted(range(p.ncols), key=lambda j: rank[j])
    r = search.distance(p, k_table=2, kmax=6, start=6, probe=probe, rank=rank, anchors=anchors)
    assert r["distance"] == 6
    # a time limit passed during a wave stops the threshold with status "timeout" and no distance
    slow = lambda zh, zl, lg, R: (__import__("time").sleep(0.01), probe(zh, zl, lg, R))[1]
    r = search.distance(p, k_table=1, kmax=6, start=6, probe=slow, wave=2, time_limit=1e-6)
    assert r["runs"][-1]["status"] == "timeout" and r["distance"] is None and r["lower_bound"] == 6


def test_threads_share_anchors_with_the_same_results():
    rng = random.Random(11)
    for t in range(60):
        m, n, nobs = rng.randint(1, 10), rng.randint(1, 13), rng.randint(1, 3)
        h = [rng.randrange(1 << m) for _ in range(n)]
        l = [rng.randrange(1 << nobs) for _ in range(n)]
        p = problem(m, n, nobs, h, l)
        r = search.distance(p, k_table=t % 3, kmax=n, probe=oracle_probe(p, t % 3), wave=1 + t % 5, threads=4)
        assert r["distance"] == brute(h, l), t
        for s in r["solutions"]:
            syn, lg = p.check(list(s))
            assert syn == 0 and lg != 0 and len(s) == r["distance"]
    for name in ("bb72_Z", "surface_d9_Z"):
        c = next(x for x in CODES if x["name"] == name)
        h = [int(x, 16) if isinstance(x, str) else int(x) for x in c["h"]]
        l = [int(x, 16) if isinstance(x, str) else int(x) for x in c["l"]]
        p = problem(c["nrows"], len(h), c["nobs"], h, l, name)
        r = search.distance(p, k_table=2, kmax=c["distance"], probe=oracle_probe(p, 2), threads=8)
        assert r["distance"] == c["distance"]


def test_partner_exclusions_keep_the_distance():
    """Columns that sum to another column (with the label) are partners; forbidding them below each
    other changes no distance (a minimum logical never holds both) and prunes nodes."""
    rng = random.Random(21)
    pruned = 0
    for t in range(60):
        m, n, nobs = rng.randint(2, 8), rng.randint(3, 13), rng.randint(1, 2)
        h = [rng.randrange(1, 1 << m) for _ in range(n)]
        l = [rng.randrange(1 << nobs) for _ in range(n)]
        # plant sums: some columns are the XOR of two others (with their labels)
        for _ in range(rng.randint(0, 3)):
            a, b = rng.sample(range(len(h)), 2)
            h.append(h[a] ^ h[b])
            l.append(l[a] ^ l[b])
        p = problem(m, len(h), nobs, h, l)
        probe = oracle_probe(p, 1)
        a = search.distance(p, k_table=1, kmax=len(h), probe=probe, exclusions=True)
        b = search.distance(p, k_table=1, kmax=len(h), probe=probe, exclusions=False)
        assert a["distance"] == b["distance"] == brute(h, l), t
        na, nb = (sum(x["nodes"][0] for x in r["runs"]) for r in (a, b))
        assert na <= nb
        pruned += nb - na
        if a["exclusion_pairs"]:
            # partners lie on a zero-sum triple: a third column is their XOR, labels included
            ex_start, ex_cols, _ = search.partners(p)
            for f in range(p.ncols):
                for y in ex_cols[ex_start[f]:ex_start[f + 1]].tolist():
                    assert any(p.h[j] == p.h[f] ^ p.h[y] and p.l[j] == p.l[f] ^ p.l[y] for j in range(p.ncols))
    assert pruned > 0


def port_table(p, k, seed=12345):
    """oracle/table_port.c: the reference's completion table in C, and its native probe."""
    import ctypes
    import math
    from tropidist_gb300._sigs_extra import PROBE_FN
    lib = ctypes.CDLL(os.path.join(ROOT, "oracle", "table_port.so"))
    lib.tp_create.restype = ctypes.c_void_p
    lib.tp_create.argtypes = [ctypes.c_int]
    lib.tp_build.argtypes = [ctypes.c_void_p, ctypes.c_int] + [ctypes.c_void_p] * 3 + [ctypes.c_int]
    lib.tp_free.argtypes = [ctypes.c_void_p]
    zh, zl = search.column_hashes(p.h, search.row_hashes(p.nrows, seed))
    lg = np.array(p.l, dtype=np.uint64)
    total = sum(math.comb(p.ncols, i) for i in range(k + 1))
    t = lib.tp_create(max(10, math.ceil(math.log2(total / 0.5 + 1))))
    lib.tp_build(t, p.ncols, zh.ctypes.data, zl.ctypes.data, lg.ctypes.data, k)
    return lib, t, PROBE_FN(("tp_probe", lib))


def test_native_probe_with_the_c_table():
    rng = random.Random(31)
    for t in range(40):
        m, n, nobs = rng.randint(1, 10), rng.randint(1, 13), rng.randint(1, 3)
        h = [rng.randrange(1 << m) for _ in range(n)]
        l = [rng.randrange(1 << nobs) for _ in range(n)]
        p = problem(m, n, nobs, h, l)
        lib, tab, fn = port_table(p, 2)
        r = search.distance(p, k_table=2, kmax=n, probe_fn=fn, probe_ctx=tab, wave=1 + t % 7)
        lib.tp_free(tab)
        assert r["distance"] == brute(h, l), t
    c = next(x for x in CODES if x["name"] == "surface_d9_Z")
    h = [int(x, 16) if isinstance(x, str) else int(x) for x in c["h"]]
    l = [int(x, 16) if isinstance(x, str) else int(x) for x in c["l"]]
    p = problem(c["nrows"], len(h), c["nobs"], h, l, "d9")
    lib, tab, fn = port_table(p, 2)
    assert search.distance(p, k_table=2, kmax=9, probe_fn=fn, probe_ctx=tab)["distance"] == 9
    lib.tp_free(tab)


@pytest.mark.parametrize("cover", [True, "simple"])
def test_covering_bound_keeps_the_distance(cover):
    rng = random.Random(41)
    pruned = 0
    for t in range(80):
        m, n, nobs = rng.randint(1, 10), rng.randint(1, 13), rng.randint(1, 3)
        h = [rng.randrange(1 << m) for _ in range(n)]
        l = [rng.randrange(1 << nobs) for _ in range(n)]
        p = problem(m, n, nobs, h, l)
        lib, tab, fn = port_table(p, t % 3)
        r = search.distance(p, k_table=t % 3, kmax=n, probe_fn=fn, probe_ctx=tab, cover=cover)
        lib.tp_free(tab)
        assert r["distance"] == brute(h, l), t
        pruned += sum(x["cover_pruned"] for x in r["runs"])
    assert pruned > 0
    for name, d in (("bb72_Z", 6), ("surface_d9_Z", 9)):
        c = next(x for x in CODES if x["name"] == name)
        h = [int(x, 16) if isinstance(x, str) else int(x) for x in c["h"]]
        l = [int(x, 16) if isinstance(x, str) else int(x) for x in c["l"]]
        p = problem(c["nrows"], len(h), c["nobs"], h, l, name)
        lib, tab, fn = port_table(p, 2)
        a = search.distance(p, k_table=2, kmax=d, probe_fn=fn, probe_ctx=tab, cover=cover)
        b = search.distance(p, k_table=2, kmax=d, probe_fn=fn, probe_ctx=tab)
        lib.tp_free(tab)
        assert a["distance"] == b["distance"] == d
        assert sum(x["nodes"][0] for x in a["runs"]) <= sum(x["nodes"][0] for x in b["runs"])
