"""Completion tables: hashes and entry counts against the reference's builds; device tables (GPU)
against the enumeration oracle."""
import random

import numpy as np
import pytest

from helpers import golden, unhex
from oracle import table as ot
from tropidist_gb300 import search
from tropidist_gb300.problem import Problem


def _problem(case):
    return Problem("tab", case["m"], case["nobs"], unhex(case["h"]), case["l"])


def test_hashes_match_reference():
    for case in golden("tables.json"):
        p = _problem(case)
        rh = search.row_hashes(p.nrows, case["seed"])
        zh, zl = search.column_hashes(p.h, rh)
        assert [format(int(x), "x") for x in zh] == case["zh"]
        assert [format(int(x), "x") for x in zl] == case["zl"]


def test_oracle_entry_counts_match_reference():
    for case in golden("tables.json"):
        zl = unhex(case["zl"])
        ent = ot.entries(unhex(case["zh"]), zl, case["l"], case["k"])
        assert len(ent) == case["entries"]


@pytest.mark.gpu
def test_device_tables_match_reference_and_oracle():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    for case in golden("tables.json"):
        p = _problem(case)
        T = search.Table(p, case["k"], seed=case["seed"])
        assert T.log2slots == case["log2slots"] and T.entries == case["entries"]
        ent = ot.entries(T.zh, T.zl, T.lg, case["k"])
        syn = [int(q["syn"], 16) for q in case["probes"]]
        lab = [q["lg"] for q in case["probes"]]
        R = [q["R"] for q in case["probes"]]
        got = T.lookup_syndromes(syn, lab, R)
        zh, zl = T.hashes_for(syn)
        want = [ot.lookup(ent, zl[i], lab[i], R[i]) for i in range(len(syn))]
        assert got.tolist() == want
        T.free()


@pytest.mark.gpu
def test_wide_and_labelfree_tables():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    rng = random.Random(8)
    m, n, nobs = 30, 40, 20
    h = [sum(1 << r for r in rng.sample(range(m), rng.randint(1, 3))) for _ in range(n)]
    l = [rng.randrange(0, 1 << nobs) for _ in range(n)]
    p = Problem("wide", m, nobs, h, l)
    for labelfree in (False, True):
        T = search.Table(p, 2, labelfree=labelfree)
        assert T.wide == (not labelfree)
        ent = ot.entries(T.zh, T.zl, T.lg, 2, wide=T.wide)
        assert T.entries == len(ent)
        probes = [rng.sample(range(n), rng.randint(1, 3)) for _ in range(100)]
        syn, lab = [], []
        for cols in probes:
            s = g = 0
            for j in cols:
                s ^= h[j]
                g ^= l[j]
            syn.append(s)
            lab.append(g if not labelfree else 1)
        got = T.lookup_syndromes(syn, lab, 2)
        zh, zl = T.hashes_for(syn)
        want = [ot.lookup(ent, zl[i], lab[i], 2, wide=T.wide) for i in range(len(syn))]
        assert got.tolist() == want
        T.free()


@pytest.mark.gpu
def test_reference_named_table_entry_points():
    """tab_create / tab_build / tab_count / tab_free with the reference's own names and arity
    (cdist/search.py:58-67), called as its ctypes binding calls them: the reference's entry counts."""
    import ctypes
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from tropidist_gb300 import _lib
    L = _lib.lib()
    for case in golden("tables.json"):
        zh = np.array(unhex(case["zh"]), dtype=np.uint64)
        zl = np.array(unhex(case["zl"]), dtype=np.uint64)
        lg = np.array(case["l"], dtype=np.uint64)
        t = L.tab_create(case["log2slots"], 0)
        assert t
        L.tab_build(t, len(zh), zh.ctypes.data, zl.ctypes.data, lg.ctypes.data, case["k"])
        assert L.tab_count(t) == case["entries"]
        L.tab_free(t)
