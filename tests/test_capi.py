"""The C-ABI library loads and exports every function that include/tropidist_gb300.h declares."""
import os
import re

from helpers import ROOT


def declared_functions():
    text = open(os.path.join(ROOT, "include", "tropidist_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"typedef[^;]*;", "", text)            # function-pointer types are not exports
    names = re.findall(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(", text)
    return sorted({n for n in names if n not in ("if", "sizeof")})


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_library_reports_version_and_errors(lib):
    assert lib.tg_version() >= 1
    assert lib.tg_dense_set_tuning(99, 99, 99, 99) == -1
    assert b"tuning" in lib.tg_last_error()


def test_witness_sizes_count_every_table_of_the_sweep(lib):
    """tg_dense_witness_bytes (host only): the bytes of the tables T_0 .. T_n of a sweep, and -1 for
    an op stream whose width leaves 0..30."""
    import numpy as np
    from tropidist_gb300 import synth, trellis
    p = synth.dense_small(3)
    plan = trellis.build_plan(p.h, p.l, 1, list(range(p.ncols)), p.nrows)
    enc = np.ascontiguousarray(plan.encode(), dtype=np.int64)
    w, tot = 0, 1
    for code in enc[:, 0].tolist():
        w += 1 if code == trellis.OP_EXPAND else -1 if code == trellis.OP_SELECT else 0
        tot += 1 << w
    assert lib.tg_dense_witness_bytes(enc.ctypes.data, len(enc), 1) == tot
    assert lib.tg_dense_witness_bytes(enc.ctypes.data, len(enc), 2) == 2 * tot
    bad = np.array([[trellis.OP_SELECT, 0, 0]], dtype=np.int64)      # a select below width 0
    assert lib.tg_dense_witness_bytes(bad.ctypes.data, 1, 1) == -1
    assert lib.tg_dense_witness_bytes(enc.ctypes.data, len(enc), 3) == -1


def test_wide_walk_sizes_and_limit(lib):
    """Host-side sizing of the multi-word walk: the scratch grows with the capacity, the state
    words and the steps; the one-block limit reads back what was set."""
    s = [lib.tg_spw_walk_scratch_bytes(3, cap, 100) for cap in (1 << 10, 1 << 12, 1 << 14)]
    assert 0 < s[0] < s[1] < s[2]
    assert lib.tg_spw_walk_scratch_bytes(2, 1 << 12, 100) < lib.tg_spw_walk_scratch_bytes(8, 1 << 12, 100)
    assert lib.tg_spw_walk_scratch_bytes(3, 1 << 12, 10) < lib.tg_spw_walk_scratch_bytes(3, 1 << 12, 1000)
    assert lib.tg_spw_walk_scratch_bytes(9, 1 << 12, 10) < 0 and lib.tg_spw_walk_scratch_bytes(3, 0, 10) < 0
    old = lib.tg_spw_set_small_limit(-1)
    try:
        assert lib.tg_spw_set_small_limit(64) == old
        assert lib.tg_spw_set_small_limit(-1) == 64
    finally:
        lib.tg_spw_set_small_limit(old)
