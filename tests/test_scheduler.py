"""The launch scheduler of libtropigpu, checked on the CPU through its host emulation: every
fusion schedule reproduces the oracle's tables entry for entry."""
import random

import numpy as np
import pytest

from helpers import emulate, golden, ops_from_json, sha, unhex
from oracle import dense as od
from tropidist_gb300 import _lib, synth, trellis
from tropidist_gb300.trellis import Plan

TUNINGS = [(16, 15, 15, 14), (12, 11, 10, 9), (8, 7, 6, 5), (6, 5, 4, 3)]


@pytest.fixture(autouse=True)
def restore_tuning(lib):
    yield
    lib.tg_dense_set_tuning(*TUNINGS[0])
    lib.tg_dense_set_stream_span(3, 2)


@pytest.mark.parametrize("span", [(3, 3), (4, 3), (4, 2)])
def test_lane_dimension_schedules(lib, span):
    """Streaming passes with a lane-pair dimension: emulated schedules against the oracle's tables."""
    lib.tg_dense_set_stream_span(*span)
    rng = random.Random(5)
    for tune in TUNINGS[:3]:
        lib.tg_dense_set_tuning(*tune)
        for _ in range(30):
            m = rng.randint(8, 15)
            n = rng.randint(m + 3, m + 14)
            h = [rng.randrange(1, 1 << m) for _ in range(n)]
            l = [rng.randrange(0, 2) for _ in range(n)]
            plan = trellis.build_plan(h, l, 1, list(range(n)), m)
            if not plan.feasible:
                continue
            assert emulate(plan)[0] == od.run_plan_numpy(plan)
        for case in golden("dense_synth.json"):
            h, l = unhex(case["h"]), unhex(case["l"])
            plan = trellis.build_plan(h, l, 1, list(range(len(h))), case["nrows"])
            ks = [int(k) for k in case["table_sha"]]
            v, tabs, info = emulate(plan, checkpoints=ks)
            assert v == case["value"]
            for k, t in zip(ks, tabs):
                assert sha(t) == case["table_sha"][str(k)]
    # a wider banded plan: lane passes with and without an in-chunk part
    lib.tg_dense_set_tuning(*TUNINGS[0])
    p = synth.banded(120, 240, 24, seed=3)
    plan = trellis.build_plan(p.h, p.l, 1, list(range(p.ncols)), p.nrows)
    ks = list(range(len(plan.ops) // 4, len(plan.ops), len(plan.ops) // 4))
    v, tabs, info = emulate(plan, checkpoints=ks)
    assert v == od.run_plan_numpy(plan)
    for k, t in zip(ks, tabs):
        assert np.array_equal(t, od.table_after(plan, k))


def test_random_plans_all_tunings(lib):
    rng = random.Random(2)
    for tune in TUNINGS:
        lib.tg_dense_set_tuning(*tune)
        for _ in range(60):
            m = rng.randint(8, 15)
            n = rng.randint(m + 3, m + 14)
            h = [rng.randrange(1, 1 << m) for _ in range(n)]
            l = [rng.randrange(0, 2) for _ in range(n)]
            plan = trellis.build_plan(h, l, 1, list(range(n)), m)
            if not plan.feasible:
                continue
            want = od.run_plan_numpy(plan)
            assert emulate(plan)[0] == want
            assert emulate(plan, "u16")[0] == od.run_plan_numpy(plan, dtype=np.uint16)


def test_checkpoint_tables_match_reference(lib):
    for tune in TUNINGS:
        lib.tg_dense_set_tuning(*tune)
        for case in golden("dense_big.json")[:15]:
            if not case["feasible"]:
                continue
            plan = Plan(ops_from_json(case["ops"]), case["peak_bits"], [], 0)
            ks = sorted(int(k) for k in case["table_sha"])[1::3]
            v, tabs, _ = emulate(plan, checkpoints=ks)
            assert v == case["value_c"]
            for k, t in zip(ks, tabs):
                assert sha(t) == case["table_sha"][str(k)]


def test_synth_checkpoints(lib):
    for tune in TUNINGS:
        lib.tg_dense_set_tuning(*tune)
        for case in golden("dense_synth.json"):
            h, l = unhex(case["h"]), unhex(case["l"])
            plan = trellis.build_plan(h, l, 1, list(range(len(h))), case["nrows"])
            ks = [int(k) for k in case["table_sha"]]
            v, tabs, info = emulate(plan, checkpoints=ks)
            assert v == case["value"]
            for k, t in zip(ks, tabs):
                assert sha(t) == case["table_sha"][str(k)]
    # a wider banded plan: lane passes with and without an in-chunk part
    lib.tg_dense_set_tuning(*TUNINGS[0])
    p = synth.banded(120, 240, 24, seed=3)
    plan = trellis.build_plan(p.h, p.l, 1, list(range(p.ncols)), p.nrows)
    ks = list(range(len(plan.ops) // 4, len(plan.ops), len(plan.ops) // 4))
    v, tabs, info = emulate(plan, checkpoints=ks)
    assert v == od.run_plan_numpy(plan)
    for k, t in zip(ks, tabs):
        assert np.array_equal(t, od.table_after(plan, k))


def test_weighted_and_wide_masks(lib):
    rng = random.Random(9)
    lib.tg_dense_set_tuning(6, 5, 4, 3)       # tiny tiles: many updates need the one-op pass
    for _ in range(40):
        m = rng.randint(6, 12)
        n = rng.randint(m + 2, m + 10)
        h = [rng.randrange(1, 1 << m) for _ in range(n)]
        l = [rng.randrange(0, 2) for _ in range(n)]
        w = [rng.randint(1, 3) for _ in range(n)]
        plan = trellis.build_plan(h, l, 1, list(range(n)), m, weights=w)
        if not plan.feasible:
            continue
        assert emulate(plan)[0] == od.run_plan_numpy(plan)
        assert emulate(plan, "u16")[0] == od.run_plan_numpy(plan, dtype=np.uint16)


def test_mid_width_banded(lib):
    p = synth.banded(200, 400, 20, 3, 1, seed=4)
    plan = trellis.build_plan(p.h, p.l, 1, list(range(p.ncols)), p.nrows)
    assert plan.peak_bits >= 16
    v, _, (npass, nsweep) = emulate(plan)
    assert npass > 0
    assert v == od.run_plan_numpy(plan)


def test_bad_op_streams_are_rejected(lib):
    import ctypes
    bad = [
        [(1, 1, 1)],                 # update on a width-0 table
        [(0, 0, 0), (2, 1, 0)],      # select beyond the width
        [(0, 0, 0)],                 # does not end at width 0
        [(0, 0, 0), (1, 1, 0), (2, 0, 1)],   # weight 0
        [(7, 0, 0)],
    ]
    for ops in bad:
        arr = np.array(ops, dtype=np.int64)
        st = ctypes.c_int(0)
        h = lib.tg_dense_plan(arr.ctypes.data, len(arr), 1, None, 0, ctypes.byref(st))
        assert not h and st.value == -1


def test_random_checkpoint_sets(lib):
    """Random checkpoint sets over random plans and tunings: every table at a checkpoint is in
    the canonical layout and equals the oracle's, whatever layouts the passes chose between."""
    rng = random.Random(21)
    for trial in range(60):
        lib.tg_dense_set_tuning(*rng.choice(TUNINGS))
        m = rng.randint(40, 140)
        p = synth.banded(m, rng.randint(2 * m, 3 * m), rng.randint(6, 18), 3, 1, seed=rng.randrange(1 << 30))
        plan = trellis.build_plan(p.h, p.l, 1, list(range(p.ncols)), p.nrows)
        if not plan.feasible or plan.peak_bits > 17:
            continue
        ks = sorted(rng.sample(range(1, len(plan.ops) + 1), min(len(plan.ops), rng.randint(1, 12))))
        tabs_ref = []
        want = od.run_plan_numpy(plan, tables=tabs_ref)
        v, tabs, _ = emulate(plan, checkpoints=ks)
        assert v == want
        for k, t in zip(ks, tabs):
            assert np.array_equal(t, tabs_ref[k - 1]), (trial, k)


def test_plans_from_a_given_table(lib):
    """Plans that start from a table of the sweep (tg_dense_plan_from) reproduce the oracle's table
    at the end of any op range, under every tuning (emulated on the host)."""
    import ctypes
    from tropidist_gb300 import kernel
    rng = random.Random(11)
    for tune in TUNINGS[:3]:
        lib.tg_dense_set_tuning(*tune)
        p = synth.banded(60, 120, 14, seed=rng.randrange(1000))
        plan = trellis.build_plan(p.h, p.l, 1, list(range(p.ncols)), p.nrows)
        if not plan.feasible:
            continue
        enc = plan.encode()
        n = len(plan.ops)
        for _ in range(6):
            lo = rng.randrange(0, n - 1)
            hi = rng.randrange(lo + 1, n + 1)
            t_lo = od.table_after(plan, lo)
            want = od.table_after(plan, hi)
            cp = kernel.CompiledPlan(None, "u8", (), w_start=int(np.log2(len(t_lo))) if lo else 0, ops=enc[lo:hi])
            size = 1 << max(cp.peak_bits, 1)
            a = np.zeros(size, dtype=np.uint8)
            b = np.zeros(size, dtype=np.uint8)
            a[:len(t_lo)] = t_lo
            arr = (ctypes.c_void_p * 1)()
            _lib.check(lib.tg_debug_emulate_dense(cp.handle, a.ctypes.data, b.ctypes.data, arr))
            got = (b if cp.final_buf else a)[:len(want)]
            assert np.array_equal(got, want), (tune, lo, hi)
            cp.free()
