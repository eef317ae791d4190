"""Host planning: the trellis op streams are identical to the reference's."""
from helpers import golden, ops_from_json, sha, unhex
import numpy as np
from tropidist_gb300 import auto, synth, trellis
from tropidist_gb300.problem import Problem


def test_plans_identical_to_reference_random():
    for case in golden("dense_random.json"):
        plan = trellis.build_plan(case["h"], case["l"], case["obs_mask"], case["order"], case["m"])
        assert plan.feasible == case["feasible"]
        assert plan.ops == ops_from_json(case["ops"])
        assert plan.peak_bits == case["peak_bits"] and plan.work() == case["work"]


def test_plans_identical_to_reference_big():
    for case in golden("dense_big.json"):
        plan = trellis.build_plan(case["h"], case["l"], 1, list(range(len(case["h"]))), case["m"])
        assert plan.ops == ops_from_json(case["ops"])


def test_synth_problems_reproduce_and_plan_identically():
    for case in golden("dense_synth.json"):
        p = synth.dense_small(case["seed"])
        assert [format(x, "x") for x in p.h] == case["h"] and [format(x, "x") for x in p.l] == case["l"]
        plan = trellis.build_plan(p.h, p.l, 1, list(range(p.ncols)), p.nrows)
        assert sha(plan.encode()) == case["ops_sha"] and len(plan.ops) == case["nops"]


def test_codes_cut_rank():
    for case in golden("codes.json"):
        h = unhex(case["h"])
        assert max(trellis.cut_profile(h, case["order"])) == case["cut_rank"]


def test_encode_roundtrip_and_limits():
    p = synth.dense_small(0)
    plan = trellis.build_plan(p.h, p.l, 1, list(range(p.ncols)), p.nrows)
    enc = plan.encode()
    assert enc.shape == (len(plan.ops), 3) and enc.dtype == np.int64
    for row, op in zip(enc, plan.ops):
        assert row[0] == {"expand": 0, "update": 1, "select": 2}[op[0]]
    import pytest
    with pytest.raises(ValueError):
        trellis.encode_ops([("update", 1 << 63)])


def test_infeasible_query():
    p = Problem("no logical", 1, 1, [1, 1], [1, 1], [(0, 0)])
    plan = trellis.build_plan(p.h, p.l, 1, [0, 1], p.nrows)
    assert not plan.feasible


def test_estimate_counts_work():
    p = synth.dense_small(1)
    est = auto.estimate(p, list(range(p.ncols)))
    plan = trellis.build_plan(p.h, p.l, 1, list(range(p.ncols)), p.nrows)
    assert est["work"] == plan.work() and est["peak_bits"] == plan.peak_bits


def test_rank_profile_host_routine_matches_restatement():
    """The library's bitset rank profile equals the Python restatement of cdist/trellis.py:20-36."""
    import random
    from tropidist_gb300 import synth, trellis
    rng = random.Random(4)
    for _ in range(30):
        n = rng.randint(1, 80)
        h = [rng.randrange(0, 1 << rng.randint(1, 70)) for _ in range(n)]
        order = list(range(n))
        rng.shuffle(order)
        assert trellis.rank_profile(h, order) == trellis.rank_profile_py(h, order)
    p = synth.circuit_dem(seed=2, rounds=6, checks=20, ncols=800)
    order = list(range(p.ncols))
    assert trellis.rank_profile(p.h, order) == trellis.rank_profile_py(p.h, order)


def test_cpp_planner_matches_python_planner():
    """tg_make_plan (C++) builds the op stream, widths and update positions of make_plan_py."""
    import random
    from tropidist_gb300 import trellis
    rng = random.Random(3)
    for t in range(200):
        m, n = rng.randint(1, 12), rng.randint(1, 40)
        h = [rng.randrange(1 << m) for _ in range(n)]
        l = [rng.randrange(2) for _ in range(n)]
        order = list(range(n))
        rng.shuffle(order)
        hrows = trellis.minimal_span_form(trellis.rows_from_columns(h, order, m))
        lrow = trellis.reduce_target_row(trellis.target_row(l, 1, order), hrows)
        w = [rng.randint(1, 3) for _ in range(n)] if t % 3 == 0 else None
        a, b = trellis.make_plan(hrows, lrow, n, w), trellis.make_plan_py(hrows, lrow, n, w)
        assert a.feasible == b.feasible
        if a.feasible:
            assert a.ops == b.ops and a.peak_bits == b.peak_bits and a.widths == b.widths
            assert a.columns == b.columns and a.work() == b.work()
            assert (a.encode() == b.encode()).all()


def test_planner_edge_cases():
    import pytest
    from tropidist_gb300 import trellis
    # 70 nested rows open at once: a mask on a row beyond position 63 is refused as by encode()
    n = 160
    hrows = [(1 << i) | (1 << (n - 1 - i)) for i in range(70)]
    lrow = (1 << 70) | (1 << 89)
    a = trellis.make_plan_py(hrows, lrow, n)
    with pytest.raises(ValueError):
        a.encode()
    with pytest.raises(ValueError):
        trellis.make_plan(hrows, lrow, n)
    # an infeasible query and an empty problem
    assert not trellis.make_plan([1], 0, 1).feasible
    ptr, pos = trellis.bit_positions([])
    assert ptr.tolist() == [0] and pos.size == 0
    ptr, pos = trellis.bit_positions([0, 5, 0, 1 << 200])
    assert ptr.tolist() == [0, 0, 2, 2, 3] and pos.tolist() == [0, 2, 200]
