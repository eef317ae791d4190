"""The dense oracle (numpy restatement and C port) against the reference's own outputs."""
import numpy as np
import pytest

from helpers import golden, ops_from_json, port_run, sha, unhex
from oracle import dense as od
from tropidist_gb300 import trellis
from tropidist_gb300.trellis import Plan


def _plan(case):
    ops = ops_from_json(case["ops"])
    return Plan(ops, case["peak_bits"], [], 0, feasible=case["feasible"])


def test_numpy_oracle_matches_reference_values():
    for case in golden("dense_random.json"):
        plan = _plan(case)
        assert od.run_plan_numpy(plan) == case["value_numpy"] == case["value_c"] == case["brute"]


def test_numpy_oracle_tables_match_reference_tables():
    for case in golden("dense_big.json"):
        if not case["feasible"]:
            continue
        plan = _plan(case)
        tabs = []
        assert od.run_plan_numpy(plan, tables=tabs) == case["value_c"]
        for k, digest in case["table_sha"].items():
            assert sha(tabs[int(k) - 1]) == digest, k


def test_c_port_matches_reference_tables():
    for case in golden("dense_big.json")[:20]:
        if not case["feasible"]:
            continue
        plan = _plan(case)
        for k, digest in list(case["table_sha"].items())[::5]:
            assert sha(port_run(plan, int(k))) == digest
        assert int(port_run(plan)[0]) == case["value_c"]


def test_synth_tables_and_values():
    for case in golden("dense_synth.json")[:4]:
        h, l = unhex(case["h"]), unhex(case["l"])
        plan = trellis.build_plan(h, l, 1, list(range(len(h))), case["nrows"])
        assert plan.work() == case["work"] and plan.peak_bits == case["peak_bits"]
        tabs = []
        assert od.run_plan_numpy(plan, tables=tabs) == case["value"] == case["numpy_value"]
        for k, digest in case["table_sha"].items():
            assert sha(tabs[int(k) - 1]) == digest


def test_eight_bit_boundary():
    for case in golden("dense_chain.json"):
        h, l = unhex(case["h"]), unhex(case["l"])
        n = case["n"]
        plan = trellis.build_plan(h, l, 1, list(range(n)), case["nrows"])
        if case["value"] == "overflow":
            with pytest.raises(OverflowError):
                od.run_plan_numpy(plan)
        else:
            assert od.run_plan_numpy(plan) == case["value"] == n
        # 16-bit tables hold every chain distance
        assert od.run_plan_numpy(plan, dtype=np.uint16) == n


def test_weighted_oracle_against_brute_force():
    import random
    rng = random.Random(5)
    for _ in range(150):
        m, n = rng.randint(1, 7), rng.randint(1, 10)
        h = [rng.randrange(0, 1 << m) for _ in range(n)]
        l = [rng.randrange(0, 2) for _ in range(n)]
        w = [rng.randint(1, 3) for _ in range(n)]
        order = list(range(n))
        rng.shuffle(order)
        plan = trellis.build_plan(h, l, 1, order, m, weights=w)
        want = od.brute(h, l, 1, w)
        assert od.run_plan_numpy(plan) == want
        assert od.run_plan_numpy(plan, dtype=np.uint16) == want


def test_witness_oracle_matches_reference():
    for case in golden("codes.json")[:2]:
        h, l = unhex(case["h"]), unhex(case["l"])
        obs = case["per_obs"].index(case["distance"])
        wit = od.witness(h, l, case["order"], case["nrows"], obs,
                         lambda hh, o, nr: trellis.minimal_span_form(trellis.rows_from_columns(hh, o, nr)),
                         trellis.reduce_target_row, trellis.lowbit)
        assert wit == case["witness"]
