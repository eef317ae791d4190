"""Batched persistent launch: every plan's value equals the one-at-a-time executor's and the
reference's."""
import random

import pytest

from helpers import golden, ops_from_json, unhex

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def gpu():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")


def test_batch_of_reference_plans():
    from tropidist_gb300.batch import DenseBatch
    from tropidist_gb300.trellis import Plan
    cases = golden("dense_random.json") + golden("dense_big.json")
    plans = [Plan(ops_from_json(c["ops"]), c["peak_bits"], [], 0, feasible=c["feasible"]) for c in cases]
    vals = DenseBatch(plans).run()
    for c, v in zip(cases, vals):
        assert v == c["value_c"]


def test_batch_of_uneven_widths_matches_one_at_a_time():
    from tropidist_gb300 import kernel, synth, trellis
    from tropidist_gb300.batch import DenseBatch
    rng = random.Random(3)
    plans = []
    for k in range(24):
        m = rng.randint(60, 400)
        p = synth.banded(m, 2 * m, rng.randint(8, 24), 3, 1, seed=rng.randrange(1 << 30))
        plans.append(trellis.build_plan(p.h, p.l, 1, list(range(p.ncols)), p.nrows))
    assert max(pl.peak_bits for pl in plans) >= 18 and min(pl.peak_bits for pl in plans) <= 14
    b = DenseBatch(plans)
    for _ in range(2):
        vals = b.run()
        for pl, v in zip(plans, vals):
            assert v == kernel.run_plan(pl)[0]


def test_batched_distances_of_instances():
    from tropidist_gb300 import auto, synth
    from tropidist_gb300.batch import batched_dp_distances
    ps = synth.batch_instances(seed=1, count=6, wmin=12, wmax=20, max_obs=4)
    got = batched_dp_distances(ps)
    for p, g in zip(ps, got):
        assert g == auto.dp_distance(p, list(range(p.ncols)))


def test_bounded_wait_runs_out_and_returns_timeout():
    """A device wait for work bounded at one poll: the blocks that find no unit at once give up, the
    run returns TG_ERR_TIMEOUT (TimeoutError here) instead of waiting on, and the context stays
    usable: the same batch then gives the right value under the default bound."""
    from tropidist_gb300 import _lib, kernel, synth, trellis
    from tropidist_gb300.batch import DenseBatch
    p = synth.banded(200, 400, 20, 3, 1, seed=4)
    plan = trellis.build_plan(p.h, p.l, 1, list(range(p.ncols)), p.nrows)
    b = DenseBatch([plan])
    L = _lib.lib()
    try:
        assert L.tg_batch_set_spin_limit(1) == 0
        with pytest.raises(TimeoutError):
            b.run()
    finally:
        L.tg_batch_set_spin_limit(0)
    assert b.run() == [kernel.run_plan(plan)[0]]
