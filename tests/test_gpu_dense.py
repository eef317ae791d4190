"""Dense Rank DP on the GPU, through the C-ABI, against the reference's outputs and the oracle."""
import ctypes
import random

import numpy as np
import pytest

from helpers import golden, ops_from_json, port_run, sha, unhex
from oracle import dense as od

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def gpu():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from tropidist_gb300 import _lib
    _lib.lib()
    yield
    _lib.lib().tg_dense_set_tuning(16, 15, 15, 14)


TUNINGS = [(16, 15, 15, 14), (12, 11, 10, 9), (8, 7, 6, 5), (6, 5, 4, 3)]


@pytest.fixture(autouse=True)
def default_tuning():
    from tropidist_gb300 import _lib
    _lib.lib().tg_dense_set_tuning(*TUNINGS[0])
    _lib.lib().tg_dense_set_stream_span(3, 2)
    yield
    _lib.lib().tg_dense_set_stream_span(3, 2)


def gpu_tables(plan, ks, dtype="u8"):
    from tropidist_gb300 import kernel
    cp = kernel.CompiledPlan(plan, dtype, ks)
    a, b = cp.buffers()
    outs = [kernel.device.empty((1 << kernel._width_after(plan.ops, k)) * cp.eb) for k in cp.ckpts]
    cp.execute(a, b, outs)
    v = cp.result(a, b)
    torch.cuda.synchronize()
    dt = np.uint8 if cp.eb == 1 else np.uint16
    tabs = [o.cpu().numpy().view(dt) for o in outs]
    cp.free()
    return v, tabs


def test_run_plan_random_matches_reference():
    from tropidist_gb300 import kernel
    from tropidist_gb300.trellis import Plan
    for case in golden("dense_random.json"):
        plan = Plan(ops_from_json(case["ops"]), case["peak_bits"], [], 0, feasible=case["feasible"])
        v, _ = kernel.run_plan(plan)
        assert v == case["value_c"] == case["brute"]


@pytest.mark.parametrize("tune", TUNINGS)
def test_checkpoint_tables_bit_identical(tune):
    from tropidist_gb300 import _lib
    from tropidist_gb300.trellis import Plan
    _lib.lib().tg_dense_set_tuning(*tune)
    for case in golden("dense_big.json"):
        if not case["feasible"]:
            continue
        plan = Plan(ops_from_json(case["ops"]), case["peak_bits"], [], 0)
        ks = sorted(int(k) for k in case["table_sha"])
        v, tabs = gpu_tables(plan, ks)
        assert v == case["value_c"]
        for k, t in zip(ks, tabs):
            assert sha(t) == case["table_sha"][str(k)], (tune, k)


@pytest.mark.parametrize("span", [(3, 3), (4, 3)])
@pytest.mark.parametrize("prob", [(120, 240, 24, 3), (160, 320, 26, 1)])
def test_lane_dimension_tables_bit_identical(prob, span):
    """Streaming passes whose updates span a fourth dimension across a lane pair (with and without
    an in-chunk part), and passes closing an in-chunk row with 3 dimensions: checkpoint tables and
    the value against the oracle."""
    from tropidist_gb300 import _lib, kernel, synth, trellis
    from oracle import dense as od
    _lib.lib().tg_dense_set_stream_span(*span)
    m, n, win, seed = prob
    p = synth.banded(m, n, win, seed=seed)
    plan = trellis.build_plan(p.h, p.l, 1, list(range(p.ncols)), p.nrows)
    ks = list(range(len(plan.ops) // 5, len(plan.ops), len(plan.ops) // 5))
    flags = [int(s[6]) for s in kernel.CompiledPlan(plan, "u8", ks).segments() if s[0] == 3]
    if span[0] == 4:
        assert sum(1 for f in flags if f & 32) > 0 and sum(1 for f in flags if f & 64) > 0
    v, tabs = gpu_tables(plan, ks)
    assert v == od.run_plan_numpy(plan)
    for k, t in zip(ks, tabs):
        assert np.array_equal(t, od.table_after(plan, k)), (prob, span, k)


def test_synth_checkpoints_and_values():
    from tropidist_gb300 import trellis
    for case in golden("dense_synth.json"):
        h, l = unhex(case["h"]), unhex(case["l"])
        plan = trellis.build_plan(h, l, 1, list(range(len(h))), case["nrows"])
        ks = [int(k) for k in case["table_sha"]]
        v, tabs = gpu_tables(plan, ks)
        assert v == case["value"]
        for k, t in zip(ks, tabs):
            assert sha(t) == case["table_sha"][str(k)]


def test_eight_bit_boundary():
    from tropidist_gb300 import auto, kernel, trellis
    from tropidist_gb300.problem import Problem
    for case in golden("dense_chain.json"):
        h, l = unhex(case["h"]), unhex(case["l"])
        n = case["n"]
        p = Problem("chain", case["nrows"], 1, h, l)
        plan = trellis.build_plan(h, l, 1, list(range(n)), case["nrows"])
        if case["value"] == "overflow":
            with pytest.raises(OverflowError):
                kernel.run_plan(plan)
            with pytest.raises(OverflowError):
                auto.dp_distance(p, list(range(n)), dtype="u8")
        else:
            assert kernel.run_plan(plan)[0] == n
        assert kernel.run_plan(plan, dtype="u16")[0] == n
    p = Problem("no logical", 1, 1, [1, 1], [1, 1])
    plan = trellis.build_plan(p.h, p.l, 1, [0, 1], p.nrows)
    assert kernel.run_plan(plan)[0] is None


def test_known_codes():
    from tropidist_gb300 import auto
    from tropidist_gb300.problem import Problem
    for case in golden("codes.json"):
        p = Problem(case["name"], case["nrows"], case["nobs"], unhex(case["h"]), unhex(case["l"]))
        best, per = auto.dp_distance(p, case["order"])
        assert best == case["distance"] == case["known"]
        assert per == case["per_obs"]


def test_weighted_and_uint16_plans():
    from tropidist_gb300 import kernel, trellis
    rng = random.Random(12)
    for _ in range(120):
        m, n = rng.randint(1, 9), rng.randint(1, 12)
        h = [rng.randrange(0, 1 << m) for _ in range(n)]
        l = [rng.randrange(0, 2) for _ in range(n)]
        w = [rng.randint(1, 3) for _ in range(n)]
        order = list(range(n))
        rng.shuffle(order)
        plan = trellis.build_plan(h, l, 1, order, m, weights=w)
        want = od.brute(h, l, 1, w)
        assert kernel.run_plan(plan)[0] == want
        assert kernel.run_plan(plan, dtype="u16")[0] == want


def test_per_op_dropin_functions_match_oracle():
    """dp_update / dp_update_w / dp_expand_update / dp_select / dp_fill / dp_hist on device
    tables against the numpy rules, over sizes 2^0..2^20 and random masks."""
    from tropidist_gb300 import _lib
    L = _lib.lib()
    L.tg_set_stream(None)
    rng = np.random.default_rng(3)
    for bits in list(range(0, 13)) + [16, 20]:
        n = 1 << bits
        T = rng.integers(0, 256, n, dtype=np.uint8)
        T[rng.random(n) < 0.2] = 255
        d = torch.from_numpy(T.copy()).cuda()
        ref = T.copy()
        for _ in range(6):
            if bits == 0:
                break
            h = int(rng.integers(1, n))
            w = int(rng.integers(1, 4))
            if w == 1:
                L.dp_update(d.data_ptr(), n, h)
            else:
                L.dp_update_w(d.data_ptr(), n, h, w)
            ref = od.apply_op(ref, ("update", h, w))
        torch.cuda.synchronize()
        assert np.array_equal(d.cpu().numpy(), ref), bits
        hist = np.zeros(256, dtype=np.uint64)
        L.dp_hist(d.data_ptr(), n, hist.ctypes.data)
        assert np.array_equal(hist, np.bincount(ref, minlength=256).astype(np.uint64))
        # expand with the starting column, then select
        big = torch.empty(2 * n, dtype=torch.uint8, device="cuda")
        big[:n] = d
        hl = int(rng.integers(0, n))
        L.dp_expand_update(big.data_ptr(), n, hl)
        exp = np.concatenate([ref, np.full(n, 255, np.uint8)])
        exp[n + (np.arange(n) ^ hl)] = np.where(ref == 255, 255, ref + 1).astype(np.uint8)
        torch.cuda.synchronize()
        assert np.array_equal(big.cpu().numpy(), exp), bits
        pos, tgt = int(rng.integers(0, bits + 1)), int(rng.integers(0, 2))
        assert L.dp_select(big.data_ptr(), 2 * n, pos, tgt) == n
        torch.cuda.synchronize()
        assert np.array_equal(big[:n].cpu().numpy(), od.apply_op(exp, ("select", pos, tgt)))
        L.dp_fill(big.data_ptr(), 2 * n, 7)
        torch.cuda.synchronize()
        assert int(big.min()) == int(big.max()) == 7
    assert L.dp_num_threads() >= 1


def test_uint16_per_op_functions():
    from tropidist_gb300 import _lib
    L = _lib.lib()
    rng = np.random.default_rng(4)
    for bits in (1, 3, 5, 9, 14):
        n = 1 << bits
        T = rng.integers(0, 65536, n).astype(np.uint16)
        T[rng.random(n) < 0.2] = 65535
        d = torch.from_numpy(T.view(np.int16).copy()).cuda()
        ref = T.copy()
        for _ in range(5):
            h, w = int(rng.integers(1, n)), int(rng.integers(1, 4))
            assert L.dp16_update(d.data_ptr(), n, h, w) == 0
            ref = od.apply_op(ref, ("update", h, w), inf=od.INF16)
        torch.cuda.synchronize()
        assert np.array_equal(d.cpu().numpy().view(np.uint16), ref)


def test_wide_banded_against_c_port():
    """A width-24 banded plan: final value and a checkpoint table against the C port."""
    from tropidist_gb300 import synth, trellis
    p = synth.banded(500, 1000, 28, 3, 1, seed=2)
    plan = trellis.build_plan(p.h, p.l, 1, list(range(p.ncols)), p.nrows)
    assert plan.peak_bits >= 20
    k = len(plan.ops) // 2
    v, tabs = gpu_tables(plan, [k])
    assert v == int(port_run(plan)[0])
    assert np.array_equal(tabs[0], port_run(plan, k))


def test_full_width_schedules_agree():
    """At the bench width (about 30 bits) the table after half of the ops and the final value do
    not depend on the fusion schedule: unfused one-op passes and 16-bit tiles agree bit for bit
    (a size-independent check; the CPU checker is too slow at this width)."""
    from tropidist_gb300 import _lib, synth, trellis
    p = synth.dense_scale(0, window=36)
    plan = trellis.build_plan(p.h, p.l, 1, list(range(p.ncols)), p.nrows)
    assert plan.peak_bits >= 29
    k = next(i for i in range(len(plan.ops)) if i > len(plan.ops) // 2 and
             sum(1 if o[0] == "expand" else -1 if o[0] == "select" else 0 for o in plan.ops[:i]) >= plan.peak_bits - 1)
    res = []
    for tune in ((16, 15, 15, 14), (9, 8, 15, 14)):
        _lib.lib().tg_dense_set_tuning(*tune)
        v, tabs = gpu_tables(plan, [k])
        t = torch.from_numpy(tabs[0])
        res.append((v, sha(tabs[0]), torch.bincount(t.long(), minlength=256)))
        del tabs
    assert res[0][0] == res[1][0] and res[0][1] == res[1][1]
    assert torch.equal(res[0][2], res[1][2])


@pytest.mark.parametrize("case", [(60, 120, 14, 3, None), (80, 160, 16, 5, None), (60, 120, 12, 7, (1, 2, 3))])
def test_witness_traceback_on_device(case, monkeypatch):
    """dp_witness: the one-launch traceback of small plans (every table kept on the device), and
    device checkpoints with a bisection traceback (small budgets forcing several checkpoints), give
    a logical of the distance's weight (zero syndrome, the observable flipped)."""
    from tropidist_gb300 import auto, synth
    from tropidist_gb300.problem import verify_witness
    m, n, win, seed, wts = case
    p = synth.banded(m, n, win, seed=seed, nobs=2)
    if wts is not None:
        import random
        rng = random.Random(seed)
        p.weights = [rng.choice(wts) for _ in range(p.ncols)]
    order = list(range(p.ncols))
    best, per = auto.dp_distance(p, order)
    for small, budget in ((True, None), (False, None), (False, 1 << 16)):
        monkeypatch.setattr(auto, "SMALL_WITNESS_BYTES", 256 << 20 if small else 0)
        r = auto.dp_witness(p, order, budget_bytes=budget, leaf=4)
        assert r["distance"] == best
        cols = r["witness"]
        assert verify_witness(p, cols, r["observable"])
        w = sum(p.weights[j] for j in cols) if getattr(p, "weights", None) is not None else len(cols)
        assert w == best
