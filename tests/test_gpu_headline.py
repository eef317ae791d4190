"""The benchmark's dense workload at full size (31-bit frontier, 2 GB tables) against the
reference's own results on it (tests/golden/headline.json, written by running the reference's
planner and C kernels): per observable the op stream, the distance, and the table at two
checkpoints near full width, entry for entry (sha256) and as a value histogram."""
import hashlib

import numpy as np
import pytest

from helpers import golden

torch = pytest.importorskip("torch")


def _plans():
    from tropidist_gb300 import synth, trellis
    p = synth.dense_scale(0, window=37)
    order = list(range(p.ncols))
    return [trellis.build_plan(p.h, p.l, 1 << o, order, p.nrows) for o in range(p.nobs)]


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()[:16]


def test_headline_plans_match_reference():
    """The package's planner and the oracle's restatement give the reference's op streams."""
    from oracle import plan as oplan
    from tropidist_gb300 import synth
    p = synth.dense_scale(0, window=37)
    order = list(range(p.ncols))
    for case, pl in zip(golden("headline.json")["cases"], _plans()):
        assert pl.peak_bits == case["peak_bits"] == 31
        assert pl.work() == case["work"] and len(pl.ops) == case["nops"]
        assert _sha(pl.encode()) == case["ops_sha"]
        q = oplan.plan(p.h, p.l, 1 << case["observable"], order, p.nrows)
        assert _sha(q.encoded()) == case["ops_sha"]


@pytest.mark.gpu
def test_headline_tables_and_distances_match_reference():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from tropidist_gb300 import _lib, device, kernel
    _lib.lib().tg_dense_set_tuning(16, 15, 15, 14)
    _lib.lib().tg_dense_set_stream_span(3, 2)
    for case, pl in zip(golden("headline.json")["cases"], _plans()):
        ks = sorted(int(k) for k in case["tables"])
        cp = kernel.CompiledPlan(pl, "u8", ks)
        a, b = cp.buffers()
        outs = [device.empty(case["tables"][str(k)]["entries"]) for k in cp.ckpts]
        cp.execute(a, b, outs)
        assert cp.result(a, b) == case["value"], case["observable"]
        torch.cuda.synchronize()
        for k, o in zip(cp.ckpts, outs):
            want = case["tables"][str(k)]
            t = o.cpu().numpy()
            assert t.size == want["entries"]
            assert np.bincount(t, minlength=256).tolist() == want["hist"], (case["observable"], k)
            assert _sha(t) == want["sha"], (case["observable"], k)
            del t
        del outs, a, b
        cp.free()
        torch.cuda.empty_cache()
