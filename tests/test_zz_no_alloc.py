"""The allocation-free whole-plan entry point, tg_dense_run_noalloc.

Some callers of this library cannot allocate device memory: a runtime that owns the whole
device-memory budget and hands out only the buffers it planned for, or a caller on a
latency-critical stream where cudaMalloc would synchronize the device.  For them the executor's
second (ping-pong) table lives in a fixed array inside the library.  This test calls that entry
point through the C-ABI twice in a row on each plan and checks both results, and the whole table
buffer it was given, against the ordinary entry point, tg_dense_run, bit for bit.  The file sorts last so that a run stopping at the first
failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _plans():
    from tropidist_gb300 import synth, trellis
    out = []
    for seed in range(3):
        p = synth.dense_small(seed)
        out.append(trellis.build_plan(p.h, p.l, 1, list(range(p.ncols)), p.nrows))
    p = synth.banded(300, 600, 22, 3, 1, seed=5)          # fused passes, peak about 19 bits
    out.append(trellis.build_plan(p.h, p.l, 1, list(range(p.ncols)), p.nrows))
    p = synth.banded(300, 600, 24, 3, 1, seed=2)          # peak exactly 22 bits: the whole scratch
    out.append(trellis.build_plan(p.h, p.l, 1, list(range(p.ncols)), p.nrows))
    return [pl for pl in out if pl.feasible]


def test_noalloc_matches_allocating_entry_point_twice():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from tropidist_gb300 import _lib
    L = _lib.lib()
    stream = torch.cuda.current_stream().cuda_stream
    plans = _plans()
    assert any(pl.peak_bits > 16 for pl in plans)
    assert any(pl.peak_bits == 22 for pl in plans)          # the largest plan the scratch holds
    wants = []
    for plan in plans:
        ops = np.ascontiguousarray(plan.encode())
        n = 1 << plan.peak_bits
        a = torch.full((n,), 77, dtype=torch.uint8, device="cuda")
        b = torch.full((n,), 77, dtype=torch.uint8, device="cuda")
        want = ctypes.c_uint32(0)
        assert L.tg_dense_run(ops.ctypes.data, len(ops), 1, a.data_ptr(), b.data_ptr(), ctypes.byref(want), stream) == 0
        wants.append(want.value)
        table = torch.full((n,), 77, dtype=torch.uint8, device="cuda")
        for rep in range(2):
            got = ctypes.c_uint32(12345)
            st = L.tg_dense_run_noalloc(ops.ctypes.data, len(ops), table.data_ptr(), n, ctypes.byref(got), stream)
            assert st == 0, L.tg_last_error()
            assert got.value == want.value, (plan.peak_bits, got.value, want.value)
            if rep == 0:
                # the same schedule over the same start contents: the caller's table holds, byte
                # for byte, what the allocating entry point left in its first buffer (the tables
                # of every other pass of the sweep, the last of them whole)
                assert torch.equal(table, a), plan.peak_bits
    # the scratch keeps the last call's contents: calls alternating between plans of different
    # widths still agree with the allocating entry point
    for plan, want in list(zip(plans, wants))[::-1] + list(zip(plans, wants)):
        ops = np.ascontiguousarray(plan.encode())
        n = 1 << plan.peak_bits
        table = torch.full((n,), 200, dtype=torch.uint8, device="cuda")
        got = ctypes.c_uint32(12345)
        assert L.tg_dense_run_noalloc(ops.ctypes.data, len(ops), table.data_ptr(), n, ctypes.byref(got), stream) == 0
        assert got.value == want


def test_noalloc_refuses_plans_beyond_its_scratch():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from tropidist_gb300 import _lib, synth, trellis
    L = _lib.lib()
    p = synth.banded(500, 1000, 30, 3, 1, seed=3)          # peak above 22 bits
    plan = trellis.build_plan(p.h, p.l, 1, list(range(p.ncols)), p.nrows)
    assert plan.peak_bits > 22
    ops = np.ascontiguousarray(plan.encode())
    small = torch.empty(16, dtype=torch.uint8, device="cuda")
    got = ctypes.c_uint32(0)
    st = L.tg_dense_run_noalloc(ops.ctypes.data, len(ops), small.data_ptr(), 16, ctypes.byref(got),
                                torch.cuda.current_stream().cuda_stream)
    assert st == -4 and b"2^22" in L.tg_last_error()
