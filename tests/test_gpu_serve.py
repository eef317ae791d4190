"""Serving: every request's distance is the same alone and in the continuous-batching mix."""
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def gpu():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")


def _requests(seed, count):
    from tropidist_gb300 import auto, synth
    from tropidist_gb300.serve import compile_request
    ps = synth.batch_instances(seed=seed, count=count, wmin=10, wmax=22, max_obs=4)
    reqs = []
    for k, p in enumerate(ps):
        plans = [pl for _, pl in auto._plans(p, list(range(p.ncols)))]
        reqs.append(compile_request(k, plans))
    return ps, reqs


def test_each_result_is_the_same_alone_and_in_the_mix():
    from tropidist_gb300 import auto
    from tropidist_gb300.serve import poisson_arrivals, serve_continuous, serve_plain
    ps, reqs = _requests(7, 24)
    alone = [auto.dp_distance(p, list(range(p.ncols)))[0] for p in ps]
    arr = poisson_arrivals(len(reqs), rate=2000.0, seed=1)
    done, wall, peak = serve_continuous(reqs, arr, slots=8)
    assert [r.distance for r in done] == alone
    assert peak > 1, "requests never overlapped"
    _, reqs2 = _requests(7, 24)
    done2, _ = serve_plain(reqs2, arr)
    assert [r.distance for r in done2] == alone


def test_budget_admission():
    from tropidist_gb300.serve import Server
    _, reqs = _requests(3, 6)
    small = min(r.footprint for r in reqs)
    srv = Server(slots=4, budget_bytes=small)
    try:
        with pytest.raises(MemoryError):
            srv.submit(max(reqs, key=lambda r: r.footprint))
        fits = [r for r in reqs if r.footprint <= small]
        for r in fits:
            srv.submit(r)
        srv.drain()
        assert all(r.distance is not None for r in fits)
    finally:
        srv.close()


def test_persistent_server_results_match():
    from tropidist_gb300 import auto
    from tropidist_gb300.serve import poisson_arrivals, serve_persistent
    ps, reqs = _requests(9, 20)
    alone = [auto.dp_distance(p, list(range(p.ncols)))[0] for p in ps]
    arr = poisson_arrivals(len(reqs), rate=1000.0, seed=2)
    done, wall, peak = serve_persistent(reqs, arr, arena_bytes=1 << 30, jobs=1 << 16, param_bytes=1 << 26, plans=256)
    assert [r.distance for r in done] == alone
    assert peak > 1


def test_persistent_server_reuses_slots_under_a_small_arena():
    """An arena that holds only a few plans at once: plans wait for room, slots and job ranges are
    reused, every result is still exact."""
    from tropidist_gb300 import auto
    from tropidist_gb300.serve import poisson_arrivals, serve_persistent
    ps, reqs = _requests(4, 16)
    alone = [auto.dp_distance(p, list(range(p.ncols)))[0] for p in ps]
    biggest = max(r.footprint for r in reqs)
    done, wall, peak = serve_persistent(reqs, poisson_arrivals(len(reqs), 5000.0, seed=3), arena_bytes=3 * biggest,
                                        jobs=1 << 14, param_bytes=1 << 25, plans=8)
    assert [r.distance for r in done] == alone


def test_persistent_server_mixes_sparse_requests():
    """Circuit-style problems for the sparse DP served beside dense ones: each distance is the one the
    sparse DP gives alone, and the dense results are unchanged by the mix."""
    from tropidist_gb300 import auto, sparse_dp, synth
    from tropidist_gb300.serve import SparseRequest, poisson_arrivals, serve_persistent
    ps, reqs = _requests(5, 8)
    sps = [synth.circuit_dem(seed=30 + j, rounds=4, checks=12, ncols=300 + 100 * j) for j in range(3)]
    alone_sparse = [sparse_dp.distance(p, kmax=30, witness=False)["distance"] for p in sps]
    alone_dense = [auto.dp_distance(p, list(range(p.ncols)))[0] for p in ps]
    mixed = reqs[:3] + [SparseRequest(100, sps[0])] + reqs[3:6] + [SparseRequest(101, sps[1])] + reqs[6:] + \
        [SparseRequest(102, sps[2])]
    arr = poisson_arrivals(len(mixed), rate=500.0, seed=3)
    done, wall, peak = serve_persistent(mixed, arr, budget_frac=0.5, sparse_frac=0.1, sparse_sms=16,
                                        jobs=1 << 16, param_bytes=64 << 20, plans=512)
    got_dense = [r.distance for r in done if getattr(r, "kind", None) != "sparse"]
    got_sparse = [r.distance for r in done if getattr(r, "kind", None) == "sparse"]
    assert got_dense == alone_dense
    assert got_sparse == alone_sparse
    assert all(getattr(r, "error", None) is None for r in done)


def test_persistent_server_wide_lane():
    """Wide dense requests on their own lane (plain streaming launches) beside the persistent kernel
    and the sparse workers: every distance is the one computed alone."""
    from tropidist_gb300 import auto, sparse_dp, synth
    from tropidist_gb300.serve import SparseRequest, poisson_arrivals, serve_persistent
    ps, reqs = _requests(6, 10)
    widths = sorted(max((pl.peak_bits for pl in r.plans if pl.feasible), default=0) for r in reqs)
    cut = widths[len(widths) // 2]                       # about half of them take the wide lane
    sp = synth.circuit_dem(seed=40, rounds=4, checks=12, ncols=400)
    alone_dense = [auto.dp_distance(p, list(range(p.ncols)))[0] for p in ps]
    alone_sparse = sparse_dp.distance(sp, kmax=30, witness=False)["distance"]
    mixed = reqs[:5] + [SparseRequest(100, sp)] + reqs[5:]
    done, wall, peak = serve_persistent(mixed, poisson_arrivals(len(mixed), 300.0, seed=5), budget_frac=0.5,
                                        sparse_frac=0.1, sparse_sms=16, jobs=1 << 16, param_bytes=64 << 20,
                                        plans=512, wide_bits=cut)
    assert [r.distance for r in done if getattr(r, "kind", None) != "sparse"] == alone_dense
    assert [r.distance for r in done if getattr(r, "kind", None) == "sparse"] == [alone_sparse]
