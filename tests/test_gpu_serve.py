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
