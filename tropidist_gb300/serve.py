"""Serving exact distances: a request loop with continuous batching on one GPU.

Server             accepts distance requests (dense Rank DP problems, as their scheduled plans) at
                   any time; a scheduler thread admits a waiting request as soon as a stream slot
                   is free and its tables fit the device-memory budget (80 % of the free HBM by
                   default), launches all of its passes on its own CUDA stream, and retires it when
                   its completion event fires.  Requests admitted while others run overlap on the
                   device (narrow plans' sweeps and small passes share the SMs); finished requests
                   return their slot and memory at once, so the batch is continuous.
PersistentServer   the same interface on one long-lived persistent kernel (csrc/batch.cu k_server):
                   admitted plans are handed to the running kernel through a device mailbox and
                   their passes are interleaved with the plans already in flight at tile-range
                   granularity, with no kernel launches per pass.  Sparse requests (SparseRequest:
                   circuit-style problems for the sparse Rank DP) run beside it on worker threads
                   with their own streams and SMs, each worker admitting one request at a time
                   against its share of the memory budget; with `wide_bits`, dense requests with
                   a table of 2^wide_bits entries or more run on a lane of their own with the
                   plain streaming launches (their passes are bandwidth-bound: batching them gains
                   nothing and the persistent kernel's share of the SMs would slow them down).
serve_plain        the same requests one at a time on one stream (the plain GPU path).
poisson_arrivals   seeded exponential inter-arrival times.
Latency = completion time - arrival time; p50 / p99 and solves/s are computed by `summarize`.
"""
from __future__ import annotations

import collections
import threading
import time

import numpy as np

from . import device, kernel


class Request:
    __slots__ = ("rid", "plans", "cps", "arrival", "admitted", "done", "values", "distance", "footprint",
                 "bufs", "event", "host", "stream")

    def __init__(self, rid, plans, cps=None):
        self.rid = rid
        self.plans = list(plans)
        self.cps = cps
        self.arrival = self.admitted = self.done = None
        self.values = None
        self.distance = None
        peak = max((pl.peak_bits for pl in self.plans if pl.feasible), default=0)
        self.footprint = 2 << peak
        self.bufs = self.event = self.host = self.stream = None


def compile_request(rid, plans):
    """A request whose plans are scheduled ahead of time (scheduling is host work, outside the GPU
    timing of both serving modes)."""
    return Request(rid, plans, [kernel.CompiledPlan(pl) if pl.feasible else None for pl in plans])


class SparseRequest:
    """A distance problem for the sparse Rank DP (iterative deepening over the weight threshold,
    meet in the middle; the problem's tables live on the device while it runs)."""
    kind = "sparse"

    def __init__(self, rid, problem, kmax=30, max_states=1 << 26):
        self.rid = rid
        self.problem = problem
        self.kmax = kmax
        self.max_states = max_states
        self.footprint = 24 * max_states          # packed states + index + changed list, bytes
        self.plan = None                          # future of the host planning (server side)
        self.arrival = self.admitted = self.done = None
        self.distance = None
        self.values = None
        self.error = None


_PLANNERS = None


def _planners(n):
    """A shared pool of planning processes (spawned: safe beside a CUDA context), warmed up."""
    global _PLANNERS
    if _PLANNERS is None and n > 0:
        import concurrent.futures
        import multiprocessing
        _PLANNERS = concurrent.futures.ProcessPoolExecutor(max_workers=n,
                                                           mp_context=multiprocessing.get_context("spawn"))
        list(_PLANNERS.map(_warm, range(n)))
    return _PLANNERS


def _warm(_):
    from . import sparse_dp  # noqa: F401  (imports the package and loads the library once)
    return 0


def _plan_sparse(problem):
    from . import sparse_dp
    return sparse_dp.plan_trellises(problem)


def _run_sparse(req):
    from . import sparse_dp
    try:
        trs = req.plan.result() if getattr(req, "plan", None) is not None else None
        r = sparse_dp.distance(req.problem, kmax=req.kmax, witness=False, trellises=trs)
        req.distance = r["distance"]
    except (sparse_dp.BudgetExceeded, MemoryError, ValueError) as e:
        req.error = "%s: %s" % (type(e).__name__, e)
    req.values = [req.distance]


def _launch(req, stream):
    import torch
    peak = max((pl.peak_bits for pl in req.plans if pl.feasible), default=0)
    n = 1 << peak
    with torch.cuda.stream(stream):
        a = torch.empty(n, dtype=torch.uint8, device="cuda")
        b = torch.empty(n, dtype=torch.uint8, device="cuda")
        res = torch.empty(max(1, len(req.plans)), dtype=torch.uint8, device="cuda")
    req.host = torch.empty(max(1, len(req.plans)), dtype=torch.uint8).pin_memory()
    sp = stream.cuda_stream
    for k, (pl, cp) in enumerate(zip(req.plans, req.cps)):
        if cp is None:
            continue
        cp.execute(a, b, stream=sp)
        src = b if cp.final_buf else a
        with torch.cuda.stream(stream):
            res[k:k + 1].copy_(src[:1])
    with torch.cuda.stream(stream):
        req.host.copy_(res, non_blocking=True)
    ev = torch.cuda.Event()
    ev.record(stream)
    req.bufs = (a, b, res)
    req.event = ev


def _finish(req):
    vals = req.host.tolist()
    req.values = []
    best = None
    for k, pl in enumerate(req.plans):
        if not pl.feasible:
            req.values.append(None)
            continue
        v = kernel.final_value(vals[k])
        req.values.append(v)
        best = v if best is None else min(best, v)
    req.distance = best
    req.bufs = None


class Server:
    """Continuous-batching request loop (see the module docstring)."""

    def __init__(self, slots=16, budget_bytes=None, budget_frac=0.8):
        import torch
        device.require_gpu()
        self.torch = torch
        self.streams = [torch.cuda.Stream() for _ in range(slots)]
        self.free_slots = list(range(slots))
        self.budget = int(budget_frac * device.free_bytes()) if budget_bytes is None else int(budget_bytes)
        self.in_use = 0
        self.pending = collections.deque()
        self.running = {}
        self.finished = []
        self.lock = threading.Lock()
        self.wake = threading.Event()
        self.stop_flag = False
        self.peak_running = 0
        self.submitted = 0
        self.thread = threading.Thread(target=self._loop, daemon=True)
        self.thread.start()

    def submit(self, req, arrival=None):
        if req.footprint > self.budget:
            raise MemoryError("request %s needs %d bytes of tables, beyond the budget" % (req.rid, req.footprint))
        req.arrival = time.perf_counter() if arrival is None else arrival
        with self.lock:
            self.pending.append(req)
            self.submitted += 1
        self.wake.set()
        return req

    def _loop(self):
        while not self.stop_flag:
            progressed = False
            # retire finished requests (their slot and memory return at once)
            for slot, req in list(self.running.items()):
                if req.event.query():
                    req.done = time.perf_counter()
                    _finish(req)
                    del self.running[slot]
                    self.free_slots.append(slot)
                    self.in_use -= req.footprint
                    self.finished.append(req)
                    progressed = True
            # admit waiting requests in arrival order while slots and memory allow
            while self.free_slots:
                with self.lock:
                    if not self.pending or self.in_use + self.pending[0].footprint > self.budget:
                        break
                    req = self.pending.popleft()
                slot = self.free_slots.pop()
                req.admitted = time.perf_counter()
                req.stream = self.streams[slot]
                _launch(req, req.stream)
                self.running[slot] = req
                self.in_use += req.footprint
                self.peak_running = max(self.peak_running, len(self.running))
                progressed = True
            if not progressed:
                if self.running:
                    time.sleep(20e-6)
                else:
                    self.wake.wait(0.001)
                    self.wake.clear()

    def drain(self, timeout=600.0):
        """Wait until every submitted request has finished."""
        t0 = time.perf_counter()
        while True:
            with self.lock:
                todo = self.submitted
            if len(self.finished) >= todo:
                return
            if time.perf_counter() - t0 > timeout:
                raise TimeoutError("requests still running after %.0f s" % timeout)
            time.sleep(0.0005)

    def close(self):
        self.stop_flag = True
        self.wake.set()
        self.thread.join(timeout=10)


def poisson_arrivals(n, rate, seed=0):
    """n arrival offsets (seconds) of a Poisson process of the given rate."""
    rng = np.random.default_rng(seed)
    return np.cumsum(rng.exponential(1.0 / rate, size=n))


def serve_continuous(reqs, arrivals, slots=16, budget_bytes=None):
    """Submit the requests at their arrival offsets to a Server; returns (requests, wall seconds, peak in flight)."""
    srv = Server(slots=slots, budget_bytes=budget_bytes)
    t0 = time.perf_counter()
    for req, at in zip(reqs, arrivals):
        now = time.perf_counter() - t0
        if at > now:
            time.sleep(at - now)
        srv.submit(req, arrival=t0 + at)
    srv.drain()
    wall = time.perf_counter() - t0
    peak = srv.peak_running
    srv.close()
    return reqs, wall, peak


def serve_plain(reqs, arrivals):
    """The plain path: one request at a time, in arrival order, each waited for before the next."""
    import torch
    stream = torch.cuda.Stream()
    t0 = time.perf_counter()
    for req, at in zip(reqs, arrivals):
        now = time.perf_counter() - t0
        if at > now:
            time.sleep(at - now)
        req.arrival = t0 + at
        req.admitted = time.perf_counter()
        if getattr(req, "kind", None) == "sparse":
            with torch.cuda.stream(stream):
                _run_sparse(req)
            stream.synchronize()
            req.done = time.perf_counter()
            continue
        _launch(req, stream)
        req.event.synchronize()
        req.done = time.perf_counter()
        _finish(req)
    return reqs, time.perf_counter() - t0


def summarize(reqs, wall):
    lat = np.array([r.done - r.arrival for r in reqs])
    return {"requests": len(reqs), "seconds": wall, "solves_per_s": len(reqs) / wall,
            "p50_ms": float(np.percentile(lat, 50) * 1e3), "p99_ms": float(np.percentile(lat, 99) * 1e3),
            "mean_ms": float(lat.mean() * 1e3)}


class PersistentServer:
    """Continuous batching inside one persistent kernel.  A request's plans are submitted as soon as
    the arena (device tables) and the descriptor pools have room; finished plans are collected by
    polling, and a request completes when all of its plans have."""

    def __init__(self, arena_bytes=None, budget_frac=0.8, jobs=1 << 20, param_bytes=1 << 30, plans=8192,
                 sparse_frac=0.0, sparse_sms=0, sparse_workers=2, sparse_planners=4, wide_bits=None,
                 wide_workers=1):
        import ctypes
        import torch
        from . import _lib
        device.require_gpu()
        self.torch, self.ctypes, self.L = torch, ctypes, _lib.lib()
        free = device.free_bytes()
        if arena_bytes is None:
            arena_bytes = int((budget_frac - sparse_frac) * free) - param_bytes - 64 * jobs
        self.arena = device.empty(arena_bytes)
        st = ctypes.c_int(0)
        # sparse requests run beside the persistent kernel: it leaves `sparse_sms` SMs to them
        blocks = max(1, _lib.lib().tg_sm_count() - int(sparse_sms)) if sparse_sms else 0
        self.handle = self.L.tg_server_create(self.arena.data_ptr(), arena_bytes, jobs, param_bytes, plans, blocks,
                                              ctypes.byref(st))
        if not self.handle:
            _lib.check(st.value)
        self.plan_cap = plans
        self.pending = collections.deque()
        self.owner = {}                # slot -> (request, plan index)
        self.left = {}                 # request id -> plans still running
        self.finished = []
        self.submitted = 0
        self.peak_running = 0
        self.lock = threading.Lock()
        self.stop_flag = False
        self.slots = np.zeros(plans, dtype=np.int32)
        self.vals = np.zeros(plans, dtype=np.uint32)
        self.thread = threading.Thread(target=self._loop, daemon=True)
        self.thread.start()
        # sparse requests: a worker on its own stream, admitted one at a time against the sparse share
        # of the memory budget
        self.sparse_budget = int(sparse_frac * free) // max(1, sparse_workers)
        # the sparse requests' host planning runs in worker processes as they arrive
        self.planner = _planners(sparse_planners) if sparse_frac > 0 else None
        self.sparse_q = collections.deque()
        self.sparse_wake = threading.Event()
        self.sparse_threads = [threading.Thread(target=self._sparse_loop, daemon=True) for _ in range(sparse_workers)]
        for t in self.sparse_threads:
            t.start()
        # wide dense requests (a table of 2^wide_bits entries or more: bandwidth-bound passes) run on
        # a lane of their own with the plain streaming launches, one request at a time, beside the
        # persistent kernel; their tables come from the same memory budget, checked at submit
        self.wide_bits = wide_bits
        self.wide_q = collections.deque()
        self.wide_wake = threading.Event()
        self.wide_threads = []
        if wide_bits is not None:
            self.wide_threads = [threading.Thread(target=self._wide_loop, daemon=True) for _ in range(wide_workers)]
            for t in self.wide_threads:
                t.start()

    def submit(self, req, arrival=None):
        req.arrival = time.perf_counter() if arrival is None else arrival
        with self.lock:
            self.submitted += 1
            if getattr(req, "kind", None) == "sparse":
                if req.footprint > self.sparse_budget:
                    self.submitted -= 1
                    raise MemoryError("sparse request %s needs %d bytes, beyond the sparse budget" %
                                      (req.rid, req.footprint))
                if self.planner is not None:
                    req.plan = self.planner.submit(_plan_sparse, req.problem)
                self.sparse_q.append(req)
                self.sparse_wake.set()
            elif self.wide_bits is not None and req.cps is not None and \
                    max((pl.peak_bits for pl in req.plans if pl.feasible), default=0) >= self.wide_bits:
                self.wide_q.append(req)
                self.wide_wake.set()
            else:
                self.pending.append(req)
        return req

    def _wide_loop(self):
        stream = self.torch.cuda.Stream()
        while not self.stop_flag:
            with self.lock:
                req = self.wide_q.popleft() if self.wide_q else None
            if req is None:
                self.wide_wake.wait(0.001)
                self.wide_wake.clear()
                continue
            req.admitted = time.perf_counter()
            _launch(req, stream)
            req.event.synchronize()
            req.done = time.perf_counter()
            _finish(req)
            self.finished.append(req)

    def _sparse_loop(self):
        stream = self.torch.cuda.Stream()
        while not self.stop_flag:
            with self.lock:
                req = self.sparse_q.popleft() if self.sparse_q else None
            if req is None:
                self.sparse_wake.wait(0.001)
                self.sparse_wake.clear()
                continue
            req.admitted = time.perf_counter()
            with self.torch.cuda.stream(stream):
                _run_sparse(req)
            stream.synchronize()
            req.done = time.perf_counter()
            self.finished.append(req)

    def _admit(self, req):
        """Submit every feasible plan of the request; False (nothing submitted) if there is no room."""
        from . import _lib
        slots = []
        for k, pl in enumerate(req.plans):
            if not pl.feasible:
                continue
            cp = req.cps[k] if req.cps is not None else None
            if cp is not None:
                r = self.L.tg_server_submit_plan(self.handle, cp.handle)
            else:
                enc = np.ascontiguousarray(pl.encode())
                r = self.L.tg_server_submit(self.handle, enc.ctypes.data, len(enc))
            if r == -3 and not slots and not self.owner:
                _lib.check(r)               # does not fit even in an empty server
            if r == -3:
                return slots, False
            if r < 0:
                _lib.check(r)
            slots.append((r, k))
        return slots, True

    def _loop(self):
        partial = None
        idle = 50e-6
        while not self.stop_flag:
            progressed = False
            n = self.L.tg_server_poll(self.handle, self.slots.ctypes.data, self.vals.ctypes.data, self.plan_cap)
            if n < 0:
                from . import _lib
                _lib.check(n)
            for i in range(n):
                req, k = self.owner.pop(int(self.slots[i]))
                req.values[k] = kernel.final_value(int(self.vals[i]))
                self.left[req.rid] -= 1
                if self.left[req.rid] == 0:
                    req.done = time.perf_counter()
                    feas = [v for v in req.values if v is not None]
                    req.distance = min(feas) if feas else None
                    self.finished.append(req)
                progressed = True
            # admit waiting requests (a request whose plans did not all fit keeps its place)
            while True:
                if partial is None:
                    with self.lock:
                        if not self.pending:
                            break
                        req = self.pending.popleft()
                    req.admitted = time.perf_counter()
                    req.values = [None] * len(req.plans)
                    feasible = [k for k, pl in enumerate(req.plans) if pl.feasible]
                    self.left[req.rid] = len(feasible)
                    partial = (req, feasible)
                    if not feasible:
                        req.done = time.perf_counter()
                        self.finished.append(req)
                        partial = None
                        continue
                req, todo = partial
                sub = _Sub(req, todo)
                got, ok = self._admit(sub)
                for slot, kk in got:
                    self.owner[slot] = (req, todo[kk])
                partial = None if ok else (req, todo[len(got):])
                progressed = progressed or bool(got)
                self.peak_running = max(self.peak_running, len(self.owner))
                if not ok:
                    break
            # back off while nothing moves (the polling thread shares the interpreter with the
            # sparse workers' host work), poll fast while results come in
            if not progressed:
                time.sleep(idle)
                idle = min(2 * idle, 1e-3)
            else:
                idle = 50e-6

    def drain(self, timeout=600.0):
        t0 = time.perf_counter()
        while len(self.finished) < self.submitted:
            if time.perf_counter() - t0 > timeout:
                raise TimeoutError("requests still running after %.0f s" % timeout)
            time.sleep(0.0005)

    def close(self):
        self.stop_flag = True
        self.thread.join(timeout=10)
        self.sparse_wake.set()
        for t in self.sparse_threads:
            t.join(timeout=60)
        self.wide_wake.set()
        for t in self.wide_threads:
            t.join(timeout=60)
        if self.handle:
            self.L.tg_server_free(self.handle)
            self.handle = None


class _Sub:
    """The not yet submitted plans of a request."""

    def __init__(self, req, todo):
        self.plans = [req.plans[k] for k in todo]
        self.cps = [req.cps[k] for k in todo] if req.cps is not None else None


def serve_persistent(reqs, arrivals, **kw):
    """Submit the requests at their arrival offsets to a PersistentServer; (requests, seconds, peak plans)."""
    srv = PersistentServer(**kw)
    t0 = time.perf_counter()
    for req, at in zip(reqs, arrivals):
        now = time.perf_counter() - t0
        if at > now:
            time.sleep(at - now)
        srv.submit(req, arrival=t0 + at)
    srv.drain()
    wall = time.perf_counter() - t0
    peak = srv.peak_running
    srv.close()
    return reqs, wall, peak
