#!/usr/bin/env python
"""Benchmark of the dense Rank DP: trellis state-updates per second on one GB300.

Workload: the seeded banded problem m=1000 x n=2000 (column weight 3), window 37, whose natural
column order has a 31-bit frontier (a 2^31-entry, 2 GB uint8 table), with its four logical rows
taken one at a time.  One step = the four exact dense sweeps of dp_distance (all plan ops, from
the empty table to the final entry).  The tables (2 GB) are far larger than L2, so no flush is
needed between steps.

`value` is state-updates/s (Plan.work(), cdist/trellis.py:133-144) with the op stream already
scheduled and the tables resident in HBM; `e2e` is the same metric through the public API
(tropidist_gb300.auto.dp_distance: host planning, scheduling, launches and the result read back).
`roofline` reports the dominant kernel: table bytes read + written per launch over its average
launch time in the CUDA-event-timed region (the region's time times the kernel's share of the GPU
time, the share taken from an instrumented repeat with an event pair around every launch), against
the measured HBM copy bandwidth.  The four distances are compared
with the ones the reference itself computed on this workload (tests/golden/headline.json); a
mismatch fails the run.  `cpu_baseline` times the C/OpenMP port of the reference's kernels
(oracle/dense_port.c) on observable 0's whole sweep with every host core, and on a window of it
with one core.

--impl reference runs that CPU implementation alone (every host core) on the same four plans,
planned by the oracle's restatement of the reference's planner, each timed step one observable's
whole sweep; it loads no library of the package.
Multi-GPU (torchrun): replicas only; rank r sweeps its own instance (seed + r), no collective on
the data path; the time is the maximum over ranks.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "trellis state-updates/s"
UNIT = "state-updates/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--window", type=int, default=37)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--sparse-query", type=int, default=0,
                    help="only run the circuit-style sparse query at this threshold (profiling aid)")
    ap.add_argument("--tree-only", action="store_true",
                    help="run only the tree DP section (for profiling) and print its JSON")
    ap.add_argument("--wide-bits", type=int, default=24,
                    help="served: dense requests with tables of 2^wide_bits entries or more take the wide lane (0: none)")
    ap.add_argument("--sections", default="search,tree,witness,sparse,sparse_full,batched,served",
                    help="secondary workloads reported beside the headline (comma list, empty for none)")
    return ap.parse_args()


def problem(args, rank=0):
    """The seeded banded problem of the headline (pure Python: no library is loaded)."""
    from tropidist_gb300 import synth
    p = synth.dense_scale(args.seed + rank, window=args.window)
    return p, list(range(p.ncols))


def workload(args, rank=0):
    """The problem and its four plans from the package's planner (the GPU arm)."""
    from tropidist_gb300 import trellis
    p, order = problem(args, rank)
    plans = [trellis.build_plan(p.h, p.l, 1 << o, order, p.nrows) for o in range(p.nobs)]
    return p, order, plans


def oracle_plans(p, order):
    """The same plans from the oracle's restatement of the reference's planner (the CPU arm)."""
    from oracle import plan as oplan
    return [oplan.plan(p.h, p.l, 1 << o, order, p.nrows) for o in range(p.nobs)]


def dist_string(dists):
    return ",".join("none" if d is None else "overflow" if d == "overflow" else str(int(d)) for d in dists)


def config(args, plans, dists):
    """The workload, identical in both arms (both sweep the same plans to the same distances)."""
    feas = [pl for pl in plans if pl.feasible]
    peak = max(pl.peak_bits for pl in feas)
    return {"workload": "dense Rank DP, banded m=1000 n=2000 col-weight 3 window %d seed %d, natural order, "
                        "4 logical rows one at a time" % (args.window, args.seed),
            "m": 1000, "n": 2000, "window": args.window, "seed": args.seed, "observables": len(plans),
            "peak_bits": peak, "table_bytes": 1 << peak, "work_per_step": int(sum(pl.work() for pl in feas)),
            "entry": "uint8", "l2": "inputs larger than L2 (2 GB tables), no flush",
            "distances": dist_string(dists)}


def golden_headline(args):
    """Per observable the distance the reference itself computed on this workload (its planner and
    C kernels, tests/golden/headline.json), or None for another seed / window."""
    if args.seed != 0 or args.window != 37:
        return None
    try:
        with open(os.path.join(ROOT, "tests", "golden", "headline.json")) as f:
            return [c["value"] for c in json.load(f)["cases"]]
    except (OSError, ValueError, KeyError):
        return None


# ---------------------------------------------------------------------- CPU implementation (port)
def port_lib():
    import ctypes as C
    so = os.path.join(ROOT, "oracle", "dense_port.so")
    if not os.path.exists(so):
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    L = C.CDLL(so)
    L.port_run_plan.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_uint64]
    L.port_run_plan.restype = C.c_uint64
    L.port_num_threads.restype = C.c_int
    L.port_set_threads.argtypes = [C.c_int]
    return L


def _full_width_start(plan):
    """The first op after which the table is 2^(peak_bits - 1) entries wide."""
    w = 0
    for i, op in enumerate(plan.ops):
        w += 1 if op[0] == "expand" else -1 if op[0] == "select" else 0
        if w >= plan.peak_bits - 1:
            return i + 1
    return len(plan.ops)


def port_sweep(L, plan, buf):
    """One whole sweep of the plan by the C port: (distance or None / "overflow", seconds)."""
    enc = plan.encoded()
    buf[0] = 0
    t0 = time.perf_counter()
    n = L.port_run_plan(enc.ctypes.data, len(enc), buf.ctypes.data, 1)
    dt = time.perf_counter() - t0
    assert n == 1
    v = int(buf[0])
    return ("overflow" if v == 255 else v), dt


def port_window(L, plan, buf, seconds):
    """The C port on the ops after the table first reaches full width, for about `seconds`:
    (state-updates/s, state-updates, seconds, first op, last op)."""
    enc = plan.encoded()
    start = _full_width_start(plan)
    buf[0] = 0
    n = L.port_run_plan(enc.ctypes.data, start, buf.ctypes.data, 1)
    bits = int(n).bit_length() - 1
    i, work, t0 = start, 0, time.perf_counter()
    while i < len(enc) and time.perf_counter() - t0 < seconds:
        j = min(len(enc), i + 4)
        for op in plan.ops[i:j]:
            if op[0] == "expand":
                bits += 1
            elif op[0] == "select":
                bits -= 1
            else:
                work += 1 << bits
        n = L.port_run_plan(enc[i:j].ctypes.data, j - i, buf.ctypes.data, n)
        i = j
    secs = time.perf_counter() - t0
    return work / secs, work, secs, start, i


def cpu_legs(p, order, seconds_one=8.0):
    """The GPU arm's CPU baseline: observable 0's whole sweep by the C port on every host core, and
    a window of the same plan at full width on one core."""
    import numpy as np
    plans = oracle_plans(p, order)
    plan = plans[0]
    L = port_lib()
    buf = np.zeros(1 << plan.peak_bits, dtype=np.uint8)
    buf.fill(0)
    L.port_set_threads(os.cpu_count() or 1)
    cores = L.port_num_threads()
    v, dt = port_sweep(L, plan, buf)
    out = {"value": plan.work() / dt, "unit": UNIT, "cores": cores, "kind": "port",
           "sample": "observable 0's whole sweep (%.3g state-updates, 2^%d-entry peak), oracle planner + C/OpenMP "
                     "port of cdist/viterbi.c" % (plan.work(), plan.peak_bits), "seconds": dt, "distance": v}
    L.port_set_threads(1)
    rate, work, secs, a, b = port_window(L, plan, buf, seconds_one)
    out["one_thread"] = {"value": rate, "cores": 1, "seconds": secs,
                         "sample": "ops %d..%d of observable 0's plan at full width (%.3g state-updates)" % (a, b, work)}
    L.port_set_threads(os.cpu_count() or 1)
    return out


def run_reference(args):
    """The CPU arm: the reference's dense algorithm (the C/OpenMP port of cdist/viterbi.c driven in
    the executor order of cdist/kernel.py:94-138) on every host core, on the plans of the oracle's
    restatement of cdist/trellis.py.  No library of the package is loaded.  Each timed step is one
    observable's whole sweep (observables in turn, so the distances of all four are computed); the
    warm-up steps run the first plan up to full width (thread pool and page faults)."""
    import numpy as np
    p, order = problem(args)
    plans = oracle_plans(p, order)
    feas = [(o, pl) for o, pl in enumerate(plans) if pl.feasible]
    L = port_lib()
    L.port_set_threads(os.cpu_count() or 1)
    cores = L.port_num_threads()
    peak = max(pl.peak_bits for _, pl in feas)
    buf = np.zeros(1 << peak, dtype=np.uint8)
    buf.fill(0)                                # the pages are touched before any timing
    for _ in range(args.warmup):
        enc = feas[0][1].encoded()
        buf[0] = 0
        L.port_run_plan(enc.ctypes.data, _full_width_start(feas[0][1]), buf.ctypes.data, 1)
    dists = [None] * len(plans)
    work = secs = 0.0
    for k in range(args.steps):
        o, pl = feas[k % len(feas)]
        dists[o], dt = port_sweep(L, pl, buf)
        work += pl.work()
        secs += dt
    for o, pl in feas[args.steps:]:            # fewer steps than observables: the rest untimed
        dists[o], _ = port_sweep(L, pl, buf)
    value = work / secs
    gold = golden_headline(args)
    sample = "each step one observable's whole sweep (observables in turn), all host cores"
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * secs / max(1, args.steps), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic (seeded banded problem)",
            "impl": "reference", "config": config(args, plans, dists),
            "step": "one observable's whole sweep (the GPU arm's step sweeps all four)",
            "parity": {"reference_fixture": dist_string(gold) if gold else None,
                       "equal": (dists == gold) if gold else None},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------- clocks
class Clocks:
    FIELDS = "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active," \
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown," \
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, gpu_index):
        self.rows, self.proc = [], None
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(gpu_index)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except (OSError, ValueError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if not self.rows:
            return None
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4) if r[5 + k].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def measured_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def traffic_per_launch(kernel):
    """DRAM bytes / algorithmic bytes of `kernel` from the committed ncu summaries
    (profiles/<kernel>_traffic.json, or the older fused_pass_traffic.json), or None."""
    for name in ("%s_traffic.json" % kernel, "fused_pass_traffic.json"):
        try:
            with open(os.path.join(ROOT, "profiles", name)) as f:
                tr = json.load(f)
        except (OSError, ValueError):
            continue
        if tr.get("kernel") == kernel:
            return tr
    return None


# ---------------------------------------------------------------------- secondary workloads
def _time_gpu(fn, reps=1):
    import torch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        out = fn()
    torch.cuda.synchronize()
    return (time.perf_counter() - t0) / reps, out


def section_batched(args):
    """256 uneven banded instances (widths 12-26, 1-12 logical rows) in one persistent launch
    against the same plans run one instance at a time with the plain path; the autotuned schedule
    knobs per width."""
    from tropidist_gb300 import auto, autotune, kernel, synth
    from tropidist_gb300.batch import DenseBatch
    ps = synth.batch_instances(seed=0, count=256, wmin=12, wmax=26, max_obs=12)
    owner, plans = [], []
    for k, p in enumerate(ps):
        for _, pl in auto._plans(p, list(range(p.ncols))):
            owner.append(k)
            plans.append(pl)
    tuner = autotune.Tuner().tune([16, 20, 24, 26], reps=2)
    batch = DenseBatch(plans)
    batch.run()
    tb, vals = _time_gpu(batch.run)
    cps = [autotune.compiled(pl, tuner) if pl.feasible else None for pl in plans]
    peak = max(cp.peak_bits for cp in cps if cp is not None)
    import torch
    a = torch.empty(1 << peak, dtype=torch.uint8, device="cuda")
    b = torch.empty_like(a)

    def plain():
        out = []
        for k in range(len(ps)):                     # one instance at a time, its result read back
            best = None
            for i, cp in enumerate(cps):
                if owner[i] != k or cp is None:
                    continue
                cp.execute(a, b)
                v = cp.result(a, b)
                best = v if best is None else min(best, v)
            out.append(best)
        return out
    plain()
    ts, seq = _time_gpu(plain)
    per = [None] * len(ps)
    for i, v in enumerate(vals):
        if v is not None:
            per[owner[i]] = v if per[owner[i]] is None else min(per[owner[i]], v)
    for cp in cps:
        if cp is not None:
            cp.free()
    knobs = {w: "%d/%d/%d" % (r["dmax"], r["span"], r["span_sel"]) for w, r in tuner.report().items()}
    return {"plans": len(plans), "solves_s": round(len(ps) / tb, 1), "plain_solves_s": round(len(ps) / ts, 1),
            "speedup": round(ts / tb, 3), "equal": per == seq, "knobs_dmax_span_sel": knobs}


def _serve_requests(seed=11):
    from tropidist_gb300 import auto, serve, synth
    ps = synth.batch_instances(seed=seed, count=96, wmin=10, wmax=28, max_obs=12)
    dense = [serve.compile_request(k, [pl for _, pl in auto._plans(p, list(range(p.ncols)))])
             for k, p in enumerate(ps)]
    sparse = []
    for j, n in enumerate([2000, 5000, 10000, 20000]):
        p = synth.circuit_dem(seed=100 + j, rounds=max(4, n // 500), checks=24, ncols=n)
        sparse.append(serve.SparseRequest(1000 + j, p, kmax=30))
    # interleave: a sparse problem after every 24 dense ones
    out, si = [], 0
    for k, r in enumerate(dense):
        out.append(r)
        if k % 24 == 23 and si < len(sparse):
            out.append(sparse[si])
            si += 1
    return out + sparse[si:]


def section_served(args):
    """Poisson request streams (rates 10 to 2000 req/s) of 96 banded instances (widths 10-28, 1-12
    logical rows, seed 11) and 4 circuit-style sparse problems (n = 2000-20000, 24 checks per
    round), served by the persistent-kernel request loop with continuous batching (dense tables in
    an arena of 60 % of the free HBM, sparse against 20 %; requests with tables of 2^24 entries or
    more on two wide lanes), against the plain path (one request at a time); per rate p50 / p99
    latency in ms and solves/s of both, and whether every distance is the same."""
    from tropidist_gb300 import serve
    res = {}
    for rate in (10, 50, 200, 1000, 2000):
        arr = serve.poisson_arrivals(100, rate, seed=rate)
        r1, w1, peak = serve.serve_persistent(_serve_requests(), arr, budget_frac=0.8, sparse_frac=0.2,
                                              sparse_sms=24, jobs=1 << 21, param_bytes=2 << 30, plans=4096,
                                              wide_bits=args.wide_bits if args.wide_bits > 0 else None,
                                              wide_workers=2)
        r2, w2 = serve.serve_plain(_serve_requests(), arr)
        s1, s2 = serve.summarize(r1, w1), serve.summarize(r2, w2)
        res[str(rate)] = {"p50": round(s1["p50_ms"], 1), "p99": round(s1["p99_ms"], 1),
                          "solves_s": round(s1["solves_per_s"], 1), "plain_p50": round(s2["p50_ms"], 1),
                          "plain_p99": round(s2["p99_ms"], 1), "plain_solves_s": round(s2["solves_per_s"], 1),
                          "ratio": round(s1["solves_per_s"] / s2["solves_per_s"], 3),
                          "equal": [a.distance for a in r1] == [b.distance for b in r2]}
    return res


def _sparse_run(tr, K, backend="gpu", witness=False, limit_s=None):
    """One meet-in-the-middle query timed around the whole call: value, seconds, state-steps (the
    states of every table stepped, both sweeps), peak states.  limit_s: the query's deadline
    (sparse_dp.BudgetExceeded past it)."""
    import torch
    from tropidist_gb300 import sparse_dp
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    deadline = time.monotonic() + limit_s if limit_s else None
    r = sparse_dp.query(tr, K, mode="mitm", backend=backend, witness=witness, deadline=deadline)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    sm = sparse_dp.summary(r)
    steps = sum(v for k, v in sm.items() if k.endswith("_states_total"))
    return {"value": r["value"], "s": round(dt, 3), "state_steps": int(steps),
            "steps_per_s": round(steps / dt), "peak": sm.get("peak_states")}


def section_sparse(args):
    """The circuit-style detector error model scaled to 24 checks per round (40 rounds, n=20000,
    weights {1,2,3}, seed 0; 37 row slots: one-word states, the reference's C tables can hold it)
    through the meet in the middle at K = 4, 8 and 10 on the device tables; the C port of the
    reference's sparse kernels (oracle/sparse_port.c, one core, as the reference's
    sparse_dp.c) behind the same host driver at K = 4 and 8 (at K = 10 it would take minutes)."""
    from tropidist_gb300 import sparse_dp, synth
    from oracle.sparse import CPortTables
    p = synth.circuit_dem(seed=0, rounds=40, checks=24, ncols=20000)
    order = sparse_dp.default_order(p)
    tr = sparse_dp.Trellis.for_query(p, 0, order)
    import torch
    _sparse_run(tr, 2)                                  # warm-up (library, allocator)
    out = {"slots": tr.nslots}
    for K in (4, 8, 10):
        try:
            out["K%d" % K] = _sparse_run(tr, K, limit_s=120)
        except (MemoryError, RuntimeError) as e:        # torch's OutOfMemoryError, BudgetExceeded
            out["K%d" % K] = {"error": type(e).__name__}
        torch.cuda.empty_cache()
    if not args.no_cpu_baseline:
        for K in (4, 8):
            c = _sparse_run(tr, K, backend=CPortTables(tr))
            c["equal"] = c["value"] == out["K%d" % K]["value"]
            out["cpu_K%d" % K] = c
    return out


def section_sparse_full(args):
    """The circuit-style detector error model as written: 40 rounds x 150 checks (m = 6000), n =
    20000, weights {1,2,3}, seed 0, the package's column order: 153 row slots, so three-word
    states on the device (the reference refuses more than 56).  Meet in the middle at K = 4, 8,
    then 10, 12 and 14 while a query stays within 90 s (each query stops at 150 s); the multi-word
    numpy restatement of the reference's table rules (oracle/sparse_wide.py) at K = 4 and 5 on one
    core."""
    from tropidist_gb300 import sparse_dp, synth
    from oracle.sparse_wide import WideTables
    p = synth.circuit_dem(seed=0, rounds=40, checks=150, ncols=20000)
    tr = sparse_dp.Trellis.for_query(p, 0, sparse_dp.default_order(p))
    _sparse_run(tr, 2)
    out = {"slots": tr.nslots, "words": tr.words}
    import torch
    for K in (4, 8, 10, 12, 14):
        torch.cuda.empty_cache()
        try:
            r = _sparse_run(tr, K, limit_s=150)
        except (MemoryError, RuntimeError) as e:        # torch's OutOfMemoryError, BudgetExceeded
            out["K%d" % K] = {"error": type(e).__name__}
            break
        out["K%d" % K] = r
        if r["s"] > 90:
            break
    torch.cuda.empty_cache()
    if not args.no_cpu_baseline:
        for K in (4, 5):
            c = _sparse_run(tr, K, backend=WideTables(tr))
            c["equal"] = c["value"] == out.get("K%d" % K, {}).get("value", c["value"])
            out["cpu_K%d" % K] = c
    return out


def sparse_query(K):
    """One meet-in-the-middle query of the scaled circuit-style problem at threshold K."""
    import torch
    from tropidist_gb300 import sparse_dp, synth
    p = synth.circuit_dem(seed=0, rounds=40, checks=24, ncols=20000)
    tr = sparse_dp.Trellis.for_query(p, 0, sparse_dp.default_order(p))
    t0 = time.perf_counter()
    r = sparse_dp.query(tr, K, mode="mitm", witness=False)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    sm = sparse_dp.summary(r)
    steps = sum(v for k, v in sm.items() if k.endswith("_states_total"))
    return {"sparse_query": K, "value": r["value"], "seconds": dt, "state_steps_per_s": steps / dt,
            "peak_states": sm.get("peak_states")}


def _tree_workload():
    """The banded m=120 n=240 window-16 problem (seed 1), first logical row appended as the target
    row, on the balanced binary tree over the natural column order."""
    from tropidist_gb300 import synth, tree_dp as td

    def balanced(xs):
        if len(xs) == 1:
            return xs[0]
        m = len(xs) // 2
        return balanced(xs[:m]), balanced(xs[m:])
    p = synth.banded(120, 240, 16, 3, 1, seed=1)
    cols, nrows = td._augmented(p.h, p.l, 1)
    return td.CompiledTreeDP(cols, balanced(list(range(p.ncols)))), 1 << nrows


def section_tree(args):
    """Exact min-plus tree DP (cdist/tree_dp.py) of one logical query: every join's compatible
    pairs on the device (height-batched launches, uint32 tables in one arena), against the
    reference's single-threaded executor loop over a C port of its join on the host."""
    import torch
    from tropidist_gb300 import device
    prog, target = _tree_workload()
    lim = dict(max_join_work=None, max_memory_bytes=None, max_seconds=None)
    pf = prog.preflight(max_join_work=None, max_memory_bytes=None)
    arena = device.empty(pf["device_arena_bytes"])
    for _ in range(3):
        v, _st = prog.run(target, arena=arena, **lim)
    reps = 5
    st = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(st)
    for _ in range(reps):
        v, _st = prog.run(target, arena=arena, **lim)
    e1.record(st)
    torch.cuda.synchronize()
    sec = e0.elapsed_time(e1) / 1e3 / reps
    work = pf["join_work"]
    out = {"distance": v, "pairs": work, "ms": round(sec * 1e3, 3), "pairs_s": round(work / sec)}
    if not args.no_cpu_baseline:
        from oracle import tree as ot
        t0 = time.perf_counter()
        vc = ot.run_port(prog, target)
        cpu = time.perf_counter() - t0
        out["cpu_pairs_s"] = round(work / cpu)      # the reference's executor loop over the C port, one core
        out["equal"] = vc == v
    prog.free()
    return out


def section_witness(args):
    """Witness traceback (cdist/auto.py:126-182): the columns of a minimum logical from device table
    checkpoints and a bisection recomputation, on the banded m=1000 n=2000 window 30 problem (four
    logical rows, natural order: 26-bit frontier), checked against H and L on the host.  The
    reference keeps the table before every update (about 2000 tables of 64 MB here, beyond memory);
    its traceback (restated in numpy, oracle/dense.py witness) is timed on the m=120 n=240 problem."""
    import torch
    from tropidist_gb300 import auto, synth, trellis
    from tropidist_gb300.problem import verify_witness
    p = synth.dense_scale(0, window=30)
    order = list(range(p.ncols))
    best, _ = auto.dp_distance(p, order)
    auto.dp_witness(synth.dense_small(2), list(range(240)))       # warm-up (library, allocator)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    r = auto.dp_witness(p, order)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    cols = r["witness"]
    out = {"s": round(dt, 3), "distance": r["distance"],
           "verified": bool(verify_witness(p, cols, r["observable"]) and len(cols) == r["distance"] == best),
           "peak_bits": max(pl.peak_bits for _, pl in auto._plans(p, order) if pl.feasible)}
    if not args.no_cpu_baseline:
        from oracle import dense as od
        q = synth.dense_small(1)
        qo = list(range(q.ncols))
        span = lambda h, o, m: trellis.minimal_span_form(trellis.rows_from_columns(h, o, m))
        t0 = time.perf_counter()
        w = od.witness(q.h, q.l, qo, q.nrows, 0, span, trellis.reduce_target_row, trellis.lowbit)
        cpu = time.perf_counter() - t0
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        g = auto.dp_witness(q, qo, obs=0)
        torch.cuda.synchronize()
        out["small_s"] = round(time.perf_counter() - t0, 4)
        out["small_cpu_s"] = round(cpu, 4)            # the reference's store-every-table traceback, numpy
        out["small_equal"] = len(w) == len(g["witness"])
    return out


def section_search(args):
    """The weight-bounded search (cdist/search.py distance) with completion tables of depth k = 2 and
    3 built and probed on the device (each wave of probes answered natively), on the stim-free
    known-answer codes bb72 (Z, 12 observables, distance 6) and the rotated surface codes d = 9 and
    15 (Z); beside each, the same search with its probes answered by a C port of the reference's
    completion table on one host core (table build included in both)."""
    import torch
    from tropidist_gb300 import search
    from tropidist_gb300.problem import Problem
    codes = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "tests", "golden", "codes.json")))
    out = {}
    for name in ("bb72_Z", "surface_d9_Z", "surface_d15_Z"):
        c = next(x for x in codes if x["name"] == name)
        h = [int(x, 16) if isinstance(x, str) else int(x) for x in c["h"]]
        l = [int(x, 16) if isinstance(x, str) else int(x) for x in c["l"]]
        p = Problem(name, c["nrows"], c["nobs"], h, l, [(i, 0) for i in range(c["nrows"])])
        search.distance(p, k_table=2, kmax=2)                     # warm-up (library, table kernels)
        for k in (2, 3):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            r = search.distance(p, k_table=k, kmax=c["distance"])
            dt = time.perf_counter() - t0
            rec = {"d": r["distance"], "known": c["distance"], "s": round(dt, 4),
                   "nodes": sum(sum(x["nodes"]) for x in r["runs"]), "entries": r["table_entries"]}
            if not args.no_cpu_baseline:
                rec["cpu_s"] = round(_search_cpu(p, c["distance"], k)["seconds"], 4)
            out["%s_k%d" % (name, k)] = rec
    return out


def _search_cpu(p, kmax, k=2):
    """The same search with its probes answered by oracle/table_port.c (the reference's completion
    table in C) on one host core: table build and search time."""
    import ctypes
    import math
    from tropidist_gb300 import search
    from tropidist_gb300._sigs_extra import PROBE_FN
    lib = ctypes.CDLL(os.path.join(os.path.dirname(os.path.abspath(__file__)), "oracle", "table_port.so"))
    lib.tp_create.restype = ctypes.c_void_p
    lib.tp_create.argtypes = [ctypes.c_int]
    lib.tp_build.argtypes = [ctypes.c_void_p, ctypes.c_int] + [ctypes.c_void_p] * 3 + [ctypes.c_int]
    lib.tp_free.argtypes = [ctypes.c_void_p]
    t0 = time.perf_counter()
    zh, zl = search.column_hashes(p.h, search.row_hashes(p.nrows, 12345))
    import numpy as np
    lg = np.array(p.l, dtype=np.uint64)
    total = sum(math.comb(p.ncols, i) for i in range(k + 1))
    tab = lib.tp_create(max(10, math.ceil(math.log2(total / 0.5 + 1))))
    lib.tp_build(tab, p.ncols, zh.ctypes.data, zl.ctypes.data, lg.ctypes.data, k)
    r = search.distance(p, k_table=k, kmax=kmax, probe_fn=PROBE_FN(("tp_probe", lib)), probe_ctx=tab)
    dt = time.perf_counter() - t0
    lib.tp_free(tab)
    return {"seconds": dt, "distance": r["distance"], "cores": 1, "kind": "port"}


SECTIONS = {"batched": section_batched, "served": section_served, "sparse": section_sparse,
            "sparse_full": section_sparse_full, "tree": section_tree, "witness": section_witness,
            "search": section_search}


# ---------------------------------------------------------------------- GPU arm
def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        if rank == 0:
            run_reference(args)
        return
    if args.sparse_query:
        print(json.dumps(sparse_query(args.sparse_query)), flush=True)
        return
    if args.tree_only:
        print(json.dumps(section_tree(args)), flush=True)
        return
    import torch
    import torch.distributed as dist
    from tropidist_gb300 import _lib, auto, kernel, replicas
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    L = _lib.lib()
    p, order, plans = workload(args, rank)
    cps = [kernel.CompiledPlan(pl) for pl in plans if pl.feasible]
    peak = max(cp.peak_bits for cp in cps)
    a = torch.empty(1 << peak, dtype=torch.uint8, device="cuda")
    b = torch.empty(1 << peak, dtype=torch.uint8, device="cuda")
    st = torch.cuda.current_stream()
    # the observables alternate between two streams with a table pair each, as auto.dp_distance
    # runs them: one sweep's pass boundaries overlap the other's passes
    side = auto._side_stream()
    a2 = torch.empty(1 << peak, dtype=torch.uint8, device="cuda")
    b2 = torch.empty(1 << peak, dtype=torch.uint8, device="cuda")
    work = sum(cp.plan.work() for cp in cps)

    def step(timed=None):
        vals = []
        if timed is None:
            side.wait_stream(st)
        for k, cp in enumerate(cps):
            if timed is None:
                if k % 2:
                    cp.execute(a2, b2, stream=side.cuda_stream)
                else:
                    cp.execute(a, b)
            else:
                out = (ctypes.c_double * 12)()
                _lib.check(L.tg_dense_execute_timed(cp.handle, a.data_ptr(), b.data_ptr(), st.cuda_stream, out, 12))
                for k in range(12):
                    timed[k] += out[k]
            vals.append(cp)
        if timed is None:
            st.wait_stream(side)
        return vals

    for _ in range(args.warmup):
        step()
    values = [cp.result(a, b) for cp in cps[-1:]]
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    gpu_index = os.environ.get("CUDA_VISIBLE_DEVICES", str(local)).split(",")[local] if \
        os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",")[0].isdigit() else str(local)
    clocks = Clocks(gpu_index)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    acc = [0.0] * 12
    e0.record(st)
    for _ in range(args.steps):
        step()
    e1.record(st)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    clk = clocks.stop()
    # per-launch breakdown (an event pair around every launch), outside the timed region: the same
    # steps again; events between launches serialise them, so these launch times are conservative
    for _ in range(args.steps):
        step(acc)
    torch.cuda.synchronize()
    ms, total_work = replicas.aggregate(ms, work, device="cuda")
    value = total_work * args.steps / (ms / 1e3)
    launches = sum(cp.nsegs for cp in cps) * args.steps
    # distances of the four observables (checked for consistency with the e2e path below)
    dists, it = [], iter(cps)
    for pl in plans:
        if not pl.feasible:
            dists.append(None)
            continue
        cp = next(it)
        cp.execute(a, b)
        v = cp.result(a, b)
        dists.append("overflow" if v == 255 else v)
    gold = golden_headline(args)

    # end to end through the public API (host problem in, distance out)
    e2e_ms = []
    h2d = sum(cp.ops.nbytes for cp in cps)
    if args.e2e_steps:
        auto.dp_distance(p, order)           # warm-up: the API's own buffers come from the allocator once
    for _ in range(args.e2e_steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        best, per = auto.dp_distance(p, order)
        torch.cuda.synchronize()
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    if e2e_ms:
        assert per == [d if d != "overflow" else None for d in dists], (per, dists)
        e2e_value = work / (statistics.median(e2e_ms) / 1e3) * (world if world > 1 else 1)
    else:
        e2e_value = None

    peak_gbs, peak_kind = measured_peak()
    # the dominant kernel by GPU time: coset-streaming passes or fused tile passes
    kinds = {"k_fused_pass_u8": 1, "k_stream_pass_u8": 3}
    kname = max(kinds, key=lambda k: acc[3 * kinds[k] + 1])
    ki = kinds[kname]
    n_fp, ms_fp, bytes_fp = acc[3 * ki], acc[3 * ki + 1], acc[3 * ki + 2]
    # the kernel's average launch in the timed region: the region's time times the kernel's share of
    # the GPU time (from the per-launch events of the instrumented repeat, which serialise the
    # launches and so overstate each one) over its launches
    share = ms_fp / sum(acc[1::3]) if sum(acc[1::3]) else None
    avg_s = (ms / 1e3) * share / n_fp if (n_fp and share) else None
    achieved = (bytes_fp / n_fp) / avg_s / 1e9 if avg_s else None
    tr = traffic_per_launch(kname)
    roofline = {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": peak_gbs,
                "unit": "GB/s", "frac": achieved / peak_gbs if achieved else None,
                "peak_source": "measured hbm_gbs" if peak_kind == "measured" else peak_kind,
                "algorithmic_bytes_per_launch": bytes_fp / n_fp if n_fp else None,
                "avg_launch_us": 1e6 * avg_s if avg_s else None,
                "avg_launch_us_serialised": 1e3 * ms_fp / n_fp if n_fp else None, "launches": int(n_fp),
                "share_of_gpu_time": share,
                "traffic": (tr["ratio"] * bytes_fp / n_fp) if (tr and n_fp) else None,
                "whole_step_gbs": (sum(acc[2::3]) / args.steps) / (ms / args.steps / 1e3) / 1e9 if ms else None,
                "traffic_source": ("ncu DRAM/algorithmic bytes %.3f (profiles/), scaled to the average launch"
                                   % tr["ratio"]) if tr else None}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u8", "data": "synthetic (seeded banded problem)",
            "config": config(args, plans, dists),
            "parallelism": "replicas (one instance per rank)" if world > 1 else "1 GPU",
            "schedule": {"streams": 2, "fused_passes_per_step": int((acc[3] + acc[9]) / args.steps),
                         "streaming_passes_per_step": int(acc[9] / args.steps),
                         "segments_per_step": sum(cp.nsegs for cp in cps)},
            "parity": {"reference_fixture": dist_string(gold) if gold else None,
                       "equal": (dists == gold) if gold else None},
            "roofline": roofline, "clocks": clk, "gpu_launches": int(launches),
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": 4 * len(cps), "ms_per_step": statistics.median(e2e_ms) if e2e_ms else None,
                    "path": "tropidist_gb300.auto.dp_distance(problem, order)"}}
    if gold is not None and dists != gold:
        # the timed sweeps disagree with the reference's own distances: report and fail
        print(json.dumps(line), flush=True)
        raise SystemExit("distances %s differ from the reference's %s" % (dists, gold))
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_legs(p, order)
        if gold is not None and line["cpu_baseline"]["distance"] != gold[0]:
            raise SystemExit("the CPU port's distance differs from the reference's")
    del a, b, cps
    torch.cuda.empty_cache()
    sections = [x for x in args.sections.split(",") if x] if rank == 0 and world == 1 else []
    for name in sections:
        try:
            line[name] = SECTIONS[name](args)
        except Exception as e:          # a section's failure is reported in the line, not hidden
            line[name] = {"error": "%s: %s" % (type(e).__name__, e)}
        torch.cuda.empty_cache()
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
