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
`roofline` reports the fused tile pass (the dominant kernel): table bytes read + written per
launch over its average CUDA-event launch time, against the measured HBM copy bandwidth.
`cpu_baseline` times the C/OpenMP port of the reference's kernels (oracle/dense_port.c) on the
host cores over a window of the same plan at full width.

--impl reference runs that CPU implementation alone (all host threads) on the same workload,
each step a bounded window of ops of the first observable's plan.
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
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    return ap.parse_args()


def workload(args, rank=0):
    from tropidist_gb300 import synth, trellis
    p = synth.dense_scale(args.seed + rank, window=args.window)
    order = list(range(p.ncols))
    plans = [trellis.build_plan(p.h, p.l, 1 << o, order, p.nrows) for o in range(p.nobs)]
    return p, order, plans


def config(args, plans, extra=None):
    c = {"workload": "dense Rank DP, banded m=1000 n=2000 col-weight 3 window %d, 4 logical rows one at a time"
                     % args.window,
         "m": 1000, "n": 2000, "window": args.window, "seed": args.seed, "observables": len(plans),
         "peak_bits": max(pl.peak_bits for pl in plans), "table_bytes": 1 << max(pl.peak_bits for pl in plans),
         "work_per_step": int(sum(pl.work() for pl in plans)), "entry": "uint8",
         "l2": "inputs larger than L2 (2 GB tables), no flush"}
    if extra:
        c.update(extra)
    return c


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
    return L


def cpu_window(plan, seconds, threads=None):
    """Time the C port on a window of the plan's ops starting where the table first reaches
    peak_bits - 1 (the prefix that gets there runs untimed).  Returns (rate, work, secs, desc)."""
    import numpy as np
    from tropidist_gb300 import trellis
    if threads:
        os.environ["OMP_NUM_THREADS"] = str(threads)
    L = port_lib()
    enc = trellis.encode_ops(plan.ops)
    w, start = 0, None
    for i, op in enumerate(plan.ops):
        w += 1 if op[0] == "expand" else -1 if op[0] == "select" else 0
        if w >= plan.peak_bits - 1:
            start = i + 1
            break
    buf = np.zeros(1 << plan.peak_bits, dtype=np.uint8)
    n = L.port_run_plan(enc.ctypes.data, start, buf.ctypes.data, 1)
    i, work, t0 = start, 0, time.perf_counter()
    bits = int(n).bit_length() - 1
    while i < len(enc) and time.perf_counter() - t0 < seconds:
        j = min(len(enc), i + 8)
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
    desc = "ops %d..%d of observable 0's plan (%.3g state-updates, table 2^%d..2^%d), C/OpenMP port" % (
        start, i, work, plan.peak_bits - 1, plan.peak_bits)
    return work / secs, work, secs, desc, L.port_num_threads()


def run_reference(args):
    p, order, plans = workload(args)
    plan = plans[0]
    cores = None
    rates = []
    per_step = max(1.0, min(6.0, args.cpu_seconds / 3))
    for k in range(args.warmup + args.steps):
        rate, work, secs, desc, cores = cpu_window(plan, per_step)
        if k >= args.warmup:
            rates.append((work, secs))
    work = sum(w for w, _ in rates)
    secs = sum(s for _, s in rates)
    value = work / secs
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * secs / max(1, args.steps), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic (seeded banded problem)",
            "impl": "reference",
            "config": config(args, plans, {"sample": desc}),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": desc},
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
    import torch
    import torch.distributed as dist
    from tropidist_gb300 import _lib, auto, kernel
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
    work = sum(cp.plan.work() for cp in cps)

    def step(timed=None):
        vals = []
        for cp in cps:
            if timed is None:
                cp.execute(a, b)
            else:
                out = (ctypes.c_double * 12)()
                _lib.check(L.tg_dense_execute_timed(cp.handle, a.data_ptr(), b.data_ptr(), st.cuda_stream, out, 12))
                for k in range(12):
                    timed[k] += out[k]
            vals.append(cp)
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
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
        wt = torch.tensor([float(work)], device="cuda")
        dist.all_reduce(wt)
        total_work = float(wt.item())
    else:
        total_work = float(work)
    value = total_work * args.steps / (ms / 1e3)
    launches = sum(cp.nsegs for cp in cps) * args.steps
    # distances of the four observables (checked for consistency with the e2e path below)
    dists = []
    for cp in cps:
        cp.execute(a, b)
        dists.append(cp.result(a, b))

    # end to end through the public API (host problem in, distance out)
    e2e_ms = []
    h2d = sum(cp.ops.nbytes for cp in cps)
    for _ in range(args.e2e_steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        best, per = auto.dp_distance(p, order)
        torch.cuda.synchronize()
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    if e2e_ms:
        assert per == dists, (per, dists)
        e2e_value = work / (statistics.median(e2e_ms) / 1e3) * (world if world > 1 else 1)
    else:
        e2e_value = None

    peak_gbs, peak_kind = measured_peak()
    # the dominant kernel by GPU time: coset-streaming passes or fused tile passes
    kinds = {"k_fused_pass_u8": 1, "k_stream_pass_u8": 3}
    kname = max(kinds, key=lambda k: acc[3 * kinds[k] + 1])
    ki = kinds[kname]
    n_fp, ms_fp, bytes_fp = acc[3 * ki], acc[3 * ki + 1], acc[3 * ki + 2]
    achieved = (bytes_fp / n_fp) / (ms_fp / n_fp / 1e3) / 1e9 if n_fp else None
    tr = traffic_per_launch(kname)
    roofline = {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": peak_gbs,
                "unit": "GB/s", "frac": achieved / peak_gbs if achieved else None,
                "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else peak_kind,
                "algorithmic_bytes_per_launch": bytes_fp / n_fp if n_fp else None,
                "avg_launch_us": 1e3 * ms_fp / n_fp if n_fp else None, "launches": int(n_fp),
                "share_of_gpu_time": ms_fp / sum(acc[1::3]) if sum(acc[1::3]) else None,
                "traffic": (tr["ratio"] * bytes_fp / n_fp) if (tr and n_fp) else None,
                "whole_step_gbs": (sum(acc[2::3]) / args.steps) / (ms / args.steps / 1e3) / 1e9 if ms else None,
                "traffic_source": ("ncu DRAM bytes / algorithmic bytes = %.3f on %s, scaled to the average launch"
                                   % (tr["ratio"], tr["source"])) if tr else None}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u8", "data": "synthetic (seeded banded problem)",
            "config": config(args, plans, {"parallelism": "replicas (one instance per rank)" if world > 1 else "1 GPU",
                                           "distances": dists,
                                           "fused_passes_per_step": int((acc[3] + acc[9]) / args.steps),
                                           "streaming_passes_per_step": int(acc[9] / args.steps),
                                           "segments_per_step": sum(cp.nsegs for cp in cps)}),
            "roofline": roofline, "clocks": clk, "gpu_launches": int(launches),
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": 4 * len(cps), "ms_per_step": statistics.median(e2e_ms) if e2e_ms else None,
                    "path": "tropidist_gb300.auto.dp_distance(problem, order)"}}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        rate, cwork, secs, desc, cores = cpu_window(plans[0], args.cpu_seconds)
        line["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": cores, "kind": "port", "sample": desc,
                                "seconds": secs}
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
