"""Generate the golden vectors of the Rank DP path by running the reference itself.

Run in a checkout where the reference tree is available (default /root/reference, or the
REFERENCE environment variable).  The reference compiles its C kernels next to its sources, so
the script copies the needed parts to a temporary directory first.  Outputs (JSON, small) go
next to this script; the test-suite reads only those files.

  dense_random.json   random small problems (the generator of tests/test_dp.py:26-33): the
                      reference's plan ops, run_plan / run_plan_numpy values, brute-force truth
  dense_big.json      tests/test_dp.py:65-78 problems (tables >= 128 entries)
  dense_synth.json    seeded banded problems (tropidist_gb300.synth.dense_small, seeds 0-9):
                      plan digest, work, value, sha256 of the table after every 16th op
  dense_chain.json    the 8-bit boundary: chain(n) for n = 254, 255, 256 (tests/test_false_bounds.py:170-202)
  codes.json          stim-free known-answer codes: bb72 (Z), rotated surface d9/d15/d25, with the
                      reference's best_order and dense distances
  sparse_random.json  sparse_dp.query results on random small problems (tests/test_sparse_dp.py:41-46)
  sparse_tables.json  the reference's NumpyTables at every cut of a few sweeps (keys/vals digests)
  tables.json         completion-table builds (count) and lookups of random syndromes
  tree_dp.json        the tree DP (cdist/tree_dp.py) on random matrices and trees, logical queries,
                      distances beyond 255, larger joins  (`make_golden.py tree` writes only this)
  search.json         the weight-bounded search (cdist/search.py distance) on random problems
                      (`make_golden.py search` writes only this)
  headline.json       the benchmark's dense workload (banded m=1000 n=2000 window 37, 31-bit
                      frontier, four logical rows): op-stream digests, distances and two 2 GB
                      tables per observable (sha256 + histogram) from the reference's planner and
                      C kernels (`make_golden.py headline` writes only this; a few minutes)
"""
from __future__ import annotations

import hashlib
import json
import os
import random
import shutil
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF = os.environ.get("REFERENCE", "/root/reference")


def hexs(xs):
    return [format(int(x), "x") for x in xs]


def sha(arr):
    return hashlib.sha256(arr.tobytes()).hexdigest()[:16]


def ops_json(ops):
    return [list(op) for op in ops]


def main():
    tmp = tempfile.mkdtemp(prefix="tropi_ref_")
    for d in ("cdist", "papers", "scripts"):
        shutil.copytree(os.path.join(REF, d), os.path.join(tmp, d))
    sys.path[:0] = [tmp, os.path.join(tmp, "papers"), os.path.join(tmp, "scripts"), REPO]
    import numpy as np
    from cdist import kernel, trellis, auto, sparse_dp, search
    from cdist.problem import Problem
    import stabcode
    import dp_vs_search_local as dvs
    from tropidist_gb300 import synth

    out = {}

    # ---------------------------------------------------------------- dense: random small problems
    def brute(h, l, obs_mask):
        import itertools
        n = len(h)
        for w in range(1, n + 1):
            for sup in itertools.combinations(range(n), w):
                s = lg = 0
                for j in sup:
                    s ^= h[j]
                    lg ^= l[j]
                if s == 0 and bin(lg & obs_mask).count("1") & 1:
                    return w
        return None

    rng = random.Random(1)
    cases = []
    for t in range(300):
        m = rng.randint(1, 9)
        n = rng.randint(1, 14)
        k = rng.randint(1, 3)
        dens = rng.choice([0.15, 0.3, 0.5])
        h = [sum(1 << i for i in range(m) if rng.random() < dens) for _ in range(n)]
        l = [sum(1 << i for i in range(k) if rng.random() < 0.3) for _ in range(n)]
        order = list(range(n))
        rng.shuffle(order)
        obs_mask = rng.randrange(1, 1 << k)
        plan = trellis.build_plan(h, l, obs_mask, order, m)
        got_np = kernel.run_plan_numpy(plan)
        got_c, _ = kernel.run_plan(plan)
        cases.append({"m": m, "h": h, "l": l, "order": order, "obs_mask": obs_mask, "feasible": plan.feasible,
                      "peak_bits": plan.peak_bits, "work": plan.work(), "ops": ops_json(plan.ops),
                      "value_numpy": got_np, "value_c": got_c, "brute": brute(h, l, obs_mask)})
    out["dense_random.json"] = cases

    rng = random.Random(7)
    cases = []
    for t in range(40):
        m = rng.randint(10, 16)
        n = rng.randint(m + 4, m + 14)
        h = [rng.randrange(1, 1 << m) for _ in range(n)]
        l = [rng.randrange(0, 2) for _ in range(n)]
        plan = trellis.build_plan(h, l, 1, list(range(n)), m)
        a = kernel.run_plan_numpy(plan)
        b, _ = kernel.run_plan(plan)
        tabs = {}
        if plan.feasible:
            for nops, T in ref_tables(kernel, plan):
                tabs[nops] = sha(T)
        cases.append({"m": m, "h": h, "l": l, "feasible": plan.feasible, "peak_bits": plan.peak_bits,
                      "ops": ops_json(plan.ops), "value_numpy": a, "value_c": b, "table_sha": tabs})
    out["dense_big.json"] = cases

    # ---------------------------------------------------------------- dense: seeded banded problems
    cases = []
    for seed in range(10):
        p = synth.dense_small(seed)
        order = list(range(p.ncols))
        plan = trellis.build_plan(p.h, p.l, 1, order, p.nrows)
        v, _ = kernel.run_plan(plan)
        tabs = {}
        for nops, T in ref_tables(kernel, plan):
            if nops % 16 == 0 or nops == len(plan.ops):
                tabs[nops] = sha(T)
        enc = np.array([[0, 0, 0] if op[0] == "expand" else [1, op[1], 1] if op[0] == "update" else [2, op[1], op[2]]
                        for op in plan.ops], dtype=np.int64)
        cases.append({"seed": seed, "h": hexs(p.h), "l": hexs(p.l), "nrows": p.nrows, "peak_bits": plan.peak_bits,
                      "work": plan.work(), "nops": len(plan.ops), "ops_sha": sha(enc), "value": v,
                      "table_sha": tabs, "numpy_value": kernel.run_plan_numpy(plan)})
    out["dense_synth.json"] = cases

    # ---------------------------------------------------------------- dense: 8-bit boundary
    def chain(n):
        h = [1] + [(1 << (j - 1)) | (1 << j) for j in range(1, n - 1)] + [1 << (n - 2)]
        return Problem("chain", n - 1, 1, h, [1] + [0] * (n - 1), [(j, 0) for j in range(n - 1)])

    cases = []
    for n in (254, 255, 256):
        p = chain(n)
        plan = trellis.build_plan(p.h, p.l, 1, list(range(n)), p.nrows)
        rec = {"n": n, "h": hexs(p.h), "l": hexs(p.l), "nrows": p.nrows}
        try:
            rec["value"] = kernel.run_plan(plan)[0]
        except OverflowError:
            rec["value"] = "overflow"
        try:
            rec["witness"] = auto.dp_witness(p, list(range(n)), 0)
        except OverflowError:
            rec["witness"] = "overflow"
        cases.append(rec)
    out["dense_chain.json"] = cases

    # ---------------------------------------------------------------- known-answer codes
    cases = []
    builds = [("bb72_Z", lambda: stabcode.bb_matrices(6, 6, [(3, 0), (0, 1), (0, 2)], [(0, 3), (1, 0), (2, 0)]), "Z", 6)]
    for d in (9, 15, 25):
        builds.append(("surface_d%d_Z" % d, (lambda d=d: dvs.rotated_surface(d)), "Z", d))
    for name, mk, sector, d in builds:
        hx, hz, n = mk()
        p = stabcode.css_distance_problem(hx, hz, n, sector)
        order = auto.best_order(p)[0]
        best, per = auto.dp_distance(p, order)
        wit = auto.dp_witness(p, order, per.index(best)) if best is not None else None
        cases.append({"name": name, "nrows": p.nrows, "nobs": p.nobs, "h": hexs(p.h), "l": hexs(p.l),
                      "order": order, "distance": best, "per_obs": per, "known": d,
                      "cut_rank": max(trellis.cut_profile(p.h, order)), "witness": wit})
    out["codes.json"] = cases

    # ---------------------------------------------------------------- sparse DP
    rng = random.Random(3)
    cases = []
    for _ in range(40):
        n, m, k = rng.randint(2, 12), rng.randint(1, 7), rng.randint(1, 2)
        dens = rng.choice([0.2, 0.35, 0.5])
        h = [sum(1 << r for r in range(m) if rng.random() < dens) for _ in range(n)]
        l = [sum(1 << r for r in range(k) if rng.random() < 0.4) for _ in range(n)]
        p = Problem("rand", m, k, h, l, [(i, 0) for i in range(m)])
        order = list(range(n))
        rng.shuffle(order)
        for obs in range(k):
            tr = sparse_dp.Trellis.for_query(p, obs, order)
            rec = {"m": m, "k": k, "h": h, "l": l, "order": order, "obs": obs, "feasible": tr.feasible, "runs": []}
            if tr.feasible:
                rec["nslots"] = tr.nslots
                rec["slot"] = tr.slot
                rec["tmask"] = tr.tmask
                rec["col"] = tr.col
                for K in range(1, n + 2):
                    for mode, split in (("forward", None), ("mitm", None), ("mitm", 1), ("mitm", K)):
                        for use_h in (False, True):
                            r = sparse_dp.query(tr, K, mode=mode, split=split, use_h=use_h, backend="c")
                            rec["runs"].append({"K": K, "mode": mode, "split": split, "use_h": use_h,
                                                "value": r["value"], "witness": r["witness"],
                                                "peak_states": r["peak_states"],
                                                "forward_total": int(sum(r.get("forward_counts", [0]))),
                                                "backward_total": int(sum(r.get("backward_counts", [0])))})
            cases.append(rec)
    out["sparse_random.json"] = cases

    cases = []
    for seed in range(3):
        p = synth.dense_small(seed)
        order = list(range(p.ncols))
        tr = sparse_dp.Trellis.for_query(p, 0, order)
        for fwd, K, use_h in ((True, 6, True), (False, 4, False), (True, 5, False)):
            sw = sparse_dp.Sweep(tr, +1 if fwd else -1, K, K, use_h=use_h, every=1, backend="numpy")
            sw.run()
            digest = {}
            for c, (keys, vals) in sorted(sw.ckpt.items()):
                digest[c] = [int(keys.size), sha(keys), sha(vals)]
            cases.append({"seed": seed, "forward": fwd, "K": K, "use_h": use_h, "h": hexs(p.h), "l": hexs(p.l),
                          "nrows": p.nrows, "counts": sw.counts, "tables": digest})
    out["sparse_tables.json"] = cases

    # ---------------------------------------------------------------- completion tables
    cases = []
    rng = random.Random(11)
    for t in range(6):
        m = rng.randint(20, 60)
        n = rng.randint(30, 80)
        nobs = rng.randint(1, 3)
        h = [sum(1 << r for r in rng.sample(range(m), rng.randint(1, 3))) for _ in range(n)]
        l = [rng.randrange(0, 1 << nobs) for _ in range(n)]
        p = Problem("tab", m, nobs, h, l, [(i, 0) for i in range(m)])
        k = 2 if n > 50 else 3
        T = search.Table(p, k)
        # probe: syndromes of random column sets of size 1..k+1 with a random label
        probes = []
        for _ in range(200):
            sz = rng.randint(1, k + 1)
            cols = rng.sample(range(n), sz)
            s = g = 0
            for j in cols:
                s ^= h[j]
                g ^= l[j]
            probes.append({"syn": format(s, "x"), "lg": g, "R": rng.randint(0, k)})
        cases.append({"m": m, "n": n, "nobs": nobs, "h": hexs(h), "l": l, "k": k, "seed": 12345,
                      "log2slots": T.log2slots, "entries": int(T.entries), "zh": hexs(T.zh), "zl": hexs(T.zl),
                      "probes": probes})
        T.free()
    out["tables.json"] = cases

    for name, data in out.items():
        with open(os.path.join(HERE, name), "w") as f:
            json.dump(data, f, separators=(",", ":"))
        print("wrote", name, os.path.getsize(os.path.join(HERE, name)), "bytes")
    shutil.rmtree(tmp, ignore_errors=True)


def ref_tables(kernel, plan):
    """(ops done, table) after every call of the reference's C kernels, driven in the order of
    its executor loop (cdist/kernel.py:112-135: an expand followed by the update of the starting
    column is one dp_expand_update call, so no table is yielded between those two ops)."""
    import ctypes
    import numpy as np
    L = kernel.lib()
    u8p = ctypes.POINTER(ctypes.c_uint8)
    buf = np.zeros(1 << plan.peak_bits, dtype=np.uint8)
    ptr = buf.ctypes.data_as(u8p)
    n, i, ops = 1, 0, plan.ops
    while i < len(ops):
        op = ops[i]
        if op[0] == "expand":
            nxt = ops[i + 1]
            if nxt[0] == "update" and (nxt[1] >> n.bit_length() - 1) == 1:
                L.dp_expand_update(ptr, n, nxt[1] ^ n)
                n <<= 1
                i += 2
            else:
                L.dp_fill(ctypes.cast(ctypes.addressof(ptr.contents) + n, u8p), n, 255)
                n <<= 1
                i += 1
        elif op[0] == "update":
            L.dp_update(ptr, n, op[1])
            i += 1
        else:
            n = L.dp_select(ptr, n, op[1], op[2])
            i += 1
        yield i, buf[:n].copy()


def tree_main():
    """tree_dp.json: the reference's tree DP (C executor) on random matrices and tree shapes, the
    logical-query front end, the distances beyond 255 and a few joins of 2^16-2^22 pairs."""
    tmp = tempfile.mkdtemp(prefix="tropi_ref_")
    shutil.copytree(os.path.join(REF, "cdist"), os.path.join(tmp, "cdist"))
    sys.path[:0] = [tmp]
    from cdist.tree_dp import CompiledTreeDP, tree_min_distance_for_mask

    def balanced(xs):
        if not xs:
            return None
        if len(xs) == 1:
            return xs[0]
        m = len(xs) // 2
        return [balanced(xs[:m]), balanced(xs[m:])]

    def comb(xs):
        if not xs:
            return None
        t = xs[0]
        for x in xs[1:]:
            t = [t, x]
        return t

    def rtree(xs, rng):
        if len(xs) == 1:
            return xs[0]
        k = rng.randrange(1, len(xs))
        return [rtree(xs[:k], rng), rtree(xs[k:], rng)]

    def tup(t):
        return tuple(tup(x) for x in t) if isinstance(t, list) else t

    keys = ("edge_state_dimensions", "max_join_dimension", "join_work", "peak_live_table_bytes",
            "largest_table_bytes", "dtype", "infinity", "matrix_rank")
    rng = random.Random(2026)
    affine = []
    for trial in range(120):
        m, n = rng.randint(1, 8), rng.randint(1, 14)
        cols = [rng.randrange(1 << m) for _ in range(n)]
        order = list(range(n))
        rng.shuffle(order)
        tree = (comb(order), balanced(order), rtree(order, rng))[trial % 3]
        prog = CompiledTreeDP(cols, tup(tree))
        pf = prog.preflight()
        targets = sorted({rng.randrange(1 << m) for _ in range(6)} | {0})
        affine.append({"columns": cols, "tree": tree, "targets": targets,
                       "distances": [prog.run(t)[0] for t in targets], "profile": {k: pf[k] for k in keys}})
    logical = []
    for trial in range(60):
        n, m, nobs = rng.randrange(1, 13), rng.randrange(0, 7), rng.randrange(1, 4)
        h = [rng.randrange(1 << m) for _ in range(n)]
        l = [rng.randrange(1 << nobs) for _ in range(n)]
        order = list(range(n))
        rng.shuffle(order)
        tree = (comb(order), balanced(order), rtree(order, rng))[trial % 3]
        mask = rng.randrange(1 << nobs)
        d, st = tree_min_distance_for_mask(h, l, mask, tup(tree))
        logical.append({"h": h, "l": l, "mask": mask, "tree": tree, "distance": d,
                        "edge_state_dimensions": st["edge_state_dimensions"]})
    chains = []
    for n in (254, 255, 300):
        h = [1] + [(1 << (j - 1)) | (1 << j) for j in range(1, n - 1)] + [1 << (n - 2)]
        l = [1] + [0] * (n - 1)
        d, st = tree_min_distance_for_mask(h, l, 1, tup(balanced(list(range(n)))))
        chains.append({"ncols": n, "distance": d, "dtype": st["dtype"], "infinity": st["infinity"]})
    large = []
    for trial in range(6):
        # random sparse columns over 16-22 rows; a balanced tree gives joins of 2^16-2^22 pairs
        m = rng.randint(16, 22)
        n = rng.randint(40, 64)
        cols = [sum(1 << r for r in rng.sample(range(m), rng.randint(1, 3))) for _ in range(n)]
        order = list(range(n))
        rng.shuffle(order)
        tree = balanced(order) if trial % 2 == 0 else rtree(order, rng)
        prog = CompiledTreeDP(cols, tup(tree))
        pf = prog.preflight(max_join_work=None, max_memory_bytes=None)
        if pf["max_join_dimension"] > 24:
            continue
        targets = [0] + [rng.randrange(1 << m) for _ in range(3)]
        ds = [prog.run(t, max_join_work=None, max_memory_bytes=None, max_seconds=None)[0] for t in targets]
        large.append({"columns": cols, "tree": tree, "targets": targets, "distances": ds,
                      "profile": {k: pf[k] for k in keys}})
    out = {"affine": affine, "logical": logical, "chains": chains, "large": large}
    with open(os.path.join(HERE, "tree_dp.json"), "w") as f:
        json.dump(out, f, separators=(",", ":"))
    print("wrote tree_dp.json", os.path.getsize(os.path.join(HERE, "tree_dp.json")), "bytes;",
          len(large), "large cases, max join dims", [c["profile"]["max_join_dimension"] for c in large])
    shutil.rmtree(tmp, ignore_errors=True)


def search_main():
    """search.json: the reference's weight-bounded search (cdist/search.py distance, completion
    table k = 2) on random problems, with brute-force truth where it is affordable."""
    import itertools
    tmp = tempfile.mkdtemp(prefix="tropi_ref_")
    shutil.copytree(os.path.join(REF, "cdist"), os.path.join(tmp, "cdist"))
    sys.path[:0] = [tmp]
    from cdist import search
    from cdist.problem import Problem

    def brute(h, l):
        n = len(h)
        for w in range(1, n + 1):
            for cols in itertools.combinations(range(n), w):
                x = g = 0
                for j in cols:
                    x ^= h[j]
                    g ^= l[j]
                if x == 0 and g != 0:
                    return w
        return None

    rng = random.Random(77)
    cases = []
    for t in range(60):
        m = rng.randint(3, 14)
        n = rng.randint(4, 30 if t % 2 else 14)
        nobs = rng.randint(1, 3)
        h = [sum(1 << r for r in rng.sample(range(m), rng.randint(1, min(3, m)))) for _ in range(n)]
        l = [rng.randrange(1 << nobs) for _ in range(n)]
        p = Problem("rand%d" % t, m, nobs, h, l, [(i, 0) for i in range(m)])
        r = search.distance(p, k_table=2, kmax=min(n, 12))
        case = {"m": m, "n": n, "nobs": nobs, "h": h, "l": l, "k_table": 2, "kmax": min(n, 12),
                "distance": r["distance"], "lower_bound": r["lower_bound"]}
        if n <= 14:
            case["brute"] = brute(h, l)
        cases.append(case)
    with open(os.path.join(HERE, "search.json"), "w") as f:
        json.dump(cases, f, separators=(",", ":"))
    print("wrote search.json", len(cases), "cases", os.path.getsize(os.path.join(HERE, "search.json")), "bytes")
    shutil.rmtree(tmp, ignore_errors=True)


def headline_checkpoints(ops, peak_bits):
    """Op counts at which the headline fixture records the table: the first op after half of the
    plan and the first after three quarters at which the table is at least 2^(peak_bits - 1)
    entries wide, each on a boundary of the reference's executor calls (not between an expand and
    the update of its starting column)."""
    out, w = [], 0
    widths = []
    for op in ops:
        w += 1 if op[0] == "expand" else -1 if op[0] == "select" else 0
        widths.append(w)
    for frac in (2, 4 / 3):
        k = next(i for i in range(int(len(ops) / frac), len(ops))
                 if widths[i - 1] >= peak_bits - 1 and ops[i - 1][0] != "expand")
        out.append(k)
    return out


def headline_main():
    """headline.json: the benchmark's dense workload (tropidist_gb300.synth.dense_scale(0, window=37):
    banded m=1000 n=2000, col-weight 3, natural order, 31-bit frontier, four logical rows one at a
    time) planned by the reference's own cdist/trellis.py and swept by its own C kernels
    (cdist/viterbi.c through its executor order): per observable the op-stream digest, work,
    value, and the sha256 and value histogram of the table at two checkpoints near full width."""
    import ctypes
    import numpy as np
    tmp = tempfile.mkdtemp(prefix="tropi_ref_")
    shutil.copytree(os.path.join(REF, "cdist"), os.path.join(tmp, "cdist"))
    sys.path[:0] = [tmp, REPO]
    from cdist import kernel, trellis
    from tropidist_gb300 import synth
    p = synth.dense_scale(0, window=37)
    order = list(range(p.ncols))
    L = kernel.lib()
    u8p = ctypes.POINTER(ctypes.c_uint8)
    cases = []
    for o in range(p.nobs):
        plan = trellis.build_plan(p.h, p.l, 1 << o, order, p.nrows)
        enc = np.array([[0, 0, 0] if op[0] == "expand" else [1, op[1], 1] if op[0] == "update"
                        else [2, op[1], op[2]] for op in plan.ops], dtype=np.int64)
        ks = headline_checkpoints(plan.ops, plan.peak_bits)
        buf = np.zeros(1 << plan.peak_bits, dtype=np.uint8)
        ptr = buf.ctypes.data_as(u8p)
        n, i, ops, tabs = 1, 0, plan.ops, {}
        while i < len(ops):                       # the executor order of cdist/kernel.py:112-135
            op = ops[i]
            if op[0] == "expand":
                nxt = ops[i + 1]
                if nxt[0] == "update" and (nxt[1] >> n.bit_length() - 1) == 1:
                    L.dp_expand_update(ptr, n, nxt[1] ^ n)
                    i += 2
                else:
                    L.dp_fill(ctypes.cast(ctypes.addressof(ptr.contents) + n, u8p), n, 255)
                    i += 1
                n <<= 1
            elif op[0] == "update":
                L.dp_update(ptr, n, op[1])
                i += 1
            else:
                n = L.dp_select(ptr, n, op[1], op[2])
                i += 1
            if i in ks:
                t = buf[:n]
                tabs[str(i)] = {"sha": hashlib.sha256(memoryview(t)).hexdigest()[:16], "entries": int(n),
                                "hist": np.bincount(t, minlength=256).tolist()}
        assert n == 1
        value = kernel.final_value(buf[0])
        cases.append({"observable": o, "peak_bits": plan.peak_bits, "work": plan.work(), "nops": len(plan.ops),
                      "ops_sha": sha(enc), "value": value, "tables": tabs,
                      "threads": L.dp_num_threads()})
        print("observable", o, "value", value, "peak", plan.peak_bits, "checkpoints", sorted(tabs), flush=True)
    with open(os.path.join(HERE, "headline.json"), "w") as f:
        json.dump({"workload": "synth.dense_scale(0, window=37), natural order, 4 logical rows", "cases": cases},
                  f, separators=(",", ":"))
    print("wrote headline.json", os.path.getsize(os.path.join(HERE, "headline.json")), "bytes")
    shutil.rmtree(tmp, ignore_errors=True)


if __name__ == "__main__":
    if sys.argv[1:] == ["tree"]:
        tree_main()
    elif sys.argv[1:] == ["search"]:
        search_main()
    elif sys.argv[1:] == ["headline"]:
        headline_main()
    else:
        main()
        tree_main()
        search_main()
