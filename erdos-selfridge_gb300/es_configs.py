#!/usr/bin/env python3
"""Fixed-scope scans of the engine's measurement suite (one GPU), as reusable functions + CLI.

    python erdos-selfridge_gb300/es_configs.py batch64 [--json out.json]
    python erdos-selfridge_gb300/es_configs.py k390 [--log2-positions 40]
    python erdos-selfridge_gb300/es_configs.py small-k --bfile data/b003458.txt

* small-k: g(k) for k = 40..120 by the block-ordered search (GpuSieve.search), each checked
  against known values when a b-file is given.
* batch64: 64 seeded instances (k uniform in 150..400, range lengths log-uniform in 2^20..2^32
  positions of block 0, each with its own planner wheel) in ONE persistent work-stealing launch
  replayed from a CUDA graph, launch shape from the autotuner, against one launch per instance.
* replay: whole blocks of recorded frontier wheels (k = 378..400), each compared with the
  reference driver's recorded audit record (survivor counts and sha256 of the survivors).
* mitm: the meet-in-the-middle search for a few k, with the scan kernel's candidate rate.
* k390: the two recorded k = 390 wheels (primary and confirmation of evidence/through400/
  runs.json) over positions [0, 2^40) of block 0 in one persistent launch; every survivor of
  either wheel that the other wheel's scanned prefix covers must be a survivor there too.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)

import es_autotune  # noqa: E402
import es_gb300  # noqa: E402
import es_native as N  # noqa: E402

# The recorded k = 390 wheels (evidence/through400/runs.json, terms[k=390].primary/.confirmation)
K390_WHEELS = {
    "primary": [[3, 6], [2, 9], [211, 1], [139, 1], [103, 1], [137, 1], [101, 1], [67, 1], [5, 2],
                [199, 1], [23, 2], [79, 1], [197, 1], [131, 1], [7, 2], [17, 1]],
    "confirmation": [[3, 6], [2, 9], [211, 1], [139, 1], [103, 1], [137, 1], [101, 1], [67, 1],
                     [199, 1], [23, 2], [11, 1], [79, 1], [197, 1], [131, 1], [7, 2], [17, 1]],
}


def batch64_instances(seed: int = 0, count: int = 64):
    """(k_i, L_i): k uniform in 150..400, L log-uniform in [2^20, 2^32) positions."""
    rng = np.random.default_rng(seed)
    ks = rng.integers(150, 401, size=count)
    L = np.floor(2.0 ** rng.uniform(20, 32, size=count)).astype(np.int64)
    return [int(x) for x in ks], [int(x) for x in L]


def small_k(ks=range(40, 121), known: dict | None = None) -> dict:
    t0 = time.time()
    out = {}
    for k in ks:
        r = es_gb300.GpuSieve(es_gb300.Plan(k)).search(None)
        out[k] = {"status": r["status"], "g": r.get("g"), "block": r.get("block"),
                  "match": (known.get(k) == r.get("g")) if known else None}
    return {"cases": out, "wall_s": time.time() - t0,
            "all_match": all(v["match"] for v in out.values()) if known else None}


def batch64(seed: int = 0, autotune: bool = True, reps: int = 5, items_log2: int = 24,
            tune: dict | None = None) -> dict:
    """Config 3.  Besides the timings it returns, for every instance of at most 2^items_log2
    positions, the survivors and per-stage counts of a counting batch (``small_items``), which
    the GPU tests check against the oracle.  The launch shape starts from the library's per-class
    layout choice (ES_LAYOUT_AUTO) and `tune`; the autotuner then searches from there."""
    ks, L = batch64_instances(seed)
    plans = [es_gb300.Plan(k) for k in ks]
    tune0 = N.make_tune(**es_autotune.DEFAULT)
    ctxs = [N.Context(p, tune0) for p in plans]
    items, positions = [], 0
    for i, (p, c, length) in enumerate(zip(plans, ctxs, L)):
        n_outer = -(-min(length, p.R) // c.r0)
        items.append((i, i, 0, 0, n_outer))
        positions += n_outer * c.r0
    start = dict(es_autotune.DEFAULT, layout=N.LAYOUT_AUTO)
    start.update(tune or {})
    tune, tune_ms = (es_autotune.tune_batch(ctxs, items, start=start) if autotune else (start, None))
    b = N.Batch(ctxs, items, N.make_tune(**tune))
    b.run(use_graph=True)
    b.sync()
    ms = []
    for _ in range(reps):
        b.run(use_graph=True)
        ms.append(b.sync())
    batch_ms = statistics.median(ms)
    surv = b.survivors()
    b.close()
    # one launch per instance, each on its own context, synchronised like a per-instance driver
    single_ms, t_wall = [], time.perf_counter()
    for c, (_, _, _, ob, oe) in zip(ctxs, items):
        c.set_tune(N.make_tune(**tune))
        c.set_block(0)
        c.reset()
        single_ms.append(c.launch_timed(ob, oe - ob))
    single_wall = (time.perf_counter() - t_wall) * 1e3
    # per-item survivors and stage counts of a counting batch, for the small items
    bc = N.Batch(ctxs, items, N.make_tune(**dict(tune, count_stages=1)))
    bc.run(use_graph=False)
    bc.sync()
    sc = bc.survivors()
    small = []
    for i, (p, c, it) in enumerate(zip(plans, ctxs, items)):
        if (it[4] - it[3]) * c.r0 > (1 << items_log2):
            continue
        small.append({"item": i, "k": p.k, "o_range": [it[3], it[4]],
                      "survivors": sorted(int(r["idx"]) for r in sc if r["item"] == i),
                      "counts": [int(x) for x in bc.item_counts(i)]})
    bc.close()
    for c in ctxs:
        c.close()
    return {"instances": len(items), "positions": positions, "tune": tune,
            "batch_ms": batch_ms, "batch_Gcand_s": positions / batch_ms / 1e6,
            "single_ms_device_sum": sum(single_ms), "single_ms_wall": single_wall,
            "single_Gcand_s_device": positions / sum(single_ms) / 1e6,
            "single_Gcand_s_wall": positions / single_wall / 1e6,
            "speedup_vs_single_wall": single_wall / batch_ms,
            "survivors": int(len(surv)), "small_items": small}


def k390(log2_positions: int = 40, filter_orders: dict | None = None, tune: dict | None = None,
         reps: int = 1, autotune: bool = False, tune_log2: int = 34) -> dict:
    """Both recorded wheels over [0, 2^log2_positions) of block 0 in one persistent launch.  With
    autotune the launch shape (inner-stage depth, layout, CTA size, strip) is chosen by the batch
    autotuner on a 2^tune_log2-position prefix of each wheel first."""
    plans = {}
    for role, wheel in K390_WHEELS.items():
        order = (filter_orders or {}).get(role)
        plans[role] = es_gb300.Plan(390, None, wheel, filter_order=order)
    F = es_autotune.DEFAULT["mask_filters"]
    t = dict(es_autotune.DEFAULT, layout=N.layout_for_plan(plans["primary"], F))
    t.update(tune or {})
    ctxs = [N.Context(plans[r], N.make_tune(**t)) for r in ("primary", "confirmation")]
    if autotune:
        small = [(i, i, 0, 0, min(c.n_outer, -(-(1 << tune_log2) // c.r0))) for i, c in enumerate(ctxs)]
        t, _ = es_autotune.tune_batch(ctxs, small, start=t)
    pos = 1 << log2_positions
    items = []
    for i, c in enumerate(ctxs):
        n_outer = min(c.n_outer, -(-pos // c.r0))
        items.append((i, i, 0, 0, n_outer))
    b = N.Batch(ctxs, items, N.make_tune(**t))
    b.run(use_graph=True)          # the first run captures and instantiates the graph
    b.sync()
    ms, wall = [], []
    for _ in range(max(1, reps)):
        t0 = time.perf_counter()
        b.run(use_graph=True)
        ms.append(b.sync())        # device time: CUDA events around the replayed graph
        wall.append((time.perf_counter() - t0) * 1e3)   # host wall time of the same run
    surv = b.survivors()
    b.close()
    res = {}
    sets = {}
    for i, role in enumerate(("primary", "confirmation")):
        P = plans[role]
        idx = sorted(int(r["idx"]) for r in surv if r["item"] == i)
        sets[role] = (P, set(idx), items[i][4] * ctxs[i].r0)
        res[role] = {"M_bits": P.M.bit_length(), "r0": P.radix[0], "positions": items[i][4] * ctxs[i].r0,
                     "survivors": len(idx), "survivors_n": [str(P.idx_to_n(x, 0)) for x in idx[:64]]}
    # cross-wheel agreement: n admissible, n < M_other and inside the other's scanned prefix
    disagree = []
    for a, b_ in (("primary", "confirmation"), ("confirmation", "primary")):
        PA, SA, _ = sets[a]
        PB, SB, limB = sets[b_]
        for ia in SA:
            n = PA.idx_to_n(ia, 0)
            if n >= PB.M:
                continue
            tb = PB.n_to_idx(n)
            if tb is None or tb[1] >= limB:
                continue
            if tb[1] not in SB:
                disagree.append({"n": str(n), "in": a, "missing_from": b_})
    total_pos = sum(v["positions"] for v in res.values())
    ms_med = statistics.median(ms)
    for c in ctxs:
        c.close()
    return {"wheels": res, "ms": ms_med, "wall_ms": statistics.median(wall), "Gcand_s": total_pos / ms_med / 1e6,
            "tune": t, "cross_checked": True, "disagreements": disagree}


def k390_learned(model_path: str, log2_positions: int = 40, reps: int = 2, autotune: bool = True) -> dict:
    """The k = 390 fixed-scope confirmation scan with the learned cascade order of each wheel
    against the same scan in the analytic (reference) order.  Both arms get the same engine
    tuning: the batch autotuner picks each arm's launch shape for its own orders."""
    import es_learned
    model = es_learned.CostModel.load(model_path)
    orders, names = {}, {}
    for role, wheel in K390_WHEELS.items():
        P = es_gb300.Plan(390, None, wheel)
        names[role], orders[role] = es_learned.learned_order(model, P)
    learned = k390(log2_positions, filter_orders=orders, reps=reps, autotune=autotune)
    analytic = k390(log2_positions, reps=reps, autotune=autotune)
    same = all(learned["wheels"][r]["survivors_n"] == analytic["wheels"][r]["survivors_n"]
               for r in K390_WHEELS)
    return {"learned_orders": names, "learned_tune": learned["tune"], "analytic_tune": analytic["tune"],
            "learned_ms": learned["ms"], "analytic_ms": analytic["ms"],
            "learned_Gcand_s": learned["Gcand_s"], "analytic_Gcand_s": analytic["Gcand_s"],
            "wall_ratio_analytic_over_learned": analytic["ms"] / learned["ms"],
            "survivors_identical": same, "disagreements": learned["disagreements"] + analytic["disagreements"],
            "learned": learned, "analytic": analytic}


def mitm(ks, mem_gb: float = 8.0, bound_mult: float = 3.0) -> dict:
    """The meet-in-the-middle search per k (es_mitm.mitm_gpu) with its wall time, and the scan
    kernel alone on the final round's bound: candidates tested per second of device time."""
    import es_mitm
    out = {}
    for k in ks:
        t0 = time.perf_counter()
        r = es_mitm.mitm_gpu(k, mem_gb, bound_mult)
        wall = time.perf_counter() - t0
        row = {"status": r["status"], "g": r.get("g"), "wall_s": wall, "M_bits": r.get("M_bits"),
               "S1": r.get("S1"), "S2": r.get("S2"), "candidates": r.get("candidates")}
        if r["status"] == "FOUND":
            P = es_mitm.MitmPlan(k, mem_gb)
            eng = es_mitm.MitmEngine(P)
            eng.scan(r["bound"])                      # warm
            t1 = time.perf_counter()
            _, cand = eng.scan(r["bound"])
            dt = time.perf_counter() - t1
            eng.close()
            row.update({"final_bound": str(r["bound"]), "final_round_candidates": cand,
                        "final_round_s": dt, "Gcand_s": cand / dt / 1e9 if dt else None,
                        "s1_per_s": P.n1 / dt if dt else None})
        out[k] = row
    return {"cases": out, "mem_gb": mem_gb, "bound_mult": bound_mult}


AUDIT_FIELDS = ("residues_enumerated", "kernel_survivors", "after_n_gt_k_plus_1", "passed_ref_is_good",
                "sha256_survivors")


def replay(cases, chunk_log2: int = 40) -> dict:
    """Whole-block replays of recorded frontier wheels: every position of block t through the
    drop-in scan_block, then the reference driver's audit record (counts and survivor hash),
    compared field by field with the recorded one."""
    out = []
    for c in cases:
        plan = es_gb300.Plan(c["k"], {"chunk_log2": chunk_log2}, c["wheel"])
        assert str(plan.M) == str(c["M"]) and plan.R == int(c["R"]), "wheel does not rebuild"
        sieve = es_gb300.GpuSieve(plan)
        t = int(c["audit"]["t"])
        t0 = time.perf_counter()
        idx = sieve.scan_block(t)
        wall = time.perf_counter() - t0
        audit = es_gb300.block_audit(plan, t, idx)
        same = {f: audit[f] == c["audit"][f] for f in AUDIT_FIELDS}
        out.append({"k": c["k"], "role": c["role"], "t": t, "R": plan.R, "wall_s": wall,
                    "Gcand_s": plan.R / wall / 1e9, "mask_mode": sieve.mask_mode,
                    "audit": audit, "matches_record": all(same.values()), "fields": same})
    return {"cases": out, "all_match": all(x["matches_record"] for x in out),
            "positions": sum(x["R"] for x in out), "wall_s": sum(x["wall_s"] for x in out)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("which", choices=["small-k", "batch64", "k390", "k390-learned", "replay", "mitm"])
    ap.add_argument("--k", type=int, nargs="*", default=[140, 150, 160, 170], help="mitm: the k to search")
    ap.add_argument("--cases-file", default=None, help="recorded block audits (replay), JSON {cases: [...]}")
    ap.add_argument("--select", default=None, help="replay: comma list of k:role:t to run")
    ap.add_argument("--model", default=None, help="learned cost model (es_learned.py --save-model)")
    ap.add_argument("--json", default=None)
    ap.add_argument("--bfile", default=None)
    ap.add_argument("--log2-positions", type=int, default=40)
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--tune", type=json.loads, default=None,
                    help="k390, batch64: launch shape (JSON, es_autotune.DEFAULT keys) instead of the default")
    a = ap.parse_args()
    if a.which == "small-k":
        known = {k: g for k, (g, _) in es_gb300.load_known(a.bfile).items()} if a.bfile else None
        out = small_k(known=known)
    elif a.which == "batch64":
        out = batch64(autotune=not a.no_autotune, tune=a.tune)
    elif a.which == "k390":
        orders = None
        if a.model:   # the learned planner's cascade order for each wheel
            import es_learned
            model = es_learned.CostModel.load(a.model)
            orders = {role: es_learned.learned_order(model, es_gb300.Plan(390, None, w))[1]
                      for role, w in K390_WHEELS.items()}
        out = k390(a.log2_positions, filter_orders=orders, tune=a.tune)
    elif a.which == "mitm":
        out = mitm(a.k)
    elif a.which == "k390-learned":
        out = k390_learned(a.model, a.log2_positions, autotune=not a.no_autotune)
    else:
        cases = json.load(open(a.cases_file))["cases"]
        if a.select:
            want = set(a.select.split(","))
            cases = [c for c in cases if f"{c['k']}:{c['role']}:{c['audit']['t']}" in want]
        out = replay(cases)
    s = json.dumps(out, default=str)
    if a.json:
        with open(a.json, "w") as f:
            f.write(s + "\n")
    print(s)


if __name__ == "__main__":
    main()
