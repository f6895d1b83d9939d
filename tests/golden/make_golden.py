#!/usr/bin/env python3
"""Generate the golden fixtures in tests/golden from the reference project's own code.

Run where the reference checkout is available; its location comes from --ref or the
ES_REFERENCE_ROOT environment variable (one of them is required):

    python tests/golden/make_golden.py --ref <reference checkout> [--jobs 8]

Everything written here comes from the reference's CPU path, never from this repository:

* ``bfile.json``          -- data/b003458_1to400.txt and data/known_extra.txt (k -> g(k)).
* ``plans.json``          -- sieve/gpu_sieve_v9.py ``Plan(k)`` for k = 1..400 (ring order, M, R,
                             radix, filter order), plus tunable variants, sieve/gpu_sieve_v11.py
                             ``target_g`` plans and harness/plan_sweep.py ``banned_wheel`` plans.
* ``scan_small_k.json``   -- k = 2..120: every block t = 0, 1, ... up to the first block with a
                             good survivor, scanned exhaustively with ``Plan.idx_to_n`` +
                             ``erdos_ref.dominates`` over ``plan.rest`` (the emulation in
                             tests/test_enumeration.py:51-68).  Per block: sorted survivor indices
                             and per-stage pass counts in cascade order.
* ``scan_k300_sample.json`` -- k = 300, block 0: 2^19 outer indices drawn with
                             numpy.random.default_rng(0) from [0, 2^34 / r0) (deduplicated, sorted)
                             x the full inner ring; survivors + per-stage pass counts.
* ``scan_k390_sample.json`` -- k = 390 primary and confirmation wheels from
                             evidence/through400/runs.json; the same kind of 2^24-position sample
                             of [0, 2^40) for each wheel, plus the recorded block-0 survivors.
* ``scan_batch64.json``   -- the 64 seeded batch instances (k in 150..400, log-uniform lengths):
                             each instance's k, length and the reference scan of its first
                             min(n_outer, 4096) outer indices.

Pass counts: counts[j] = number of scanned positions whose n passes filters 0..j of ``plan.rest``
(order-dependent by construction); survivors pass all filters (n <= k+1 included, as the kernel
emits them; the host drops them).
"""
from __future__ import annotations

import argparse
import hashlib
import json
import math
import multiprocessing as mp
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

_REF = None
_ES = None


def _setup(ref_root: str) -> None:
    global _REF, _ES
    sys.path.insert(0, os.path.join(ref_root, "sieve"))
    sys.path.insert(0, os.path.join(ref_root, "ref"))
    sys.path.insert(0, os.path.join(ref_root, "harness"))
    import erdos_ref  # noqa: E402
    import gpu_sieve_v9  # noqa: E402
    _REF, _ES = erdos_ref, gpu_sieve_v9


def plan_record(P) -> dict:
    return {"k": P.k, "wheel": [[p, T] for p, T in P.wheel], "M": str(P.M), "R": P.R,
            "radix": P.radix, "rest": P.rest,
            "basis_sha": hashlib.sha256(",".join(map(str, P.basis)).encode()).hexdigest()}


def _plan_job(args):
    ref_root, k, tun, wheel = args
    _setup(ref_root)
    P = _ES.Plan(k, tun, wheel)
    rec = plan_record(P)
    rec["tun"] = tun
    rec["wheel_arg"] = wheel
    return rec


def _banned_job(args):
    ref_root, k, ban = args
    _setup(ref_root)
    # harness/run_k.py:208-214 with ES_ENGINE=gpu_sieve_v9: re-plan without the banned primes
    ps = [p for p in _REF.primes_upto(k) if p not in ban]
    full = _ES.Plan(k, None)
    log2E = -math.log2(full.density_all)
    w = _ES.plan_wheel(k, ps, log2E, dict(_ES.TUNABLES))
    P = _ES.Plan(k, None, [[p, T] for p, T in w])
    rec = plan_record(P)
    rec["ban"] = ban
    return rec


def scan_outer(P, t: int, outer) -> tuple[list[int], list[int]]:
    """Reference CPU path over outer indices x the full inner ring (positions oidx*r0 + d0)."""
    k = P.k
    r0 = P.radix[0] if P.radix else 1
    nf = len(P.rest)
    counts = [0] * nf
    surv = []
    for o in outer:
        for d0 in range(r0):
            idx = int(o) * r0 + d0
            n = P.idx_to_n(idx, t)
            j = 0
            while j < nf and _REF.dominates(n, k, P.rest[j]):
                counts[j] += 1
                j += 1
            if j == nf:
                surv.append(idx)
    return surv, counts


def _scan_job(args):
    ref_root, k, tun, wheel, t, outer = args
    _setup(ref_root)
    P = _ES.Plan(k, tun, wheel)
    return scan_outer(P, t, outer)


def parallel_scan(pool, ref_root, k, tun, wheel, t, outer, jobs):
    outer = [int(x) for x in outer]
    step = max(1, (len(outer) + 4 * jobs - 1) // (4 * jobs))
    parts = [outer[i:i + step] for i in range(0, len(outer), step)]
    res = pool.map(_scan_job, [(ref_root, k, tun, wheel, t, p) for p in parts])
    surv, counts = [], None
    for s, c in res:
        surv.extend(s)
        counts = c if counts is None else [a + b for a, b in zip(counts, c)]
    return sorted(surv), counts or []


def _small_k_job(args):
    ref_root, k = args
    _setup(ref_root)
    P = _ES.Plan(k)
    r0 = P.radix[0] if P.radix else 1
    R_outer = P.R // r0
    blocks = []
    t = 0
    while True:
        surv, counts = scan_outer(P, t, range(R_outer))
        good = sorted(n for n in (P.idx_to_n(i, t) for i in surv) if n > k + 1)
        blocks.append({"t": t, "survivors": surv, "counts": counts})
        if good:
            return {"k": k, "g": good[0], "blocks": blocks, "plan": plan_record(P)}
        t += 1


def outer_sample(seed: int, domain: int, size: int) -> np.ndarray:
    """Seeded sample of outer indices: unique, sorted (same recipe on every machine)."""
    rng = np.random.default_rng(seed)
    return np.unique(rng.integers(0, domain, size=size, dtype=np.uint64))


def _sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<u8").tobytes()).hexdigest()


def batch_instances(seed: int = 0, count: int = 64):
    rng = np.random.default_rng(seed)
    ks = rng.integers(150, 401, size=count)
    L = np.floor(2.0 ** rng.uniform(20, 32, size=count)).astype(np.int64)
    return [int(x) for x in ks], [int(x) for x in L]


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("ES_REFERENCE_ROOT"),
                    required="ES_REFERENCE_ROOT" not in os.environ,
                    help="reference checkout (default: $ES_REFERENCE_ROOT)")
    ap.add_argument("--jobs", type=int, default=os.cpu_count() or 4)
    ap.add_argument("--only", default="", help="comma list of fixtures to (re)build")
    a = ap.parse_args()
    ref_root = a.ref
    _setup(ref_root)
    only = set(x for x in a.only.split(",") if x)
    want = (lambda name: not only or name in only)
    ctx = mp.get_context("spawn")
    pool = ctx.Pool(a.jobs)
    t0 = time.time()

    if want("bfile"):
        rows = {}
        for line in open(os.path.join(ref_root, "data", "b003458_1to400.txt")):
            parts = line.split()
            if len(parts) >= 2 and parts[0].isdigit():
                rows[parts[0]] = parts[1]
        extra = {}
        for line in open(os.path.join(ref_root, "data", "known_extra.txt")):
            parts = line.split()
            if len(parts) >= 2 and parts[0].isdigit():
                extra[parts[0]] = parts[1]
        json.dump({"source": "data/b003458_1to400.txt, data/known_extra.txt",
                   "g": rows, "known_extra": extra}, open(os.path.join(HERE, "bfile.json"), "w"))
        print("bfile", len(rows), file=sys.stderr)

    if want("plans"):
        jobs = [(ref_root, k, None, None) for k in range(1, 401)]
        default = pool.map(_plan_job, jobs)
        variants_spec = []
        for k in (20, 57, 100, 150, 199, 250, 300, 333, 377, 390, 400):
            for tun in ({"planner": "knapsack"}, {"planner": "knapsack", "n_mult": 4.0},
                        {"planner": "knapsack", "n_mult": 0.25}, {"cost_scale": 128},
                        {"cost_scale": 512}, {"m_cap_bits": 100}, {"m_cap_bits": 80},
                        {"max_R_bits": 40}):
                variants_spec.append((ref_root, k, tun, None))
        variants = pool.map(_plan_job, variants_spec)
        # explicit wheels: the recorded frontier wheels (primary/confirmation) for k = 378..400
        runs = json.load(open(os.path.join(ref_root, "evidence", "through400", "runs.json")))["terms"]
        explicit = pool.map(_plan_job, [(ref_root, term["k"], None, term[role]["wheel"])
                                        for term in runs for role in ("primary", "confirmation")])
        # bare-prime (full power) wheel spelling
        explicit += pool.map(_plan_job, [(ref_root, 60, None, [2, 3, [5, 1], 7]),
                                         (ref_root, 120, None, [[2, 3], 11, 13])])
        # v11 known-g objective
        b = {int(l.split()[0]): int(l.split()[1]) for l in open(os.path.join(ref_root, "data", "b003458_1to400.txt"))}
        import gpu_sieve_v11 as v11  # noqa: E402
        tg = []
        for k in (150, 300, 390):
            P = v11.Plan(k, {"target_g": b[k]})
            rec = plan_record(P)
            rec["tun"] = {"target_g": b[k]}
            tg.append(rec)
        banned = pool.map(_banned_job, [(ref_root, k, ban) for k, ban in
                                        ((150, [2]), (300, [2, 3]), (390, [5]), (390, [2, 3]))])
        json.dump({"source": "sieve/gpu_sieve_v9.py Plan; sieve/gpu_sieve_v11.py target_g; "
                             "harness/plan_sweep.py banned_wheel",
                   "default": default, "variants": variants, "explicit": explicit,
                   "target_g": tg, "banned": banned},
                  open(os.path.join(HERE, "plans.json"), "w"))
        print("plans", time.time() - t0, file=sys.stderr)

    if want("small_k"):
        res = pool.map(_small_k_job, [(ref_root, k) for k in range(2, 121)])
        json.dump({"source": "tests/test_enumeration.py emulation (Plan.idx_to_n + erdos_ref.dominates)",
                   "cases": res}, open(os.path.join(HERE, "scan_small_k.json"), "w"))
        print("small_k", time.time() - t0, file=sys.stderr)

    if want("k300"):
        P = _ES.Plan(300)
        r0 = P.radix[0]
        outer = outer_sample(0, (1 << 34) // r0, 1 << 19)
        surv, counts = parallel_scan(pool, ref_root, 300, None, None, 0, outer, a.jobs)
        json.dump({"k": 300, "t": 0, "plan": plan_record(P), "seed": 0,
                   "domain": (1 << 34) // r0, "draws": 1 << 19, "n_outer": int(outer.size),
                   "outer_sha256": _sha(outer), "survivors": surv, "counts": counts},
                  open(os.path.join(HERE, "scan_k300_sample.json"), "w"))
        print("k300", time.time() - t0, file=sys.stderr)

    if want("k390"):
        runs = json.load(open(os.path.join(ref_root, "evidence", "through400", "runs.json")))["terms"]
        term = next(x for x in runs if x["k"] == 390)
        out = {"k": 390, "t": 0, "n": term["n"], "wheels": {}}
        for role in ("primary", "confirmation"):
            wheel = term[role]["wheel"]
            P = _ES.Plan(390, None, wheel)
            r0 = P.radix[0]
            domain = (1 << 40) // r0
            outer = outer_sample(0, domain, (1 << 24) // r0)
            surv, counts = parallel_scan(pool, ref_root, 390, None, wheel, 0, outer, a.jobs)
            audit = term[role]["block_audit"][0]
            out["wheels"][role] = {"wheel": wheel, "plan": plan_record(P), "seed": 0,
                                   "domain": domain, "draws": (1 << 24) // r0,
                                   "n_outer": int(outer.size), "outer_sha256": _sha(outer),
                                   "survivors": surv, "counts": counts,
                                   "recorded_block0_survivors_n": audit["survivors_n"],
                                   "recorded_sha256": audit["sha256_survivors"]}
        json.dump(out, open(os.path.join(HERE, "scan_k390_sample.json"), "w"))
        print("k390", time.time() - t0, file=sys.stderr)

    if want("replay"):
        # the recorded full-block audits of the frontier wheels (harness/run_k.py:145-158 fields),
        # for whole-block replays: every role/block of k = 378..400 with its R and survivor hash
        runs = json.load(open(os.path.join(ref_root, "evidence", "through400", "runs.json")))["terms"]
        cases = []
        for term in runs:
            for role in ("primary", "confirmation"):
                rec = term.get(role)
                if not rec:
                    continue
                for audit in rec.get("block_audit") or []:
                    cases.append({"k": term["k"], "role": role, "wheel": rec["wheel"],
                                  "M": rec["N"], "R": rec["residues_per_block"], "audit": audit})
        json.dump({"source": "evidence/through400/runs.json (block_audit records of harness/run_k.py)",
                   "recipe": "sha256 of the UTF-8 bytes of '\\n'.join(decimal(n) for n in sorted(survivors)), "
                             "no trailing newline", "cases": cases},
                  open(os.path.join(HERE, "replay_blocks.json"), "w"))
        print("replay", len(cases), file=sys.stderr)

    if want("batch64"):
        ks, L = batch_instances(0, 64)
        insts = []
        for k, length in zip(ks, L):
            P = _ES.Plan(k)
            r0 = P.radix[0]
            n_outer = -(-min(length, P.R) // r0)
            pre = min(n_outer, 4096)
            surv, counts = parallel_scan(pool, ref_root, k, None, None, 0, range(pre), a.jobs)
            insts.append({"k": k, "L": length, "n_outer": n_outer, "prefix_outer": pre,
                          "plan": plan_record(P), "survivors": surv, "counts": counts})
        json.dump({"seed": 0, "recipe": "rng=default_rng(0); k=integers(150,401,64); "
                   "L=floor(2**uniform(20,32,64)); n_outer=ceil(min(L,R)/r0)",
                   "instances": insts}, open(os.path.join(HERE, "scan_batch64.json"), "w"))
        print("batch64", time.time() - t0, file=sys.stderr)
    pool.close()


if __name__ == "__main__":
    main()
