#!/usr/bin/env python3
"""Meet-in-the-middle search for g(k) on one GB300: the alternative to the block sieve when the
wheel modulus M may exceed E = 1/density (the reference's sieve/gpu_mitm.py, with the
derivation in harness/mitm_search.py and a vectorised CPU path in harness/mitm_fast.py).

The wheel residues are r = s1 + s2 (mod M) with s1 from one half of the wheel primes and s2 from
the other.  Only n = r < B is wanted, and for a fixed s1 those s2 form one contiguous (circular)
run of the sorted S2.  So the engine holds the SMALLER half S2 sorted on the device, enumerates
the larger half S1 by mixed-radix decode inside the kernel, finds each s1's run through a
bucket directory over S2's top bits plus a short binary search, tests every n of the run against
the residual primes (the filter cascade of the block sieve: n mod q from 32-bit limb weights and
one Barrett step, then a bit-table test) and emits the survivors.  The bound B starts at
bound_mult * E and grows 4x per round until a good survivor appears or B reaches M.

Planner (kept step-for-step with harness/mitm_search.py:64-131, so that the same wheel, halves
and filter order come out and survivor lists can be compared bit-exactly with the reference's
CPU path): a 0/1 knapsack over the primes <= k minimising log2 R per log2 M bucket, ranked by
max(log2 R / 2, log2 E + log2 R - log2 M) among buckets with M >= 4E, the first whose greedy
balanced split fits the memory budget.

The device half runs only in libes_gb300.so (es_mitm_* in include/es_gb300.h); there is no CPU
fallback.  Every good survivor is re-verified on the host by the exact Kummer test.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import sys
import time
from math import prod

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)

import es_native as N  # noqa: E402
from es_plan import full_residues, is_admissible, primes_upto  # noqa: E402

SCALE = 64   # knapsack weight units per bit of log2 q


# ------------------------------------------------------------------ planner
def split_wheel(wheel, info):
    """Greedy balanced halves: primes by descending residue count, each to the half with the
    smaller product so far (harness/mitm_search.py:119-128).  Returns (w1, w2, |S1|, |S2|)."""
    halves = ([], [])
    sizes = [1, 1]
    for p in sorted(wheel, key=lambda p: -len(info[p][1])):
        side = 0 if sizes[0] <= sizes[1] else 1
        halves[side].append(p)
        sizes[side] *= len(info[p][1])
    return sorted(halves[0]), sorted(halves[1]), sizes[0], sizes[1]


def choose_wheel_mitm(k, info, log2E, mem_bytes, min_m_over_e=4.0):
    """Wheel primes for the MITM search (harness/mitm_search.py:64-116): the knapsack gives the
    least log2 R for every log2 M bucket; buckets below log2(4E) (where g(k) could lie above M)
    or whose R could not fit even a perfect split are dropped; the rest are ranked by the cost
    max(sqrt R, E R / M) and the first whose actual split keeps the smaller half within the
    memory budget (16 bytes per residue) wins.  None when nothing fits."""
    ps = list(info)
    weight = [max(1, round(math.log2(info[p][0]) * SCALE)) for p in ps]
    gain = [math.log2(len(info[p][1])) for p in ps]
    cap = min(4096 * SCALE, sum(weight))
    inf = float("inf")
    best = np.full(cap + 1, inf)
    best[0] = 0.0
    took = np.zeros((len(ps), cap + 1), dtype=bool)
    for i, (wi, gi) in enumerate(zip(weight, gain)):
        if wi > cap:
            continue
        # the 0/1 update over descending capacities reads only values of the previous prime, so
        # it is one vector step: take prime i at c when best[c - wi] + gain beats best[c]
        cand = best[:cap + 1 - wi] + gi
        better = cand < best[wi:]
        took[i, wi:] = better
        best[wi:] = np.where(better, cand, best[wi:])
    best = best.tolist()
    max_logR = 2 * math.log2(mem_bytes / 16)
    need_logM = min(log2E + math.log2(min_m_over_e), sum(weight) / SCALE)

    def primes_of(c):
        out = []
        for i in range(len(ps) - 1, -1, -1):
            if took[i][c]:
                out.append(ps[i])
                c -= weight[i]
        return sorted(out)

    ranked = []
    for c, logR in enumerate(best):
        if logR == inf or logR > max_logR:
            continue
        logM = c / SCALE
        if logM < need_logM:
            continue
        ranked.append((max(logR / 2.0, log2E + logR - logM), c))
    ranked.sort()
    for _, c in ranked:
        wheel = primes_of(c)
        _, _, n1, n2 = split_wheel(wheel, info)
        if min(n1, n2) <= mem_bytes / 16:
            return wheel
    return None


class MitmPlan:
    """The MITM wheel of k: the wheel primes at full power, the two halves (w2 the smaller, held
    sorted on the device), the CRT basis, the residual primes in cascade order (least pass rate
    first) and E = 1 / density of all primes <= k."""

    def __init__(self, k: int, mem_gb: float = 8.0, wheel=None):
        self.k = k
        ps = primes_upto(k)
        self.info = {p: full_residues(k, p) for p in ps}
        self.density_all = prod(len(r) / q for q, r in self.info.values()) if ps else 1.0
        self.E = 1.0 / self.density_all
        self.log2E = -math.log2(self.density_all)
        self.mem_bytes = mem_gb * 1e9
        if wheel is None:
            wheel = choose_wheel_mitm(k, self.info, self.log2E, self.mem_bytes)
        self.wheel = sorted(wheel) if wheel else None
        if not self.wheel:
            return
        self.M = prod(self.info[p][0] for p in self.wheel)
        self.basis = {}
        for p in self.wheel:
            q = self.info[p][0]
            Mi = self.M // q
            self.basis[p] = Mi * pow(Mi, -1, q)
        self.rest = sorted((p for p in ps if p not in self.wheel),
                           key=lambda p: len(self.info[p][1]) / self.info[p][0])
        w1, w2, n1, n2 = split_wheel(self.wheel, self.info)
        if n2 > n1:
            w1, w2, n1, n2 = w2, w1, n2, n1
        self.w1, self.w2, self.n1, self.n2 = w1, w2, n1, n2

    def terms(self, half) -> tuple[list[int], list[int]]:
        """(radix per prime, flat terms a * c_p mod M) of one half, in the half's prime order."""
        radix, terms = [], []
        for p in half:
            res = self.info[p][1]
            radix.append(len(res))
            terms.extend((a * self.basis[p]) % self.M for a in res)
        return radix, terms


# ------------------------------------------------------------------ device binding
class MitmDesc(C.Structure):
    _fields_ = [("k", C.c_uint32), ("n_rings1", C.c_uint32), ("n_rings2", C.c_uint32),
                ("n_filters", C.c_uint32), ("M_lo", C.c_uint64), ("M_hi", C.c_uint64),
                ("radix1", C.POINTER(C.c_uint32)), ("term1_lo", C.POINTER(C.c_uint64)),
                ("term1_hi", C.POINTER(C.c_uint64)),
                ("radix2", C.POINTER(C.c_uint32)), ("term2_lo", C.POINTER(C.c_uint64)),
                ("term2_hi", C.POINTER(C.c_uint64)),
                ("filter_q", C.POINTER(C.c_uint32)), ("allowed", C.POINTER(C.c_uint32))]


def _bind():
    L = N.lib()
    if getattr(L, "_mitm_bound", False):
        return L
    P, u64, i32 = C.c_void_p, C.c_uint64, C.c_int
    pu64 = C.POINTER(C.c_uint64)
    for name, args in (("es_mitm_create", [C.POINTER(MitmDesc), C.POINTER(P)]),
                       ("es_mitm_destroy", [P]),
                       ("es_mitm_info", [P, pu64, pu64]),
                       ("es_mitm_reset", [P]),
                       ("es_mitm_scan", [P, u64, u64, u64, u64]),
                       ("es_mitm_results", [P, pu64, pu64, u64, pu64, pu64]),
                       ("es_mitm_set_capacity", [P, u64])):
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = i32
    L._mitm_bound = True
    return L


def _u64(x):
    return np.ascontiguousarray(x, dtype=np.uint64)


def _u32(x):
    return np.ascontiguousarray(x, dtype=np.uint32)


class MitmEngine:
    """One MITM wheel on the device: the sorted small half S2 with its bucket directory, the
    large half's terms and the residual filters (es_mitm_create)."""

    def __init__(self, plan: MitmPlan, capacity: int = 1 << 20):
        L = _bind()
        mask = (1 << 64) - 1
        r1, t1 = plan.terms(plan.w1)
        r2, t2 = plan.terms(plan.w2)
        self._keep = [_u32(r1 or [0]), _u64([t & mask for t in t1] or [0]), _u64([t >> 64 for t in t1] or [0]),
                      _u32(r2 or [0]), _u64([t & mask for t in t2] or [0]), _u64([t >> 64 for t in t2] or [0]),
                      _u32([plan.info[p][0] for p in plan.rest] or [0]),
                      _u32(np.concatenate([N.bit_table(*plan.info[p]) for p in plan.rest]) if plan.rest else [0])]
        a = self._keep

        def ptr(x, t):
            return x.ctypes.data_as(C.POINTER(t))
        d = MitmDesc(k=plan.k, n_rings1=len(r1), n_rings2=len(r2), n_filters=len(plan.rest),
                     M_lo=plan.M & mask, M_hi=plan.M >> 64,
                     radix1=ptr(a[0], C.c_uint32), term1_lo=ptr(a[1], C.c_uint64), term1_hi=ptr(a[2], C.c_uint64),
                     radix2=ptr(a[3], C.c_uint32), term2_lo=ptr(a[4], C.c_uint64), term2_hi=ptr(a[5], C.c_uint64),
                     filter_q=ptr(a[6], C.c_uint32), allowed=ptr(a[7], C.c_uint32))
        h = C.c_void_p()
        N.check(L.es_mitm_create(C.byref(d), C.byref(h)))
        self.h = h
        n1, n2 = C.c_uint64(), C.c_uint64()
        N.check(L.es_mitm_info(h, C.byref(n1), C.byref(n2)))
        self.n1, self.n2 = n1.value, n2.value
        self.capacity = capacity
        N.check(L.es_mitm_set_capacity(h, capacity))

    def close(self):
        if getattr(self, "h", None):
            _bind().es_mitm_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def scan(self, B: int, s1_begin: int = 0, s1_end: int | None = None):
        """Every wheel residue n < B whose s1 index lies in [s1_begin, s1_end) through the filter
        cascade: returns (sorted survivors n, candidates tested)."""
        L = _bind()
        mask = (1 << 64) - 1
        s1_end = self.n1 if s1_end is None else s1_end
        N.check(L.es_mitm_reset(self.h))
        N.check(L.es_mitm_scan(self.h, B & mask, B >> 64, s1_begin, s1_end))
        lo = np.zeros(self.capacity, dtype=np.uint64)
        hi = np.zeros(self.capacity, dtype=np.uint64)
        ns, nc = C.c_uint64(), C.c_uint64()
        N.check(L.es_mitm_results(self.h, lo.ctypes.data_as(C.POINTER(C.c_uint64)),
                                  hi.ctypes.data_as(C.POINTER(C.c_uint64)), self.capacity,
                                  C.byref(ns), C.byref(nc)))
        m = ns.value
        return sorted((int(h) << 64) | int(l) for h, l in zip(hi[:m], lo[:m])), nc.value


# ------------------------------------------------------------------ search
def mitm_gpu(k: int, mem_gb: float = 8.0, bound_mult: float = 3.0, max_rounds: int = 8,
             capacity: int = 1 << 20, verbose: bool = False, wheel=None) -> dict:
    """g(k) by the MITM search (the surface of sieve/gpu_mitm.py:132-219): FOUND, or
    MITM_OUT_OF_RANGE when g(k) >= M (the block sieve is the fallback), NO_WHEEL_FITS_MEMORY,
    SURVIVOR_OVERFLOW or ROUND_LIMIT."""
    t0 = time.time()
    plan = MitmPlan(k, mem_gb, wheel)
    if not plan.wheel:
        return {"k": k, "status": "NO_WHEEL_FITS_MEMORY"}
    eng = MitmEngine(plan, capacity)
    try:
        B = max(int(bound_mult * plan.E), 1)
        tested = 0
        for _ in range(max_rounds):
            B = min(B, plan.M)
            t1 = time.time()
            try:
                surv, cand = eng.scan(B)
            except N.EsError as e:
                if e.code == N.ES_ERR_OVERFLOW:
                    return {"k": k, "status": "SURVIVOR_OVERFLOW", "bound": B}
                raise
            tested += cand
            good = [n for n in surv if is_admissible(n, k)]
            if verbose:
                print(f"# k={k} B={B:.3e} candidates={cand} survivors={len(surv)} good={len(good)} "
                      f"scan={time.time() - t1:.3f}s", file=sys.stderr)
            if good:
                return {"k": k, "status": "FOUND", "g": good[0], "wheel": plan.wheel,
                        "M_bits": plan.M.bit_length(), "S1": plan.n1, "S2": plan.n2, "bound": B,
                        "candidates": tested, "wall": round(time.time() - t0, 3)}
            if B >= plan.M:
                return {"k": k, "status": "MITM_OUT_OF_RANGE", "reason": "g(k) >= M; use the block sieve",
                        "M_bits": plan.M.bit_length(), "candidates": tested}
            B = min(B * 4, plan.M)
        return {"k": k, "status": "ROUND_LIMIT", "candidates": tested}
    finally:
        eng.close()


def main(argv=None):
    ap = argparse.ArgumentParser(description="g(k) by the meet-in-the-middle search on one GB300")
    ap.add_argument("k", type=int, nargs="+")
    ap.add_argument("--mem-gb", type=float, default=8.0)
    ap.add_argument("--bound-mult", type=float, default=3.0)
    ap.add_argument("--bfile", default=os.path.join(HERE, "..", "data", "b003458.txt"))
    a = ap.parse_args(argv)
    from es_gb300 import load_known
    known = load_known(a.bfile)
    for k in a.k:
        r = mitm_gpu(k, a.mem_gb, a.bound_mult, verbose=True)
        if r.get("status") == "FOUND" and k in known:
            r["bfile"] = str(known[k][0])
            r["matches_bfile"] = known[k][0] == r["g"]
        print(json.dumps(r, default=str), flush=True)


if __name__ == "__main__":
    main()
