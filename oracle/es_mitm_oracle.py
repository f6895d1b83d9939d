"""TEST INFRASTRUCTURE ONLY -- the CPU oracle of the meet-in-the-middle search.

Only tests/ may import this module; it is the checker of the GPU MITM kernel (es_mitm_* in the
engine library), never part of the product path.

It restates the reference's vectorised CPU path harness/mitm_fast.py (scan: :70-103, filters and
rounds: :106-147) on numpy uint64 pairs: every wheel residue n < B is s1 + s2 (mod M) for s2 in
one circular run of the sorted S2, found by two searches per s1; the candidates then pass the
residual primes in cascade order (n mod q from (hi mod q)(2^64 mod q) + lo mod q, a table
lookup).  The planner (wheel, halves, filter order) is the engine's own es_mitm.MitmPlan, which
tests/test_mitm.py pins against the reference's choices through tests/golden/mitm_small_k.json
(generated from the reference itself by tests/golden/make_golden_mitm.py).  One deliberate
difference: at B = M the reference's numpy path finds an empty run (lo == hi counts as no wrap)
while its GPU kernel (sieve/gpu_mitm.py:78-85) and this oracle take the whole circle.
"""
from __future__ import annotations

import numpy as np

MASK64 = (1 << 64) - 1


def _pair(vals):
    hi = np.array([v >> 64 for v in vals], dtype=np.uint64)
    lo = np.array([v & MASK64 for v in vals], dtype=np.uint64)
    return hi, lo


def _add_mod(ahi, alo, bhi, blo, mhi, mlo):
    """(a + b) mod m on (hi, lo) uint64 pairs, a, b < m < 2^127 (harness/u128.py:17-29)."""
    lo = alo + blo
    hi = ahi + bhi + (lo < alo).astype(np.uint64)
    ge = (hi > mhi) | ((hi == mhi) & (lo >= mlo))
    borrow = ((lo < mlo) & ge).astype(np.uint64)
    return np.where(ge, hi - mhi - borrow, hi), np.where(ge, lo - mlo, lo)


def _side(plan, half):
    """All sums of one term per prime of the half, mod M (harness/u128.py:32-52 outer sums)."""
    mhi, mlo = np.uint64(plan.M >> 64), np.uint64(plan.M & MASK64)
    hi, lo = np.zeros(1, np.uint64), np.zeros(1, np.uint64)
    for p in half:
        thi, tlo = _pair([(a * plan.basis[p]) % plan.M for a in plan.info[p][1]])
        n, m = hi.size, thi.size
        hi, lo = _add_mod(np.repeat(hi, m), np.repeat(lo, m), np.tile(thi, n), np.tile(tlo, n), mhi, mlo)
    return hi, lo


def _key(hi, lo):
    a = np.empty(hi.size, dtype=[("hi", "<u8"), ("lo", "<u8")])
    a["hi"], a["lo"] = hi, lo
    return a


class MitmOracle:
    """The halves of one MITM plan, built once; ``scan(B)`` per bound."""

    def __init__(self, plan):
        self.plan = plan
        self.h1, self.l1 = _side(plan, plan.w1)
        h2, l2 = _side(plan, plan.w2)
        self.S2 = np.sort(_key(h2, l2), order=("hi", "lo"))
        self.tabs = []
        for p in plan.rest:
            q, res = plan.info[p]
            t = np.zeros(q, dtype=bool)
            t[list(res)] = True
            self.tabs.append((np.uint64(q), np.uint64((1 << 64) % q), t))

    def scan(self, B: int) -> tuple[list[int], int]:
        """Every wheel residue n < B through the residual filters: (sorted survivors, candidates)."""
        P = self.plan
        mhi, mlo = np.uint64(P.M >> 64), np.uint64(P.M & MASK64)
        n1 = self.h1.size
        zero = np.zeros(n1, np.uint64)
        # lo = (M - s1) mod M, hi = (lo + B) mod M
        nh = np.full(n1, mhi) - self.h1 - (np.full(n1, mlo) < self.l1).astype(np.uint64)
        nl = np.full(n1, mlo) - self.l1
        lo_h, lo_l = _add_mod(nh, nl, zero, zero, mhi, mlo)
        bh, bl = _pair([B])
        hi_h, hi_l = _add_mod(lo_h, lo_l, np.full(n1, bh[0]), np.full(n1, bl[0]), mhi, mlo)
        i = np.searchsorted(self.S2, _key(lo_h, lo_l), side="left")
        j = np.searchsorted(self.S2, _key(hi_h, hi_l), side="left")
        wrap = (lo_h > hi_h) | ((lo_h == hi_h) & (lo_l > hi_l)) | ((lo_h == hi_h) & (lo_l == hi_l) & (B == P.M))
        outs_h, outs_l = [], []
        for a, b in ((i, np.where(wrap, self.S2.size, j)), (np.zeros_like(i), np.where(wrap, j, 0))):
            cnt = np.maximum(b.astype(np.int64) - a.astype(np.int64), 0)
            tot = int(cnt.sum())
            if not tot:
                continue
            start = np.concatenate(([0], np.cumsum(cnt)[:-1]))
            src = np.repeat(a, cnt) + (np.arange(tot, dtype=np.int64) - np.repeat(start, cnt))
            sel = self.S2[src]
            h, l = _add_mod(np.repeat(self.h1, cnt), np.repeat(self.l1, cnt), sel["hi"], sel["lo"], mhi, mlo)
            outs_h.append(h)
            outs_l.append(l)
        if not outs_h:
            return [], 0
        h = np.concatenate(outs_h)
        l = np.concatenate(outs_l)
        keep = np.ones(h.size, dtype=bool)
        for q, w, tab in self.tabs:
            idx = np.flatnonzero(keep)
            if not idx.size:
                break
            r = ((h[idx] % q) * w + (l[idx] % q)) % q
            keep[idx] = tab[r.astype(np.int64)]
        surv = np.flatnonzero(keep)
        return sorted((int(h[s]) << 64) | int(l[s]) for s in surv), int(h.size)


def mitm_rounds(plan, bound_mult: float = 1.0, max_rounds: int = 12):
    """The round loop of harness/mitm_fast.py:106-147: B from bound_mult * E, 4x per round, until
    a survivor with n > k + 1 passes the exact test or B reaches M.  Returns per-round
    (B, sorted survivors with n > k + 1, candidates) and the least good n (or None)."""
    from es_plan import is_admissible
    orc = MitmOracle(plan)
    B = max(int(bound_mult * plan.E), 1)
    out = []
    for _ in range(max_rounds):
        B = min(B, plan.M)
        surv, cand = orc.scan(B)
        big = [n for n in surv if n > plan.k + 1]
        out.append((B, big, cand))
        good = [n for n in big if is_admissible(n, plan.k)]
        if good:
            return out, good[0]
        if B >= plan.M:
            return out, None
        B = min(B * 4, plan.M)
    return out, None
