"""Wheel planner for the Erdős–Selfridge CRT-wheel sieve (host side, exact integers + numpy).

g(k) is the least n > k+1 such that C(n, k) has no prime factor <= k.  By Kummer's theorem,
p does not divide C(n, k) iff every base-p digit of k is <= the matching digit of n.  The
condition for p depends only on n mod q_p, q_p = p**t_p with t_p the number of base-p digits
of k, so the admissible n form a union of residue classes.

A *wheel* is a set of items (p, T), 1 <= T <= t_p, one per prime.  Its modulus is
M = prod p**T and its admissible residues mod p**T (the T low digits dominate k's) are the
*rings*.  Every residue mod M compatible with all rings is indexed in mixed radix
(ring 0 fastest) and the residual primes (every p whose full q_p is not inside the wheel) are
checked by the device filter cascade in the order given by ``Plan.rest``.

This module keeps the semantics of the reference planner exactly, because the drop-in
engine must enumerate the same index -> n map and apply filters in the same order:

* ``partial_residues``/``partial_count``   -- sieve/gpu_sieve_v9.py:127-143
* ``plan_wheel`` (group knapsack over log2 N cells, "truecost", "knapsack" and the
  known-g "target_g" objectives, then shrink-to-fit) -- sieve/gpu_sieve_v9.py:146-227 and
  sieve/gpu_sieve_v11.py:199-213
* ``order_filters``                         -- sieve/gpu_sieve_v9.py:230-237
* ``Plan`` (ring order, CRT basis, idx_to_n, summary) -- sieve/gpu_sieve_v9.py:334-413

The floating-point steps of the knapsack (weights ``round(T*log2(p)*scale)``, the values
``log2(R_T)``, the in-place "better" update across T, the objective arrays) are performed in
the same order as the reference so that ties resolve identically; the fixtures in
tests/golden pin the chosen wheels for every k <= 400.
"""
from __future__ import annotations

import math
from math import prod

import numpy as np

MAX_M_BITS = 126          # partial CRT sums stay below 2M < 2^127
MAX_R_BITS_HARD = 62      # residues per block must index in uint64 with headroom

TUNABLES = {
    "planner": "truecost",   # "truecost" | "knapsack"
    "n_mult": 1.0,           # knapsack objective: capacity log2(n_mult * E[g])
    "cost_scale": 256,       # DP cells per bit of log2(M)
    "m_cap_bits": 120,       # hard cap on log2(M)
    "max_R_bits": 62,        # residues per block must index in uint64
    "target_g": 0,           # > 0: size the wheel to a KNOWN g (confirmation runs)
    "threads": 256,          # device CTA size (engine tunable, not used by the planner)
    "chunk_log2": 30,        # positions per drop-in launch = 2**chunk_log2
    "max_survivors": 1 << 20,
    "fast_filters": 4,       # filters evaluated as word masks in the inner ring
}


# ------------------------------------------------------------------ number theory helpers
def primes_upto(k: int) -> list[int]:
    """Primes <= k (plain sieve of Eratosthenes)."""
    if k < 2:
        return []
    flags = np.ones(k + 1, dtype=bool)
    flags[:2] = False
    for i in range(2, math.isqrt(k) + 1):
        if flags[i]:
            flags[i * i::i] = False
    return [int(x) for x in np.flatnonzero(flags)]


def base_digits(x: int, p: int) -> list[int]:
    """Base-p digits of x, least significant first; [] for x == 0."""
    out = []
    while x > 0:
        x, r = divmod(x, p)
        out.append(r)
    return out


def kummer_ok(n: int, k: int, p: int) -> bool:
    """True iff each base-p digit of k is <= the matching digit of n (p does not divide C(n,k))."""
    while k:
        if k % p > n % p:
            return False
        k //= p
        n //= p
    return True


def is_admissible(n: int, k: int) -> bool:
    """n > k+1 and C(n, k) has no prime factor <= k (exact digit test over every p <= k)."""
    return n > k + 1 and all(kummer_ok(n, k, p) for p in primes_upto(k))


def _dominating_residues(kd: list[int], p: int) -> list[int]:
    """Sorted r in [0, p**len(kd)) whose base-p digits are each >= the matching kd digit."""
    res = [0]
    place = 1
    for a in kd:
        res = [r + c * place for c in range(a, p) for r in res]
        place *= p
    res.sort()
    return res


def full_residues(k: int, p: int) -> tuple[int, list[int]]:
    """(q_p, admissible residues mod q_p) -- the full-power filter table of p."""
    kd = base_digits(k, p)
    return p ** len(kd), _dominating_residues(kd, p)


def partial_residues(k: int, p: int, T: int) -> tuple[int, list[int]]:
    """(p**T, sorted residues mod p**T whose T low digits dominate k's)."""
    kd = base_digits(k, p)
    assert 1 <= T <= len(kd)
    return p ** T, _dominating_residues(kd[:T], p)


def partial_count(k: int, p: int, T: int) -> int:
    """Number of admissible residues mod p**T, prod over the T low digits of (p - a_i)."""
    return prod(p - a for a in base_digits(k, p)[:T])


# ------------------------------------------------------------------ knapsack planner
def _knapsack(k: int, ps: list[int], scale: int, max_M_bits: int):
    """Group knapsack over integer "cells" of log2(M) (``scale`` cells per bit).

    best[c] = least log2(R) reachable with item weights summing to exactly c cells;
    pick[i][c] = exponent T chosen for ps[i] on that path (0 = not in the wheel);
    cells[i][T] = rounded weight of item (ps[i], T)."""
    top = int(max_M_bits * scale)
    best = np.full(top + 1, np.inf)
    best[0] = 0.0
    pick, cells = [], []
    for p in ps:
        n_dig = len(base_digits(k, p))
        nxt = best.copy()
        sel = np.zeros(top + 1, dtype=np.int8)
        wts: dict[int, int] = {}
        lp = math.log2(p)
        for T in range(1, n_dig + 1):
            wt = max(1, round(T * lp * scale))
            wts[T] = wt
            if wt > top:
                continue
            gain = math.log2(partial_count(k, p, T))
            trial = best[:top + 1 - wt] + gain
            upd = trial < nxt[wt:]
            nxt[wt:][upd] = trial[upd]
            sel[wt:][upd] = T
        best = nxt
        pick.append(sel)
        cells.append(wts)
    return best, pick, cells


def _walk_back(ps, pick, cells, c: int) -> list[tuple[int, int]]:
    items = []
    for i in reversed(range(len(ps))):
        T = int(pick[i][c])
        if T:
            items.append((ps[i], T))
            c -= cells[i][T]
    assert c == 0
    return sorted(items)


def _objective_cell(best: np.ndarray, scale: int, log2E: float, tun: dict) -> int:
    top = len(best) - 1
    c = np.arange(top + 1)
    ok = np.isfinite(best) & (best <= float(tun.get("max_R_bits", 62)))
    mode = tun.get("planner", "truecost")
    if mode == "knapsack":
        limit = min(top, int(math.floor((log2E + math.log2(float(tun.get("n_mult", 1.0)))) * scale)))
        ok &= c <= max(limit, 0)
        score = np.where(ok, c / scale - best, -np.inf)
        j = int(np.argmax(score))
        return j if ok[j] else 0
    if int(tun.get("target_g", 0)) > 0:
        lg_over = math.log2(int(tun["target_g"])) - c / scale          # log2(g / M)
        with np.errstate(over="ignore", invalid="ignore"):
            blocks = np.where(lg_over <= 0.0, 1.0, np.ceil(np.exp2(np.clip(lg_over, -200.0, 200.0))))
        with np.errstate(divide="ignore", invalid="ignore"):
            score = np.where(ok & np.isfinite(blocks), best + np.log2(blocks), np.inf)
    else:
        x = np.minimum(2.0 ** np.clip(c / scale - log2E, -200.0, 60.0), 1e300)
        hit = -np.expm1(-x)                       # P(block holds a survivor), H1 model
        with np.errstate(divide="ignore", invalid="ignore"):
            score = np.where(ok & (hit > 0), best - np.log2(hit), np.inf)
    j = int(np.argmin(score))
    return j if np.isfinite(score[j]) else 0


def _fits(k: int, wheel) -> bool:
    return (prod(p ** T for p, T in wheel) < (1 << MAX_M_BITS)
            and prod(partial_count(k, p, T) for p, T in wheel) < (1 << MAX_R_BITS_HARD))


def _drop_weakest_digit(k: int, wheel: list[tuple[int, int]]) -> None:
    """Remove the top digit of the item whose top digit filters least per bit of modulus."""
    def value_per_bit(item):
        p, T = item
        lower = partial_count(k, p, T - 1) if T > 1 else 1
        return (math.log2(p) - math.log2(partial_count(k, p, T) / lower)) / math.log2(p)
    item = min(wheel, key=value_per_bit)
    wheel.remove(item)
    if item[1] > 1:
        wheel.append((item[0], item[1] - 1))
        wheel.sort()


def plan_wheel(k: int, ps: list[int], log2E: float, tun: dict) -> list[tuple[int, int]]:
    """Choose the wheel items (p, T) for primes ``ps`` (same contract as the reference)."""
    if not ps:
        return []
    scale = int(tun.get("cost_scale", 256))
    cap_bits = min(int(tun.get("m_cap_bits", 120)), MAX_M_BITS)
    best, pick, cells = _knapsack(k, ps, scale, cap_bits)
    wheel = _walk_back(ps, pick, cells, _objective_cell(best, scale, log2E, tun))
    while wheel and not _fits(k, wheel):
        _drop_weakest_digit(k, wheel)
    return wheel


def order_filters(k: int, filt: list[int], info: dict, wheelT: dict[int, int]) -> list[int]:
    """Cascade order: smallest pass rate first, conditioned on the wheel's low digits."""
    def rate(p):
        q, res = info[p]
        T = wheelT.get(p, 0)
        given = partial_count(k, p, T) / p ** T if T else 1.0
        return (len(res) / q) / given
    return sorted(filt, key=rate)


def norm_wheel(wheel) -> list[tuple[int, int | None]]:
    """Accept [[p, T], ...] or bare p (full power); None marks 'full power'."""
    out = []
    for it in wheel:
        if isinstance(it, (list, tuple)):
            out.append((int(it[0]), int(it[1])))
        else:
            out.append((int(it), None))
    return out


class Plan:
    """A wheel + residual-filter plan for one k (attribute-compatible with the reference)."""

    def __init__(self, k: int, tun: dict | None = None, wheel=None, filter_order=None):
        self.k = k
        self.tun = dict(TUNABLES, **(tun or {}))
        ps = primes_upto(k)
        self.info = {p: full_residues(k, p) for p in ps}
        self.tp = {p: len(base_digits(k, p)) for p in ps}
        self.density_all = prod(len(r) / q for q, r in self.info.values()) if ps else 1.0
        log2E = -math.log2(self.density_all) if self.density_all > 0 else 0.0
        if wheel is not None:
            self.wheel = sorted((p, self.tp[p] if T is None else T) for p, T in norm_wheel(wheel))
        else:
            self.wheel = plan_wheel(k, ps, log2E, self.tun)
        for p, T in self.wheel:
            assert 1 <= T <= self.tp[p], f"bad wheel item {(p, T)}"
        assert len({p for p, _ in self.wheel}) == len(self.wheel), "prime used twice in wheel"
        self.wheelT = dict(self.wheel)
        # ring 0 (swept inside a thread) is the ring with the most residues; ties by prime
        self.wheel.sort(key=lambda it: (-partial_count(k, it[0], it[1]), it[0]))
        self.rings = [partial_residues(k, p, T) for p, T in self.wheel]
        self.moduli = [q for q, _ in self.rings]
        self.M = prod(self.moduli)
        assert self.M < (1 << MAX_M_BITS), "wheel modulus too large for 128-bit path"
        filt = [p for p in ps if self.wheelT.get(p, 0) < self.tp[p]]
        if filter_order is None:
            self.rest = order_filters(k, filt, self.info, self.wheelT)
        else:
            # an explicit cascade order (learned planner); it must be a permutation of filt
            self.rest = [int(p) for p in filter_order]
            assert sorted(self.rest) == sorted(filt), "filter order is not a permutation"
        self.basis = []
        for q in self.moduli:
            co = self.M // q
            self.basis.append(co * pow(co, -1, q))
        self.radix = [len(r) for _, r in self.rings]
        self.R = prod(self.radix)
        assert self.R < (1 << MAX_R_BITS_HARD), "too many residues per block"
        self.density_wheel = self.R / self.M if self.M else 1.0
        self.density_rest = self.density_all / self.density_wheel

    def with_order(self, order) -> "Plan":
        """A copy of this plan with another cascade order (same wheel, rings and basis)."""
        assert sorted(order) == sorted(self.rest), "filter order is not a permutation"
        q = object.__new__(type(self))
        q.__dict__.update(self.__dict__)
        q.rest = [int(p) for p in order]
        return q

    # -------------------------------------------------------------- index <-> n
    def terms(self) -> list[list[int]]:
        """Per ring j: (residue * basis_j) mod M for each residue, in ring order."""
        return [[(a * b) % self.M for a in res] for (_, res), b in zip(self.rings, self.basis)]

    def idx_to_n(self, idx: int, t: int) -> int:
        """Block-relative mixed-radix index -> n (ring 0 is the fastest digit)."""
        r = 0
        for (_, res), rad, b in zip(self.rings, self.radix, self.basis):
            idx, d = divmod(idx, rad)
            r += res[d] * b
        return t * self.M + (r % self.M)

    def n_to_idx(self, n: int) -> tuple[int, int] | None:
        """Inverse map: (block t, index) of n, or None when n mod M is not a wheel residue."""
        t, r = divmod(n, self.M)
        idx, place = 0, 1
        for (q, res), rad in zip(self.rings, self.radix):
            a = r % q
            lo, hi = 0, len(res)
            while lo < hi:                       # residues are sorted
                mid = (lo + hi) // 2
                if res[mid] < a:
                    lo = mid + 1
                else:
                    hi = mid
            if lo == len(res) or res[lo] != a:
                return None
            idx += lo * place
            place *= rad
        return t, idx

    def summary(self) -> dict:
        E = 1 / self.density_all
        return {"k": self.k, "wheel": [[p, T] for p, T in self.wheel],
                "wheel_primes": [p for p, _ in self.wheel],
                "split_primes": [[p, T, self.tp[p]] for p, T in self.wheel if T < self.tp[p]],
                "N_bits": self.M.bit_length(), "M_bits": self.M.bit_length(), "M": str(self.M),
                "N": str(self.M), "n_filters": len(self.rest),
                "residues_per_block": self.R, "density_wheel": self.density_wheel,
                "density_rest": self.density_rest, "expected_g": E, "E_g": E,
                "expected_blocks": E / self.M, "N_over_E": self.M / E,
                "expected_residue_checks": self.density_wheel / self.density_all,
                "expected_checks_true": self._true_cost()}

    def _true_cost(self) -> float:
        """R / (1 - e^{-M/E}): expected positions examined including block overshoot."""
        try:
            E = 1.0 / self.density_all
            x = self.M / E
            hit = -math.expm1(-x) if x < 40 else 1.0
            return self.R / hit
        except (ZeroDivisionError, OverflowError):
            return float("inf")

    # -------------------------------------------------------------- analytic pass rates
    def conditional_pass_rates(self) -> list[float]:
        """Per filter in cascade order: P(pass | wheel rings), the order_filters key."""
        out = []
        for p in self.rest:
            q, res = self.info[p]
            T = self.wheelT.get(p, 0)
            given = partial_count(self.k, p, T) / p ** T if T else 1.0
            out.append((len(res) / q) / given)
        return out
