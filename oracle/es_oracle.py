"""TEST INFRASTRUCTURE ONLY -- the CPU oracle for the Erdős–Selfridge CRT-wheel sieve.

Only tests/, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference`` legs of
bench.py may import this module; it is the checker and the timed CPU baseline, never part of
the product path (the engine in erdos-selfridge_gb300/ has no CPU fallback).

Contents (each a restatement of the reference project's own CPU code):

* the frozen referee, ref/erdos_ref.py: ``primes_upto`` (:20-28), ``digits`` (:31-37),
  ``dominates`` (:40-48), ``is_good`` (:51-55), ``g_bruteforce`` (:58-66),
  ``allowed_residues`` (:69-81), ``g_crt`` (:93-130);
* the exact binomial check of harness/verify_release.py:102-107 (``binomial_check``);
* the reference CPU path of the sieve: ``Plan.idx_to_n`` (sieve/gpu_sieve_v9.py:385-390)
  followed by the residual filters in cascade order with early exit, counting how many
  positions pass each stage (the emulation of tests/test_enumeration.py:51-68 with pass
  counts): ``scan_py`` in pure Python, ``scan_c`` in C (es_oracle.c, pthreads), and
  ``scan_mp`` (the Python path fanned out over processes -- the CPU baseline).

Parity is pinned: tests/golden holds vectors produced by the reference's own code
(tests/golden/make_golden.py) and tests/test_oracle.py checks every function here against them.
"""
from __future__ import annotations

import ctypes as C
import math
import multiprocessing as mp
import os
from itertools import product

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")


# ------------------------------------------------------------------ referee (ref/erdos_ref.py)
def primes_upto(k: int) -> list[int]:
    if k < 2:
        return []
    s = bytearray([1]) * (k + 1)
    s[0] = s[1] = 0
    for i in range(2, int(k ** 0.5) + 1):
        if s[i]:
            s[i * i::i] = bytearray(len(s[i * i::i]))
    return [i for i in range(k + 1) if s[i]]


def digits(x: int, p: int) -> list[int]:
    d = []
    while x:
        x, r = divmod(x, p)
        d.append(r)
    return d


def dominates(n: int, k: int, p: int) -> bool:
    while k:
        if k % p > n % p:
            return False
        k //= p
        n //= p
    return True


def is_good(n: int, k: int) -> bool:
    if n <= k + 1:
        return False
    return all(dominates(n, k, p) for p in primes_upto(k))


def g_bruteforce(k: int, limit: int | None = None) -> int | None:
    n = k + 2
    ps = sorted(primes_upto(k), reverse=True)
    while limit is None or n <= limit:
        if all(dominates(n, k, p) for p in ps):
            return n
        n += 1
    return None


def allowed_residues(k: int, p: int) -> tuple[int, list[int]]:
    kd = digits(k, p)
    q = p ** len(kd)
    res = []
    for combo in product(*[range(d, p) for d in kd]):
        res.append(sum(c * p ** i for i, c in enumerate(combo)))
    res.sort()
    return q, res


def g_crt(k: int, max_wheel_modulus: int = 10 ** 9) -> int:
    """Exhaustive block search with a greedy full-power wheel (ref/erdos_ref.py:93-130)."""
    ps = primes_upto(k)
    info = {p: allowed_residues(k, p) for p in ps}
    scored = sorted(ps, key=lambda p: -math.log(info[p][0] / len(info[p][1])) / math.log(info[p][0]))
    wheel, M = [], 1
    for p in scored:
        q = info[p][0]
        if M * q <= max_wheel_modulus:
            wheel.append(p)
            M *= q
    rest = sorted((p for p in ps if p not in wheel), key=lambda p: len(info[p][1]) / info[p][0])
    moduli = [info[p][0] for p in wheel]
    basis = []
    for q in moduli:
        Mi = M // q
        basis.append(Mi * pow(Mi, -1, q))
    residues = sorted(sum(a * b for a, b in zip(combo, basis)) % M
                      for combo in product(*[info[p][1] for p in wheel]))
    t = 0
    while True:
        for r in residues:
            n = t * M + r
            if n > k + 1 and all(dominates(n, k, p) for p in rest):
                return n
        t += 1


def binomial_check(n: int, k: int) -> bool:
    """C(n, k) has no prime factor <= k, by exact big-integer division."""
    c = math.comb(n, k)
    return all(c % p != 0 for p in primes_upto(k))


# ------------------------------------------------------------------ reference CPU sieve path
class PlanView:
    """The parts of a wheel plan the reference CPU path reads: rings, basis, M, filter order."""

    def __init__(self, plan):
        self.k = plan.k
        self.M = plan.M
        self.rings = [(q, list(res)) for q, res in plan.rings]
        self.radix = [len(res) for _, res in self.rings]
        self.basis = list(plan.basis)
        self.R = math.prod(self.radix)
        self.r0 = self.radix[0] if self.radix else 1
        self.rest = list(plan.rest)
        self.tables = [allowed_residues(plan.k, p) for p in self.rest]

    def idx_to_n(self, idx: int, t: int) -> int:
        r = 0
        for (q, res), rad, b in zip(self.rings, self.radix, self.basis):
            idx, d = divmod(idx, rad)
            r += res[d] * b
        return t * self.M + (r % self.M)


def scan_py(plan, t: int, outer) -> tuple[list[int], list[int]]:
    """Pure-Python reference path over outer indices x the full inner ring."""
    V = plan if isinstance(plan, PlanView) else PlanView(plan)
    counts = [0] * len(V.rest)
    surv = []
    for o in outer:
        for d0 in range(V.r0):
            idx = int(o) * V.r0 + d0
            n = V.idx_to_n(idx, t)
            j = 0
            while j < len(V.rest) and dominates(n, V.k, V.rest[j]):
                counts[j] += 1
                j += 1
            if j == len(V.rest):
                surv.append(idx)
    return sorted(surv), counts


_MP_VIEW = None


def _mp_init(view):
    global _MP_VIEW
    _MP_VIEW = view


def _mp_job(args):
    t, outer = args
    return scan_py(_MP_VIEW, t, outer)


class ScanPool:
    """The Python reference path on a persistent pool of ``procs`` spawned processes, so that
    repeated scans (timed baseline steps) do not pay for starting the processes each time."""

    def __init__(self, plan, procs: int | None = None):
        self.V = plan if isinstance(plan, PlanView) else PlanView(plan)
        self.procs = procs or os.cpu_count() or 1
        self.pool = mp.get_context("spawn").Pool(self.procs, initializer=_mp_init, initargs=(self.V,))

    def scan(self, t: int, outer) -> tuple[list[int], list[int]]:
        outer = [int(x) for x in outer]
        step = max(1, -(-len(outer) // (4 * self.procs)))
        parts = [(t, outer[i:i + step]) for i in range(0, len(outer), step)]
        res = self.pool.map(_mp_job, parts)
        surv, counts = [], [0] * len(self.V.rest)
        for s, c in res:
            surv.extend(s)
            counts = [a + b for a, b in zip(counts, c)]
        return sorted(surv), counts

    def close(self) -> None:
        self.pool.close()
        self.pool.join()


def scan_mp(plan, t: int, outer, procs: int | None = None) -> tuple[list[int], list[int]]:
    """The Python reference path fanned out over ``procs`` processes (spawn start method)."""
    sp = ScanPool(plan, procs)
    try:
        return sp.scan(t, outer)
    finally:
        sp.close()


# ------------------------------------------------------------------ C restatement
_lib = None


def build(force: bool = False) -> str:
    """Compile es_oracle.c into oracle/liboracle.so with the host gcc."""
    import subprocess
    src = os.path.join(HERE, "es_oracle.c")
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
        subprocess.run(["gcc", "-O2", "-shared", "-fPIC", "-pthread", src, "-o", LIB], check=True)
    return LIB


def _clib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        L.es_oracle_scan.restype = C.c_int
        u32p, u64p = C.POINTER(C.c_uint32), C.POINTER(C.c_uint64)
        L.es_oracle_scan.argtypes = [C.c_uint32, u32p, u64p, C.c_uint64, C.c_uint64, C.c_uint32,
                                     u32p, C.POINTER(C.c_uint8), C.c_uint64, u64p, C.c_uint64,
                                     C.c_uint64, C.c_int, u64p, u64p, C.c_uint64, u64p]
        _lib = L
    return _lib


class CTables:
    """Flat arrays of a plan for the C oracle (term_j[d] = res_j[d] * basis_j mod M)."""

    def __init__(self, plan):
        V = plan if isinstance(plan, PlanView) else PlanView(plan)
        self.view = V
        M = V.M
        lohi = []
        for (q, res), b in zip(V.rings, V.basis):
            for a in res:
                x = (a * b) % M
                lohi += [x & ((1 << 64) - 1), x >> 64]
        self.n_rings = len(V.rings)
        self.radix = np.array(V.radix or [1], dtype=np.uint32)
        self.terms = np.array(lohi or [0, 0], dtype=np.uint64)
        self.q = np.array([q for q, _ in V.tables] or [1], dtype=np.uint32)
        tabs = []
        for q, res in V.tables:
            a = np.zeros(q, dtype=np.uint8)
            a[res] = 1
            tabs.append(a)
        self.allowed = np.concatenate(tabs) if tabs else np.zeros(1, dtype=np.uint8)


def scan_c(plan, t: int, outer=None, o_range=None, threads: int | None = None,
           surv_cap: int = 1 << 22) -> tuple[list[int], list[int], int]:
    """C restatement over an outer-index list or range; returns (sorted survivors, counts, total)."""
    T = plan if isinstance(plan, CTables) else CTables(plan)
    V = T.view
    L = _clib()
    nf = len(V.rest)
    counts = np.zeros(max(nf, 1), dtype=np.uint64)
    surv = np.zeros(surv_cap, dtype=np.uint64)
    nsurv = C.c_uint64()
    u32p, u64p = C.POINTER(C.c_uint32), C.POINTER(C.c_uint64)
    if outer is not None:
        lst = np.ascontiguousarray(outer, dtype=np.uint64)
        lp, ob, oe = lst.ctypes.data_as(u64p), 0, lst.size
    else:
        lst = None
        lp, (ob, oe) = None, o_range
    rc = L.es_oracle_scan(T.n_rings, T.radix.ctypes.data_as(u32p), T.terms.ctypes.data_as(u64p),
                          V.M & ((1 << 64) - 1), V.M >> 64, nf, T.q.ctypes.data_as(u32p),
                          T.allowed.ctypes.data_as(C.POINTER(C.c_uint8)), int(t), lp, int(ob), int(oe),
                          int(threads or os.cpu_count() or 1), counts.ctypes.data_as(u64p),
                          surv.ctypes.data_as(u64p), surv_cap, C.byref(nsurv))
    if rc != 0:
        raise RuntimeError("oracle scan failed")
    n = int(nsurv.value)
    return sorted(int(x) for x in surv[:min(n, surv_cap)]), [int(x) for x in counts[:nf]], n
