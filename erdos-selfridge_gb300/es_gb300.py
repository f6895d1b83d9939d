#!/usr/bin/env python3
"""GB300 (sm_103a) engine for the Erdős–Selfridge CRT-wheel sieve: a drop-in for the engine
module that harness/run_k.py, harness/run_k_masks.py and harness/replay_release.py drive.

Usage from the reference harness (no code change there):

    PYTHONPATH=<this directory> ES_ENGINE=es_gb300 python harness/run_k.py 300 --max-blocks 1

Module surface (sieve/gpu_sieve_v9.py): ``Plan``, ``GpuSieve``, ``TUNABLES``, ``plan_wheel``,
``order_filters``, ``partial_residues``, ``partial_count``, ``free_vram_mib``, ``load_known``
and ``main`` (same CLI and JSON line).  ``GpuSieve`` keeps every attribute the drivers touch
(harness/run_k.py:85-124): ``rest_q``, ``rest_Mmodq``, ``tconst_h``, ``tconst.set``, ``r0``,
``R_outer``, ``ochunk``, ``chunk``, ``out_n.fill/get``, ``out[:n].get()``, ``out_cap``,
``residues_checked``, ``launches``, ``_launch(ostart, ocount)``, ``scan_block(t)``,
``search(max_blocks, log)`` and ``mask_mode``.

Compute runs only in libes_gb300.so (hand-written CUDA for sm_103a) through ctypes; there is no
CPU fallback.  The host re-verifies every survivor of the concluding block with an exact
Kummer test, as the reference does with its frozen referee (sieve/gpu_sieve_v9.py:551-557).
"""
from __future__ import annotations

import argparse
import hashlib
import json
import math
import os
import re
import signal
import subprocess
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)

import es_native as N  # noqa: E402
from es_plan import (MAX_M_BITS, is_admissible, order_filters, partial_count,  # noqa: E402,F401
                     partial_residues, plan_wheel, primes_upto)
from es_plan import Plan as _PlanBase  # noqa: E402
from es_plan import TUNABLES as _PLAN_TUNABLES  # noqa: E402

# Engine tunables on top of the planner's (sieve/gpu_sieve_v9.py:98-120).  Launch shape and
# table layout never change which candidates pass.
TUNABLES = dict(_PLAN_TUNABLES)
TUNABLES.update({
    "chunk_log2": 34,        # positions per _launch chunk issued by scan_block
    "layout": "auto",        # "auto" (by table bytes) | "wordmask" | "pair" | "smem" | "scalar"
    "threads": 512,          # CTA size
    "strip": 8,              # at most this many ring-1 cycles per lane per warp-unit
    "smem_kb": 0,            # accepted, no effect (phase tables are read through L1)
    "ctas_per_sm": 4,
    "count_stages": 0,       # per-filter-stage pass counts (es_stage_counts needs 1)
    "search_batch_log2": 34, # positions per multi-block search launch
})


SEARCH_MAX_BLOCKS = 1024   # block items per multi-block search launch


class Plan(_PlanBase):
    """The reference Plan (sieve/gpu_sieve_v9.py:344-413) with this engine's TUNABLES defaults."""

    def __init__(self, k: int, tun: dict | None = None, wheel=None, filter_order=None):
        super().__init__(k, dict(TUNABLES, **(tun or {})), wheel, filter_order)


def _tune_from(tun: dict, plan=None) -> N.Tune:
    layout = tun.get("layout", "auto")
    F = max(1, min(N.MAX_MASK_FILTERS, int(tun.get("fast_filters", 4))))
    if layout == "auto":
        code = N.layout_for_plan(plan, F) if plan is not None else N.LAYOUT_WORDMASK
    else:
        code = {"scalar": N.LAYOUT_SCALAR, "pair": N.LAYOUT_PAIR, "smem": N.LAYOUT_SMEM,
                "smem-pair": N.LAYOUT_SMEM_PAIR}.get(layout, N.LAYOUT_WORDMASK)
    return N.make_tune(layout=code, mask_filters=F,
                       threads=int(tun.get("threads", 512)), strip=int(tun.get("strip", 8)),
                       smem_kb=int(tun.get("smem_kb", 0)), ctas_per_sm=int(tun.get("ctas_per_sm", 4)),
                       count_stages=int(tun.get("count_stages", 0)))


def block_from_tconst(rest_q, rest_Mmodq, tc) -> int:
    """Recover the block t from its constants tconst_j = (t*M) mod q_j (harness/run_k.py:102-104).

    The reference drivers upload only tconst; the engine also wants t (for the survivor records
    and the good/n > k+1 test).  t mod q_j is known wherever M is invertible mod q_j, and CRT
    over pairwise-coprime such q_j gives t modulo their product: exact for every block index
    below that product (> 2^64 for any plan with a few non-wheel primes)."""
    t_mod, mod = 0, 1
    for j, q in enumerate(rest_q):
        m = rest_Mmodq[j]
        if math.gcd(m, q) != 1 or math.gcd(mod, q) != 1:
            continue
        r = (int(tc[j]) * pow(m, -1, q)) % q
        k = ((r - t_mod) * pow(mod, -1, q)) % q
        t_mod += mod * k
        mod *= q
        if mod > (1 << 64):
            break
    return t_mod


def verdict(plan, t: int, surv) -> tuple[list[int], list[int], list[int]]:
    """Host re-verification of a block's kernel survivors (sieve/gpu_sieve_v9.py:551-557):
    (all survivors as n, sorted; the good ones; those with n > k+1 that the exact test rejects)."""
    cands = sorted(plan.idx_to_n(int(i), t) for i in surv)
    good = [n for n in cands if is_admissible(n, plan.k)]
    gs = set(good)
    bad = [n for n in cands if n > plan.k + 1 and n not in gs]
    return cands, good, bad


def survivor_hash(ns) -> str:
    """A block's survivor hash, reproducible by a third party (harness/run_k.py:38-44): sha256 of
    the UTF-8 bytes of the sorted decimal n joined by newlines, no trailing newline."""
    return hashlib.sha256("\n".join(str(int(n)) for n in sorted(ns)).encode()).hexdigest()


def block_audit(plan, t: int, surv) -> dict:
    """The per-block audit record the reference driver keeps (harness/run_k.py:145-158), from a
    block's kernel survivors (position indices): counts before and after n > k + 1 and the exact
    test, the survivors when there are few, and their hash."""
    cands, good, _ = verdict(plan, t, surv)
    return {"t": int(t), "residues_enumerated": plan.R, "kernel_survivors": len(cands),
            "after_n_gt_k_plus_1": sum(1 for n in cands if n > plan.k + 1),
            "passed_ref_is_good": len(good),
            "survivors_n": [str(n) for n in cands] if len(cands) <= 64 else None,
            "sha256_survivors": survivor_hash(cands)}


class _Tconst:
    """Stand-in for the CuPy tconst array: ``.set(host_array)`` uploads block constants."""

    def __init__(self, sieve: "GpuSieve"):
        self._s = sieve

    def set(self, arr) -> None:
        self._s._set_tconst(np.asarray(arr, dtype=np.uint32))


class _OutN:
    """Stand-in for the CuPy survivor counter: ``fill(0)`` resets, ``get()[0]`` syncs + reads."""

    def __init__(self, sieve: "GpuSieve"):
        self._s = sieve

    def fill(self, v) -> None:
        if int(v) != 0:
            raise ValueError("only fill(0) is supported")
        self._s.ctx.reset()

    def get(self) -> np.ndarray:
        return np.array([self._s.ctx.count()], dtype=np.uint64)


class _OutSlice:
    def __init__(self, sieve: "GpuSieve", sl: slice):
        self._s, self._sl = sieve, sl

    def get(self) -> np.ndarray:
        stop = self._sl.stop
        if stop is not None and self._sl.start in (None, 0) and self._sl.step in (None, 1) and stop >= 0:
            return self._s.ctx.survivors(int(stop))   # out[:n] with n from out_n.get()
        return self._s.ctx.survivors()[self._sl]


class _Out:
    """Stand-in for the CuPy survivor buffer: ``out[:n].get()`` returns block-relative indices."""

    def __init__(self, sieve: "GpuSieve"):
        self._s = sieve

    def __getitem__(self, sl) -> _OutSlice:
        if not isinstance(sl, slice):
            raise TypeError("index the survivor buffer with a slice")
        return _OutSlice(self._s, sl)


class GpuSieve:
    """One plan resident on the GPU with the reference GpuSieve surface (sieve/gpu_sieve_v9.py:425-568)."""

    def __init__(self, plan: Plan, tune: N.Tune | None = None):
        self.plan = plan
        P = plan
        self.w = len(P.wheel)
        self.rest_q = [P.info[p][0] for p in P.rest]
        self.rest_Mmodq = [P.M % q for q in self.rest_q]
        self.nrest = len(P.rest)
        self.tconst_h = np.zeros(max(1, self.nrest), dtype=np.uint32)
        self.r0 = P.radix[0] if P.radix else 1
        self.n_fast = max(0, min(int(P.tun.get("fast_filters", 4)), self.nrest))
        self.tune = tune if tune is not None else _tune_from(P.tun, P)
        t0 = time.time()
        self.ctx = N.Context(P, self.tune, capacity=int(P.tun["max_survivors"]))
        self.compile_s = time.time() - t0          # table build + upload (no run-time compile)
        self.out_cap = int(P.tun["max_survivors"])
        self.threads = int(self.tune.threads)
        self.chunk = 1 << int(P.tun.get("chunk_log2", 34))
        self.R_outer = P.R // self.r0
        assert self.R_outer == self.ctx.n_outer
        self.ochunk = max(1, self.chunk // self.r0)
        self.launches = 0
        self.residues_checked = 0
        self.mask_mode = {N.LAYOUT_SCALAR: "scalar-gb300", N.LAYOUT_PAIR: "pair-gb300",
                          N.LAYOUT_SMEM: "smem-gb300", N.LAYOUT_SMEM_PAIR: "smem-pair-gb300",
                          N.LAYOUT_AUTO: "auto-gb300"}.get(
            self.tune.layout, "wordmask-gb300")
        self.tconst = _Tconst(self)
        self.out_n = _OutN(self)
        self.out = _Out(self)
        self._block = 0
        self._set_tconst(self.tconst_h)

    # ---------------------------------------------------------------- device plumbing
    def _block_from_tconst(self, tc: np.ndarray) -> int:
        return block_from_tconst(self.rest_q, self.rest_Mmodq, tc)

    def _set_tconst(self, tc: np.ndarray) -> None:
        tc = np.ascontiguousarray(tc[:max(self.nrest, 1)], dtype=np.uint32)
        t = self._block if np.array_equal(tc[:self.nrest], N.tconst_for(self.plan, self._block)[:self.nrest]) \
            else self._block_from_tconst(tc)
        self.ctx.set_block(t, tc[:self.nrest] if self.nrest else np.zeros(0, dtype=np.uint32))

    def _launch(self, ostart: int, ocount: int) -> None:
        """ostart/ocount are OUTER indices; each covers r0 positions (asynchronous)."""
        self.ctx.launch(int(ostart), int(ocount))
        self.launches += 1

    # ---------------------------------------------------------------- block scans
    def scan_block(self, t: int) -> list[int]:
        """Every position of block t; one device sync per block (sieve/gpu_sieve_v9.py:508-525)."""
        self._block = int(t)
        self.tconst_h[:] = N.tconst_for(self.plan, t)[:self.tconst_h.size]
        self.tconst.set(self.tconst_h)
        self.out_n.fill(0)
        ostart = 0
        while ostart < self.R_outer:
            ocount = min(self.ochunk, self.R_outer - ostart)
            self._launch(ostart, ocount)
            self.residues_checked += ocount * self.r0
            ostart += ocount
        n = int(self.out_n.get()[0])
        if n > self.out_cap:
            return self._scan_block_chunked(t)
        return [int(x) for x in self.out[:n].get()] if n else []

    def _scan_block_chunked(self, t: int) -> list[int]:
        """Per-launch drain, used only when a block overflows the survivor buffer."""
        survivors = []
        ostart = 0
        while ostart < self.R_outer:
            ocount = min(self.ochunk, self.R_outer - ostart)
            self.out_n.fill(0)
            self._launch(ostart, ocount)
            n = int(self.out_n.get()[0])
            if n > self.out_cap:
                raise RuntimeError(f"survivor buffer overflow ({n} > {self.out_cap}); raise max_survivors")
            if n:
                survivors.extend(int(x) for x in self.out[:n].get())
            ostart += ocount
        return survivors

    def _verdict(self, t: int, surv: list[int]):
        return verdict(self.plan, t, surv)

    def search(self, max_blocks: int | None = None, log=None) -> dict:
        """Blocks t = 0, 1, ... until the first block holding a good survivor.

        Blocks are issued to the device several at a time as one block-ordered group: once a
        good survivor is found in block t the kernel skips the group's later blocks, and the
        device min-reduction names the block; every block up to it is scanned in full.  The
        host then re-reads that block's survivors and re-verifies all of them."""
        P = self.plan
        t0 = time.time()
        t = 0
        # blocks per launch: grows geometrically (most searches end in the first few blocks),
        # bounded by a position budget and by SEARCH_MAX_BLOCKS items per launch
        cap = max(1, min(SEARCH_MAX_BLOCKS, (1 << int(P.tun.get("search_batch_log2", 34))) // max(P.R, 1)))
        per = 1
        while max_blocks is None or t < max_blocks:
            nb = per if max_blocks is None else max(1, min(per, max_blocks - t))
            per = min(cap, per * 4)
            if nb == 1:
                surv = self.scan_block(t)
                found_t = t
            else:
                try:
                    found = self._scan_blocks(t, nb)
                except N.EsError as e:
                    if e.code != N.ES_ERR_OVERFLOW:
                        raise
                    # more survivors than one buffer holds: the stored records may miss the
                    # least good one, so these blocks (and the rest of the search) run one block
                    # at a time through scan_block, whose chunked fallback drains every launch
                    cap = per = 1
                    continue
                if found is None:
                    self.residues_checked += nb * P.R
                    t += nb
                    continue
                found_t = found
                self.residues_checked += (found_t - t) * P.R
                surv = self.scan_block(found_t)
            cands, good, bad = self._verdict(found_t, surv)
            if bad:
                return {"k": P.k, "status": "DISAGREEMENT", "kernel_survivors": cands[:20],
                        "ref_rejected": bad[:20], "block": found_t, "wall": time.time() - t0}
            if log and (good or time.time() - getattr(self, "_last_log", 0) > 10):
                self._last_log = time.time()
                log(f"k={P.k} block t={found_t} survivors={len(surv)} good={len(good)} "
                    f"checked={self.residues_checked:.3e} wall={time.time()-t0:.1f}s")
            if good:
                return {"k": P.k, "status": "FOUND", "g": good[0], "block": found_t,
                        "survivors_in_block": len(surv), "residues_checked": self.residues_checked,
                        "launches": self.launches, "wall": time.time() - t0}
            t = found_t + 1
        return {"k": P.k, "status": "EXHAUSTED_BLOCKS", "blocks": t,
                "residues_checked": self.residues_checked, "wall": time.time() - t0}

    def _scan_blocks(self, t: int, nb: int) -> int | None:
        """One persistent launch over blocks [t, t+nb) as a block-ordered group; returns the
        first block with a good survivor (device min-reduction) or None."""
        items = [(0, 0, t + i, 0, self.R_outer) for i in range(nb)]
        batch = N.Batch([self.ctx], items, self.tune)
        try:
            batch.run(use_graph=False)
            self.launches += 1
            m = batch.group_min(0)
        finally:
            batch.close()
        return None if m is None else int(m[0])


def free_vram_mib() -> int | None:
    try:
        o = subprocess.run(["nvidia-smi", "--query-gpu=memory.free", "--format=csv,noheader,nounits"],
                           capture_output=True, text=True, timeout=10).stdout.strip().splitlines()[0]
        return int(o)
    except Exception:
        return None


_KNOWN_LINE = re.compile(r"\s*(\d+)\s+(\d+)(?:\s|$)")


def load_known(*paths: str) -> dict[int, tuple[int, str]]:
    """Known terms for the CLI's b-file check: k -> (g(k), file name), read from text files of
    'k g' lines (other lines ignored).  A k listed in several files keeps the first file's value,
    and missing or empty paths are skipped -- the contract of sieve/gpu_sieve_v9.py:571-581."""
    terms: dict[int, tuple[int, str]] = {}
    for path in filter(None, paths):
        if not os.path.isfile(path):
            continue
        label = os.path.basename(path)
        with open(path) as fh:
            for m in filter(None, map(_KNOWN_LINE.match, fh)):
                k, g = int(m.group(1)), int(m.group(2))
                if k not in terms:
                    terms[k] = (g, label)
    return terms


# The engine CLI: the flags, exit code 124 on --timeout and the one JSON line per k that
# harness/replay_release.py:21-27 and the operators' scripts rely on (sieve/gpu_sieve_v9.py:584-618).
_CLI_FLAGS = (
    ("--plan-only", dict(action="store_true", help="print each plan's summary and stop")),
    ("--tune", dict(type=json.loads, default=None, help="JSON dict overriding TUNABLES")),
    ("--wheel", dict(type=json.loads, default=None,
                     help="explicit wheel: JSON list of [p,T] (or bare p = full power)")),
    ("--max-blocks", dict(type=int, default=None, help="stop after this many blocks")),
    ("--timeout", dict(type=float, default=None, help="seconds; process exits 124 on expiry")),
    ("--min-free-mib", dict(type=int, default=2048, help="skip a k when the GPU has less free memory")),
    ("--bfile", dict(default=os.path.join(HERE, "..", "data", "b003458.txt"), help="known terms (k g)")),
    ("--known", dict(default=os.path.join(HERE, "..", "data", "known_extra.txt"),
                     help="further known terms (k g), after the b-file")),
)


def _cli_parser() -> argparse.ArgumentParser:
    ap = argparse.ArgumentParser(description="g(k) by the CRT-wheel sieve on one GB300")
    ap.add_argument("k", type=int, nargs="+")
    for flag, kw in _CLI_FLAGS:
        ap.add_argument(flag, **kw)
    return ap


def _exit_on_timeout(seconds: float) -> None:
    """After `seconds` of wall time: one {"status": "TIMEOUT"} line, then exit status 124."""
    def expire(_sig, _frame):
        sys.stdout.write(json.dumps({"status": "TIMEOUT"}) + "\n")
        sys.stdout.flush()
        os._exit(124)
    signal.signal(signal.SIGALRM, expire)
    signal.setitimer(signal.ITIMER_REAL, seconds)


def _cli_result(k: int, args, known: dict) -> dict:
    """The JSON record of one k: the plan summary alone (--plan-only), a skip when the GPU lacks
    memory, or the search result with the b-file comparison and the plan summary appended."""
    plan = Plan(k, args.tune, args.wheel)
    if args.plan_only:
        return plan.summary()
    free = free_vram_mib()
    if free is not None and free < args.min_free_mib:
        return {"k": k, "status": "SKIPPED_LOW_VRAM", "free_mib": free}
    res = GpuSieve(plan).search(args.max_blocks, log=lambda msg: print(msg, file=sys.stderr, flush=True))
    if res.get("status") == "FOUND" and k in known:
        g_known, source = known[k]
        res.update(matches_bfile=res["g"] == g_known, bfile=g_known, known_source=source)
    res["plan"] = plan.summary()
    return res


def main(argv=None):
    args = _cli_parser().parse_args(argv)
    if args.timeout:
        _exit_on_timeout(args.timeout)
    known = load_known(args.bfile, args.known)
    for k in args.k:
        print(json.dumps(_cli_result(k, args, known), default=str), flush=True)


if __name__ == "__main__":
    main()
