#!/usr/bin/env python3
"""Golden vectors of the meet-in-the-middle search, produced by the reference's own CPU path
(harness/mitm_fast.py, with harness/mitm_search.py's planner and harness/u128.py).

For every k of the list, harness/mitm_fast.py:mitm_g runs unchanged; the fixture keeps what it
returns (g, the final bound B, the total of candidates tested, the wheel) and, per round, the
candidates tested (as mitm_g prints them, three significant digits) and the survivors of the
residual filters with n > k + 1 -- the n that mitm_g hands to the frozen referee, recorded by
wrapping ref.is_good (mitm_fast.py:136), split into rounds at the summary line mitm_g prints
after each round.  The two halves come from mitm_search.split_wheel, swapped so that the second
is the smaller (mitm_fast.py:62-64).

Run where the reference checkout is available; its location comes from --ref or the
ES_REFERENCE_ROOT environment variable (one of them is required):

    python tests/golden/make_golden_mitm.py --ref <reference checkout>
"""
from __future__ import annotations

import argparse
import contextlib
import io
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
K_LIST = list(range(8, 131)) + [140, 150]
MEM_GB = 0.05          # small halves, so that every k above finishes in seconds on one core


class _RoundLog(io.StringIO):
    """stderr stand-in: each line mitm_g prints with the number of referee calls made so far
    (mitm_fast.py prints a round's summary after testing that round's survivors)."""

    def __init__(self, seen):
        super().__init__()
        self.seen, self.lines, self._buf = seen, [], ""

    def write(self, s):
        self._buf += s
        while "\n" in self._buf:
            line, self._buf = self._buf.split("\n", 1)
            self.lines.append((line, len(self.seen)))
        return len(s)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("ES_REFERENCE_ROOT"),
                    required="ES_REFERENCE_ROOT" not in os.environ,
                    help="reference checkout (default: $ES_REFERENCE_ROOT)")
    ap.add_argument("--out", default=os.path.join(HERE, "mitm_small_k.json"))
    a = ap.parse_args()
    sys.path.insert(0, os.path.join(a.ref, "harness"))
    sys.path.insert(0, os.path.join(a.ref, "ref"))
    import erdos_ref as ref
    import mitm_fast
    import mitm_search
    cases = []
    for k in K_LIST:
        seen = []
        real = mitm_fast.ref.is_good

        def rec(n, kk, _real=real, _seen=seen):
            _seen.append(int(n))
            return _real(n, kk)
        mitm_fast.ref.is_good = rec
        err = _RoundLog(seen)
        try:
            with contextlib.redirect_stderr(err):
                r = mitm_fast.mitm_g(k, mem_gb=MEM_GB, bound_mult=1.0, verbose=True)
        finally:
            mitm_fast.ref.is_good = real
        rounds, start = [], 0
        for line, end in err.lines:
            m = re.match(r"# B=(\S+) candidates=(\S+) survivors=(\d+)", line)
            if m:
                rounds.append({"candidates": int(float(m.group(2))), "survivors_all": int(m.group(3)),
                               "referee_tested": [str(n) for n in seen[start:end]]})
                start = end
        if r.get("status") == "MITM_OUT_OF_RANGE" or "g" not in r:
            cases.append({"k": k, "status": r.get("status", "?"), "wheel": r.get("wheel")})
            continue
        info = {p: ref.allowed_residues(k, p) for p in ref.primes_upto(k)}
        w1, w2, n1, n2 = mitm_search.split_wheel(r["wheel"], info)
        if n2 > n1:
            w1, w2, n1, n2 = w2, w1, n2, n1
        cases.append({"k": k, "status": "FOUND", "g": str(r["g"]), "wheel": r["wheel"], "w1": w1, "w2": w2,
                      "M_bits": r["M_bits"], "S1": r["S1"], "S2": r["S2"], "bound": str(int(r["bound"])),
                      "candidates_total": int(r["candidates"]), "rounds": rounds})
    out = {"source": "harness/mitm_fast.py:mitm_g of the reference (mem_gb=%g, bound_mult=1.0), "
                     "referee inputs recorded by wrapping ref.is_good" % MEM_GB,
           "generator": "tests/golden/make_golden_mitm.py", "mem_gb": MEM_GB, "bound_mult": 1.0, "cases": cases}
    with open(a.out, "w") as f:
        json.dump(out, f, indent=0)
    print(f"wrote {a.out}: {len(cases)} cases")


if __name__ == "__main__":
    main()
