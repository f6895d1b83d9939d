#!/usr/bin/env python3
"""Check this engine's whole-block replay audits with the reference's own release verifier.

For every recorded frontier run whose blocks 0..terminal were all replayed by this engine
(tests/golden/replays_gb300.json), build a run record in the reference's evidence format from
the engine's audit records and pass it to harness/verify_release.py:check_run.  That function
checks the wheel, the block coverage, the survivor hashes and counts, the admissibility of every
survivor and the terminal minimum g(k).

It imports the reference, so it runs only where the reference is checked out:

    python tests/golden/check_replays_with_reference.py --ref <reference checkout>
    (or set ES_REFERENCE_ROOT)
"""
from __future__ import annotations

import argparse
import importlib.util
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("ES_REFERENCE_ROOT"),
                    required="ES_REFERENCE_ROOT" not in os.environ,
                    help="reference checkout (default: $ES_REFERENCE_ROOT)")
    a = ap.parse_args()
    sys.path.insert(0, a.ref)
    spec = importlib.util.spec_from_file_location("verify_release", os.path.join(a.ref, "harness", "verify_release.py"))
    vr = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(vr)
    recorded = json.load(open(os.path.join(HERE, "replay_blocks.json")))["cases"]
    ours = json.load(open(os.path.join(HERE, "replays_gb300.json")))["cases"]
    runs = json.load(open(os.path.join(a.ref, "evidence", "through400", "runs.json")))["terms"]
    done = {(c["k"], c["role"], c["t"]): c["audit"] for c in ours}
    results = []
    for term in runs:
        for role in ("primary", "confirmation"):
            rec = term[role]
            blocks = list(range(rec["block"] + 1))
            if not all((term["k"], role, t) in done for t in blocks):
                continue
            run = {"wheel": rec["wheel"], "N": rec["N"], "residues_per_block": rec["residues_per_block"],
                   "block": rec["block"], "block_audit": [done[(term["k"], role, t)] for t in blocks],
                   "provenance": {"record": "es_gb300 whole-block replay"}}
            try:
                n_blocks = vr.check_run(term["k"], int(term["n"]), run)
                results.append((term["k"], role, "accepted", n_blocks))
            except ValueError as e:
                results.append((term["k"], role, f"rejected: {e}", 0))
    assert recorded, "no recorded audits"
    for r in results:
        print(*r)
    return 0 if results and all(r[2] == "accepted" for r in results) else 1


if __name__ == "__main__":
    sys.exit(main())
