"""CPU: the kernel's decomposition (tests/kernel_model.py) equals the reference CPU path."""
import numpy as np
import pytest

from conftest import golden
from kernel_model import KernelModel


@pytest.mark.parametrize("F", [1, 3, 4, 8])
def test_model_small_k_blocks(F):
    import es_plan
    for case in golden("scan_small_k.json")["cases"]:
        if case["k"] > 70:
            continue
        plan = es_plan.Plan(case["k"])
        model = KernelModel(plan, F)
        for blk in case["blocks"]:
            r0 = plan.radix[0] if plan.radix else 1
            s, c = model.scan(blk["t"], range(plan.R // r0))
            assert s == blk["survivors"] and c == blk["counts"], (case["k"], blk["t"])


@pytest.mark.parametrize("k,wheel", [(300, None), (390, "primary"), (390, "confirmation"), (200, None)])
def test_model_vs_c_oracle_large_k(k, wheel):
    import es_oracle as O
    import es_plan
    w = None
    if wheel:
        w = golden("scan_k390_sample.json")["wheels"][wheel]["wheel"]
    plan = es_plan.Plan(k, None, w)
    model = KernelModel(plan, 4)
    rng = np.random.default_rng(20260822)
    outer = sorted(int(x) for x in rng.integers(0, plan.R // plan.radix[0], size=300))
    for t in (0, 3):
        s, c = model.scan(t, outer)
        ws, wc, _ = O.scan_c(plan, t, outer=np.array(outer, dtype=np.uint64), threads=2)
        assert s == ws and c == wc


def test_incremental_identity():
    """n mod q = (BQ + T0Q + c*corr) mod q with the sum below 3q (tests/test_incremental_filter.py)."""
    import random
    import es_plan
    random.seed(20260822)
    total = 0
    for k in (30, 60, 100, 200, 280, 377, 378):
        P = es_plan.Plan(k)
        terms = P.terms()
        inner = terms[0]
        for _ in range(40):
            b = 0
            for j in range(1, len(P.rings)):
                b = (b + terms[j][random.randrange(P.radix[j])]) % P.M
            t = random.randrange(0, 5)
            for d0 in random.sample(range(P.radix[0]), min(P.radix[0], 6)):
                s = b + inner[d0]
                c = 1 if s >= P.M else 0
                n = t * P.M + s - c * P.M
                for p in P.rest[:4]:
                    q = P.info[p][0]
                    BQ = (b % q + (t * P.M) % q) % q
                    m = BQ + inner[d0] % q + ((q - P.M % q) % q if c else 0)
                    assert m < 3 * q
                    assert m % q == n % q
                    total += 1
    assert total > 1000


def test_unit_mapping_covers_every_cycle_once():
    """The warp-unit decode (lanes on consecutive ring-2 rows, balanced digit windows) covers
    every ring-1 cycle of a range exactly once, for ranges that start and end inside a ring-2
    row, strips narrower and wider than ring 2, and plans without a ring 2; all lanes of a warp
    share the ring-2 digit at every step."""
    from kernel_model import unit_cycles, units_of
    rng = np.random.default_rng(5)
    for r2 in (1, 2, 13, 21, 32):
        for strip in (1, 2, 3, 4, 7, 8, 16, 64):
            for _ in range(6):
                cb = int(rng.integers(0, 5000))
                ce = cb + int(rng.integers(0, 3000))
                seen = []
                for u in range(units_of(cb, ce, r2, strip)):
                    lanes = [unit_cycles(u, lane, cb, ce, r2, strip) for lane in range(32)]
                    seen += [e for cyc in lanes for e in cyc]
                    if r2 > 1:   # every lane's digits lie in the unit's one window
                        J = -(-r2 // strip)
                        bounds = [(j * r2 // J, (j + 1) * r2 // J) for j in range(J)]
                        digits = {e % r2 for cyc in lanes for e in cyc}
                        windows = {j for j, (lo, hi) in enumerate(bounds) for d in digits if lo <= d < hi}
                        assert len(windows) <= 1, (r2, strip, u)
                        assert max(hi - lo for lo, hi in bounds) <= strip
                assert sorted(seen) == list(range(cb, ce)), (r2, strip, cb, ce)


def test_paired_digit_entries_round_trip():
    """A one-word ring's entry for digits d1, d1 + 1 gives back each candidate's digit, slot,
    carry split and ring-1 wrap."""
    from kernel_model import pair_candidate, pair_entry
    rng = np.random.default_rng(9)
    for _ in range(2000):
        d1 = 2 * int(rng.integers(0, 30000))
        sl, sh = int(rng.integers(0, 33)), int(rng.integers(0, 33))
        wl, wh = bool(rng.integers(0, 2)), bool(rng.integers(0, 2))
        lane = int(rng.integers(0, 32))
        z, w = pair_entry(d1, sl, wl, sh, wh, lane)
        for i in (0, 31, 32, 63, int(rng.integers(0, 64))):
            got = pair_candidate(z, w, i)
            want = (d1 + (i >> 5), i & 31, sh if i >= 32 else sl, wh if i >= 32 else wl, lane)
            assert got == want
