"""CPU: the planner restatement reproduces the reference Plan exactly (tests/golden/plans.json)."""
import hashlib
import math

import pytest

from conftest import golden


def _rec(P):
    return {"wheel": [[p, T] for p, T in P.wheel], "M": str(P.M), "R": P.R, "radix": P.radix,
            "rest": P.rest, "basis_sha": hashlib.sha256(",".join(map(str, P.basis)).encode()).hexdigest()}


def _check(P, want):
    got = _rec(P)
    for key in got:
        assert got[key] == want[key], (P.k, key)


def test_default_plans_k_1_to_400():
    import es_plan
    for r in golden("plans.json")["default"]:
        _check(es_plan.Plan(r["k"]), r)


@pytest.mark.parametrize("section", ["variants", "explicit", "target_g"])
def test_plan_variants(section):
    import es_plan
    for r in golden("plans.json")[section]:
        _check(es_plan.Plan(r["k"], r.get("tun"), r.get("wheel_arg")), r)


def test_banned_prime_wheels():
    """harness/run_k.py --ban: re-plan without the banned primes (run_k.py:208-214)."""
    import es_plan
    for r in golden("plans.json")["banned"]:
        k = r["k"]
        ps = [p for p in es_plan.primes_upto(k) if p not in r["ban"]]
        full = es_plan.Plan(k)
        w = es_plan.plan_wheel(k, ps, -math.log2(full.density_all), dict(es_plan.TUNABLES))
        _check(es_plan.Plan(k, None, [[p, T] for p, T in w]), r)


@pytest.mark.parametrize("k", [2, 3, 7, 13, 20, 33, 40])
def test_index_coverage_and_inverse(k):
    """Every index of a block maps to a distinct n in [tM, (t+1)M), and n_to_idx inverts it."""
    import es_plan
    P = es_plan.Plan(k)
    seen = set()
    for idx in range(P.R):
        n = P.idx_to_n(idx, 2)
        assert 2 * P.M <= n < 3 * P.M
        assert P.n_to_idx(n) == (2, idx)
        seen.add(n)
    assert len(seen) == P.R


def test_summary_and_surface():
    import es_gb300
    P = es_gb300.Plan(120)
    s = P.summary()
    for key in ("k", "wheel", "N_bits", "M", "n_filters", "residues_per_block", "expected_checks_true"):
        assert key in s
    assert P.R == math.prod(P.radix)
    assert P.R % P.radix[0] == 0
    # module surface used by harness/run_k.py (run_k.py:34-244)
    for name in ("Plan", "GpuSieve", "TUNABLES", "plan_wheel", "free_vram_mib", "load_known", "main",
                 "order_filters", "partial_residues", "partial_count"):
        assert hasattr(es_gb300, name), name
    # rest = every prime whose full power is not inside the wheel
    ps = es_gb300.primes_upto(120)
    assert sorted(P.rest) == [p for p in ps if P.wheelT.get(p, 0) < P.tp[p]]


def test_learned_filter_order_is_a_permutation():
    import es_plan
    P = es_plan.Plan(150)
    order = list(reversed(P.rest))
    Q = es_plan.Plan(150, None, [[p, T] for p, T in P.wheel], filter_order=order)
    assert Q.rest == order and Q.M == P.M
    with pytest.raises(AssertionError):
        es_plan.Plan(150, None, [[p, T] for p, T in P.wheel], filter_order=order[1:])


def test_recorded_block_audits_rebuild():
    """Every recorded frontier block (evidence/through400/runs.json audits): the wheel rebuilds the
    recorded M and R, and the survivor hash recipe reproduces the recorded hash from the
    recorded survivors; the whole-block GPU replays compare against exactly these records."""
    import es_gb300
    from conftest import golden
    g = golden("replay_blocks.json")
    assert len(g["cases"]) > 50
    plans = {}
    for c in g["cases"]:
        key = (c["k"], c["role"])
        if key not in plans:
            plans[key] = es_gb300.Plan(c["k"], None, c["wheel"])
        P = plans[key]
        assert str(P.M) == c["M"] and P.R == c["R"], key
        a = c["audit"]
        if a.get("survivors_n") is not None:
            assert es_gb300.survivor_hash(int(n) for n in a["survivors_n"]) == a["sha256_survivors"], key
            assert len(a["survivors_n"]) == a["kernel_survivors"]


def test_engine_replay_audits_equal_the_records():
    """The audit records this engine produced on GB300 for whole recorded blocks (committed after
    the runs) equal the reference's recorded ones field by field, and their hashes follow from
    their survivors."""
    import es_gb300
    from conftest import golden
    rec = {(c["k"], c["role"], c["audit"]["t"]): c["audit"] for c in golden("replay_blocks.json")["cases"]}
    ours = golden("replays_gb300.json")["cases"]
    assert len(ours) >= 5
    for c in ours:
        a, r = c["audit"], rec[(c["k"], c["role"], c["t"])]
        for f in ("t", "residues_enumerated", "kernel_survivors", "after_n_gt_k_plus_1",
                  "passed_ref_is_good", "survivors_n", "sha256_survivors"):
            assert a[f] == r[f], (c["k"], c["role"], c["t"], f)
        assert es_gb300.survivor_hash(int(n) for n in a["survivors_n"]) == a["sha256_survivors"]
