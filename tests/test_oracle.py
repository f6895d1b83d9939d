"""CPU: the oracle (oracle/) against the golden vectors made from the reference's own code."""
import hashlib

import numpy as np
import pytest

from conftest import golden


def test_referee_against_bfile(bfile):
    import es_oracle as O
    for k in range(1, 61):
        assert O.g_crt(k) == bfile[k], k
    for k in range(1, 25):
        assert O.g_bruteforce(k) == bfile[k], k


def test_referee_accepts_published_terms(bfile):
    import es_oracle as O
    for k in (100, 200, 300, 390, 400):
        assert O.is_good(bfile[k], k)
        assert not O.is_good(bfile[k] - 1, k)
    for k in (10, 50, 120):
        assert O.binomial_check(bfile[k], k)
        assert O.is_good(bfile[k], k) == O.binomial_check(bfile[k], k)


def test_allowed_residues_match_planner_tables():
    import es_oracle as O
    import es_plan
    for k in (17, 100, 390):
        for p in es_plan.primes_upto(k):
            assert O.allowed_residues(k, p) == es_plan.full_residues(k, p)


def test_scan_small_k_python_and_c():
    import es_oracle as O
    import es_plan
    for case in golden("scan_small_k.json")["cases"]:
        P = es_plan.Plan(case["k"])
        r0 = P.radix[0] if P.radix else 1
        T = O.CTables(P)
        for blk in case["blocks"]:
            s, c, _ = O.scan_c(T, blk["t"], o_range=(0, P.R // r0), threads=4)
            assert s == blk["survivors"] and c == blk["counts"], (case["k"], blk["t"])
        if case["k"] <= 45:
            blk = case["blocks"][-1]
            s, c = O.scan_py(P, blk["t"], range(P.R // r0))
            assert s == blk["survivors"] and c == blk["counts"]


def _sample(g):
    outer = np.unique(np.random.default_rng(g["seed"]).integers(0, g["domain"], size=g["draws"], dtype=np.uint64))
    assert hashlib.sha256(np.ascontiguousarray(outer, dtype="<u8").tobytes()).hexdigest() == g["outer_sha256"]
    return outer


def test_scan_k300_sample_c():
    import es_oracle as O
    import es_plan
    g = golden("scan_k300_sample.json")
    s, c, _ = O.scan_c(es_plan.Plan(300), 0, outer=_sample(g))
    assert s == g["survivors"] and c == g["counts"]


@pytest.mark.parametrize("role", ["primary", "confirmation"])
def test_scan_k390_sample_c(role):
    import es_oracle as O
    import es_plan
    g = golden("scan_k390_sample.json")["wheels"][role]
    P = es_plan.Plan(390, None, g["wheel"])
    s, c, _ = O.scan_c(P, 0, outer=_sample(g))
    assert s == g["survivors"] and c == g["counts"]


def test_recorded_k390_survivors_are_admissible():
    """The block-0 survivors recorded by the reference run pass the referee (n > k+1 only)."""
    import es_oracle as O
    g = golden("scan_k390_sample.json")
    for role in ("primary", "confirmation"):
        ns = [int(x) for x in g["wheels"][role]["recorded_block0_survivors_n"]]
        assert int(g["n"]) in ns
        assert all(O.is_good(n, 390) for n in ns if n > 391)


def test_batch64_prefixes_c():
    import es_oracle as O
    import es_plan
    for inst in golden("scan_batch64.json")["instances"][:24]:
        P = es_plan.Plan(inst["k"])
        s, c, _ = O.scan_c(P, 0, o_range=(0, inst["prefix_outer"]), threads=4)
        assert s == inst["survivors"] and c == inst["counts"], inst["k"]


def test_python_and_c_paths_agree_with_a_planted_fault():
    """Both restatements agree; a table with one residue removed changes the counts (the check bites)."""
    import es_oracle as O
    import es_plan
    P = es_plan.Plan(150)
    outer = list(range(200))
    s1, c1 = O.scan_py(P, 1, outer)
    s2, c2, _ = O.scan_c(P, 1, outer=np.array(outer, dtype=np.uint64), threads=2)
    assert s1 == s2 and c1 == c2
    V = O.PlanView(P)
    T = O.CTables(V)
    T.allowed[:T.q[0]] = 0          # planted fault: filter 0 admits nothing
    s3, c3, _ = O.scan_c(T, 1, outer=np.array(outer, dtype=np.uint64), threads=2)
    assert c3[0] == 0 and c3 != c2
