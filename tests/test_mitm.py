"""The meet-in-the-middle search: planner and oracle against the reference's own CPU path (CPU),
and the GPU kernel (es_mitm_*, through the C ABI) bit-exact against both (GPU).

tests/golden/mitm_small_k.json comes from the reference itself (harness/mitm_fast.py run
unchanged by tests/golden/make_golden_mitm.py, mem_gb = 0.05, bound_mult = 1.0): for k = 8..130,
140, 150 the wheel and halves, g(k), the final bound, the total of candidates tested and, per
round, the survivors of the residual filters with n > k + 1.
"""
import pytest

from conftest import golden


def _cases(max_k=None):
    return [c for c in golden("mitm_small_k.json")["cases"] if max_k is None or c["k"] <= max_k]


def _plan(c):
    import es_mitm
    return es_mitm.MitmPlan(c["k"], golden("mitm_small_k.json")["mem_gb"])


def test_planner_matches_reference():
    """Wheel, halves and sizes of every recorded case (harness/mitm_search.py:64-128)."""
    for c in _cases():
        P = _plan(c)
        assert P.wheel == c["wheel"], c["k"]
        assert (P.w1, P.w2, P.n1, P.n2) == (c["w1"], c["w2"], c["S1"], c["S2"]), c["k"]
        assert P.M.bit_length() == c["M_bits"]


def test_oracle_matches_reference_rounds(bfile):
    """The oracle's round loop gives the reference's per-round survivors, total candidates,
    final bound and g(k) (which is the b-file's): every recorded k <= 104 and a few larger ones
    (the numpy restatement takes seconds to minutes beyond; the GPU test covers every case)."""
    import es_mitm_oracle as MO
    for c in [c for c in _cases(130) if c["k"] <= 104 or c["k"] in (118, 120, 122, 125)]:
        P = _plan(c)
        rounds, g = MO.mitm_rounds(P, 1.0)
        assert g == int(c["g"]) == bfile[c["k"]], c["k"]
        assert len(rounds) == len(c["rounds"]), c["k"]
        assert rounds[-1][0] == int(c["bound"]), c["k"]
        assert sum(r[2] for r in rounds) == c["candidates_total"], c["k"]
        for (B, surv, cand), want in zip(rounds, c["rounds"]):
            assert surv == sorted(int(n) for n in want["referee_tested"]), (c["k"], B)


@pytest.mark.gpu
def test_gpu_rounds_match_reference(native):
    """Every recorded case on the GPU with the reference's bounds: per-round survivors (n > k+1),
    the total of candidates tested and g(k), bit-exact."""
    import es_mitm
    from es_plan import is_admissible
    for c in _cases():
        P = _plan(c)
        eng = es_mitm.MitmEngine(P)
        B = max(int(1.0 * P.E), 1)
        total, g = 0, None
        for want in c["rounds"]:
            B = min(B, P.M)
            surv, cand = eng.scan(B)
            total += cand
            big = [n for n in surv if n > P.k + 1]
            assert big == sorted(int(n) for n in want["referee_tested"]), (c["k"], B)
            good = [n for n in big if is_admissible(n, P.k)]
            if good:
                g = good[0]
            B = min(B * 4, P.M)
        eng.close()
        assert g == int(c["g"]), c["k"]
        assert total == c["candidates_total"], c["k"]


@pytest.mark.gpu
def test_gpu_scan_against_oracle_partial_ranges(native):
    """Sub-ranges of S1 and bounds that wrap past M (B near M, and B = M: the whole circle),
    against the oracle: the kernel's index decode, circular runs and chunking."""
    import es_mitm
    import es_mitm_oracle as MO
    # bounds near M test every residue of the wheel, which the oracle materialises on the host:
    # only for wheels of at most ~1e7 residues
    for k, near_m in ((40, True), (50, True), (60, True), (70, True), (97, False), (120, False)):
        P = es_mitm.MitmPlan(k, 0.05)
        orc = MO.MitmOracle(P)
        eng = es_mitm.MitmEngine(P)
        bounds = (max(int(P.E), 1), P.M // 3, P.M - 1, P.M) if near_m else (max(int(P.E), 1), 4 * max(int(P.E), 1))
        for B in bounds:
            want, wc = orc.scan(B)
            got, gc = eng.scan(B)
            assert got == want and gc == wc, (k, B)
            mid = P.n1 // 2 + 7          # two parts of S1 add up to the whole
            a, ac = eng.scan(B, 0, mid)
            b, bc = eng.scan(B, mid, P.n1)
            assert sorted(a + b) == want and ac + bc == wc, (k, B)
        eng.close()


@pytest.mark.gpu
def test_gpu_mitm_gate(native, bfile):
    """harness/gate_mitm_gpu.py's gate through the engine's search (default memory budget and
    bound multiplier): FOUND g(k) equal to the b-file, or MITM_OUT_OF_RANGE, for k = 2..160."""
    import es_mitm
    found = 0
    for k in range(2, 161):
        r = es_mitm.mitm_gpu(k)
        assert r["status"] in ("FOUND", "MITM_OUT_OF_RANGE"), (k, r)
        if r["status"] == "FOUND":
            assert r["g"] == bfile[k], (k, r)
            found += 1
    assert found >= 140
