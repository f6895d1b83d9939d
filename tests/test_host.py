"""CPU: host logic of the drop-in engine, with the device replaced by a fake backed by the C
oracle (block loop, block-ordered search, DISAGREEMENT on a planted fault, overflow fallback)."""
import pytest

from fake_device import FakeBatch, FakeCtx


def _sieve(monkeypatch, k, plant=None, cap=1 << 20, tun=None):
    import es_gb300
    plan = es_gb300.Plan(k, tun)
    fake = FakeCtx(plan, cap, plant)
    monkeypatch.setattr(es_gb300.N, "Context", lambda p, t, capacity=None: fake)
    monkeypatch.setattr(es_gb300.N, "Batch", FakeBatch)
    return es_gb300.GpuSieve(plan), fake


@pytest.mark.parametrize("k", [1, 2, 5, 30, 60, 70, 97])
def test_search_control_flow_matches_bfile(monkeypatch, bfile, k):
    sieve, _ = _sieve(monkeypatch, k)
    res = sieve.search(None)
    assert res["status"] == "FOUND" and res["g"] == bfile[k]
    assert res["residues_checked"] == (res["block"] + 1) * sieve.plan.R


def test_planted_fault_is_a_disagreement(monkeypatch):
    """A kernel 'survivor' whose n fails the exact test must end the search as DISAGREEMENT."""
    import es_gb300
    plan = es_gb300.Plan(120)
    bad_idx = next(i for i in range(plan.R) if plan.idx_to_n(i, 0) > 121
                   and not es_gb300.is_admissible(plan.idx_to_n(i, 0), 120))
    sieve, _ = _sieve(monkeypatch, 120, plant=bad_idx)
    res = sieve.search(1)
    assert res["status"] == "DISAGREEMENT"
    assert plan.idx_to_n(bad_idx, 0) in res["ref_rejected"]


def test_exhausted_blocks(monkeypatch):
    sieve, _ = _sieve(monkeypatch, 30)   # g(30) lies in block 9
    res = sieve.search(3)
    assert res["status"] == "EXHAUSTED_BLOCKS" and res["blocks"] == 3


def test_overflow_falls_back_then_raises(monkeypatch):
    sieve, fake = _sieve(monkeypatch, 40, cap=1, tun={"max_survivors": 1, "chunk_log2": 5})
    with pytest.raises(RuntimeError):
        sieve.scan_block(0)


def test_block_from_tconst_and_verdict():
    import es_gb300
    import es_native as N
    P = es_gb300.Plan(390)
    rq = [P.info[p][0] for p in P.rest]
    rm = [P.M % q for q in rq]
    for t in (0, 3, 99991, 2**50 + 3):
        assert es_gb300.block_from_tconst(rq, rm, N.tconst_for(P, t)) == t
    Q = es_gb300.Plan(60)
    cands, good, bad = es_gb300.verdict(Q, 6, [0, 1, 2])
    assert cands == sorted(Q.idx_to_n(i, 6) for i in (0, 1, 2))
    assert set(good) | set(bad) <= set(cands)


def test_load_known(tmp_path):
    import es_gb300
    a = tmp_path / "a.txt"
    b = tmp_path / "b.txt"
    a.write_text("1 3\n2 6\n# comment\n")
    b.write_text("2 99\n3 7\n")
    known = es_gb300.load_known(str(a), str(b), str(tmp_path / "missing.txt"))
    assert known == {1: (3, "a.txt"), 2: (6, "a.txt"), 3: (7, "b.txt")}


def test_layout_rule():
    """The default table layout: word masks staged in shared memory where the inner-stage tables
    fit (k = 300 at F = 2..4), else pair tables where the word masks do not fit L1 (k = 300 at
    F = 5, k = 390), word masks for inner rings wider than two words; "auto" in the drop-in
    tunables resolves through it."""
    import es_gb300
    import es_native as N
    P300 = es_gb300.Plan(300)
    assert N.layout_for_plan(P300, 4) == N.LAYOUT_SMEM
    assert N.layout_for_plan(P300, 3) == N.LAYOUT_SMEM
    assert N.layout_for_plan(P300, 2) == N.LAYOUT_SMEM
    assert N.layout_for_plan(P300, 5) == N.LAYOUT_PAIR
    wheel = [[3, 6], [2, 9], [211, 1], [139, 1], [103, 1], [137, 1], [101, 1], [67, 1], [5, 2],
             [199, 1], [23, 2], [79, 1], [197, 1], [131, 1], [7, 2], [17, 1]]
    assert N.layout_for_plan(es_gb300.Plan(390, None, wheel), 4) == N.LAYOUT_PAIR
    assert N.layout_for(96, [1009, 1013], 2) == N.LAYOUT_WORDMASK
    assert N.layout_for(48, [30011, 30013, 30047], 3) == N.LAYOUT_PAIR   # 720 KB of word masks
    assert es_gb300._tune_from(dict(es_gb300.TUNABLES), P300).layout == N.LAYOUT_SMEM
    assert es_gb300._tune_from(dict(es_gb300.TUNABLES, layout="scalar"), P300).layout == N.LAYOUT_SCALAR
    assert es_gb300._tune_from(dict(es_gb300.TUNABLES, layout="wordmask"), P300).layout == N.LAYOUT_WORDMASK
