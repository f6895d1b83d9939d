"""GPU parity: the sm_103a engine (through the C ABI) against the reference CPU path.

Golden vectors come from the reference's own code (tests/golden/make_golden.py); larger ranges
are checked against the C oracle and through size-independent properties (chunk additivity,
survivor re-verification, layout/shape independence).  Bit-exact throughout: survivor index
lists, per-filter-stage pass counts and the block-ordered minimum.
"""
import hashlib

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu

SHAPES = [
    dict(layout=0, mask_filters=4, threads=256, strip=4),
    dict(layout=0, mask_filters=8, threads=128, strip=1, smem_kb=64),
    dict(layout=0, mask_filters=2, threads=512, strip=7, smem_kb=0),
    dict(layout=1, mask_filters=4, threads=256, strip=3),
    dict(layout=1, mask_filters=6, threads=96, strip=2, smem_kb=16),
    dict(layout=2, mask_filters=4, threads=256, strip=2),
    dict(layout=2, mask_filters=3, threads=512, strip=5),
    dict(layout=3, mask_filters=4, threads=512, strip=2),
    dict(layout=3, mask_filters=6, threads=256, strip=3),
    dict(layout=4, mask_filters=4, threads=512, strip=2),
    dict(layout=4, mask_filters=5, threads=256, strip=3),
    dict(layout=3, mask_filters=4, threads=512, strip=8),
    dict(layout=0, mask_filters=3, threads=256, strip=64),   # windows wider than ring 2
    dict(layout=5, mask_filters=4, threads=512, strip=8),    # chosen per launch
]


def _tune(N, **kw):
    base = dict(layout=0, mask_filters=4, threads=256, strip=4, smem_kb=200, ctas_per_sm=2, count_stages=1)
    base.update(kw)
    return N.make_tune(**base)


def _scan(N, ctx, t, ob, oe):
    ctx.set_block(t)
    ctx.reset()
    ctx.reset_counts()
    ctx.launch(ob, oe - ob)
    return sorted(int(x) for x in ctx.survivors()), [int(x) for x in ctx.stage_counts()]


def _sample(seed, domain, draws, sha):
    outer = np.unique(np.random.default_rng(seed).integers(0, domain, size=draws, dtype=np.uint64))
    assert hashlib.sha256(np.ascontiguousarray(outer, dtype="<u8").tobytes()).hexdigest() == sha
    return outer


@pytest.mark.parametrize("shape", range(len(SHAPES)))
def test_small_k_every_block(native, shape):
    """k = 2..120: every block up to the first good one, survivors + stage counts (golden)."""
    import es_gb300
    N = native
    for case in golden("scan_small_k.json")["cases"]:
        plan = es_gb300.Plan(case["k"])
        ctx = N.Context(plan, _tune(N, **SHAPES[shape]))
        for blk in case["blocks"]:
            s, c = _scan(N, ctx, blk["t"], 0, ctx.n_outer)
            assert s == blk["survivors"], (case["k"], blk["t"])
            assert c == blk["counts"], (case["k"], blk["t"])
        ctx.close()


def test_k300_seeded_sample(native):
    """k = 300: 2^19 seeded outer indices x the inner ring (2^24 positions), golden counts."""
    import es_gb300
    N = native
    g = golden("scan_k300_sample.json")
    plan = es_gb300.Plan(300)
    assert [[p, T] for p, T in plan.wheel] == g["plan"]["wheel"]
    outer = _sample(g["seed"], g["domain"], g["draws"], g["outer_sha256"])
    for shape in (SHAPES[0], SHAPES[3], SHAPES[5], SHAPES[7], SHAPES[9],
                  dict(layout=0, mask_filters=8, threads=512, strip=16)):
        ctx = N.Context(plan, _tune(N, **shape))
        ctx.set_block(0)
        ctx.reset()
        ctx.reset_counts()
        ctx.launch_list(outer)
        assert sorted(int(x) for x in ctx.survivors()) == g["survivors"]
        assert [int(x) for x in ctx.stage_counts()] == g["counts"]
        ctx.close()


@pytest.mark.parametrize("role", ["primary", "confirmation"])
def test_k390_seeded_sample(native, role):
    """k = 390 recorded wheels: 2^24-position seeded sample of [0, 2^40), golden counts."""
    import es_gb300
    N = native
    g = golden("scan_k390_sample.json")["wheels"][role]
    plan = es_gb300.Plan(390, None, g["wheel"])
    assert str(plan.M) == g["plan"]["M"] and plan.rest == g["plan"]["rest"]
    outer = _sample(g["seed"], g["domain"], g["draws"], g["outer_sha256"])
    for shape in (dict(mask_filters=8), dict(layout=2, mask_filters=4), dict(layout=2, mask_filters=3, strip=1),
                  dict(layout=3, mask_filters=2), dict(layout=4, mask_filters=3)):
        ctx = N.Context(plan, _tune(N, **shape))
        ctx.set_block(0)
        ctx.reset()
        ctx.reset_counts()
        ctx.launch_list(outer)
        assert sorted(int(x) for x in ctx.survivors()) == g["survivors"], shape
        assert [int(x) for x in ctx.stage_counts()] == g["counts"], shape
        ctx.close()


def test_k300_chunk_additivity_and_oracle(native):
    """A 2^26-position range equals the C oracle, and any split of it sums to the same."""
    import es_gb300
    import es_oracle as O
    N = native
    plan = es_gb300.Plan(300)
    ctx = N.Context(plan, _tune(N))
    n = (1 << 26) // 32
    ob = 123456789
    s_all, c_all = _scan(N, ctx, 0, ob, ob + n)
    ws, wc, _ = O.scan_c(plan, 0, o_range=(ob, ob + n))
    assert s_all == ws and c_all == wc
    rng = np.random.default_rng(7)
    cuts = sorted(int(x) for x in rng.integers(1, n, size=5))
    ctx.set_block(0)
    ctx.reset()
    ctx.reset_counts()
    prev = 0
    for c in cuts + [n]:
        ctx.launch(ob + prev, c - prev)
        prev = c
    assert sorted(int(x) for x in ctx.survivors()) == s_all
    assert [int(x) for x in ctx.stage_counts()] == c_all


def test_wide_inner_rings_vs_c_oracle(native):
    """Recorded frontier wheels with 72..84-slot inner rings (three words: the four-word-row
    instance, alone and in a batch that mixes widths): 2^24 positions at an odd offset of block
    0, survivors and per-stage counts against the C oracle, F = 3..5."""
    import es_gb300
    import es_oracle as O
    N = native
    g = golden("replay_blocks.json")
    picks = {(379, "primary"), (380, "confirmation")}
    wheels = {(c["k"], c["role"]): c["wheel"] for c in g["cases"] if (c["k"], c["role"]) in picks}
    for (k, role), wheel in sorted(wheels.items()):
        plan = es_gb300.Plan(k, None, wheel)
        r0 = plan.radix[0]
        assert 64 < r0 <= 96
        n = (1 << 24) // r0
        ob = 987654321
        ws, wc, _ = O.scan_c(plan, 0, o_range=(ob, ob + n))
        for F in (3, 4, 5):
            ctx = N.Context(plan, _tune(N, mask_filters=F, strip=3))
            s, c = _scan(N, ctx, 0, ob, ob + n)
            assert s == ws and c == wc, (k, role, F)
            ctx.close()
    # a batch mixing one- and three-word rings: one launch per width class, caller item order kept
    plans = [es_gb300.Plan(300), es_gb300.Plan(379, None, wheels[(379, "primary")])]
    ctxs = [N.Context(p, _tune(N)) for p in plans]
    items = [(i, i, 0, 1000, 1000 + (1 << 20) // p.radix[0]) for i, p in enumerate(plans)]
    b = N.Batch(ctxs, items, _tune(N, mask_filters=4, strip=2))
    b.run(use_graph=False)
    b.sync()
    surv = b.survivors()
    for i, (p, it) in enumerate(zip(plans, items)):
        ws, wc, _ = O.scan_c(p, 0, o_range=(it[3], it[4]))
        assert sorted(int(r["idx"]) for r in surv if r["item"] == i) == ws, i
        assert [int(x) for x in b.item_counts(i)] == wc, i
    b.close()


def test_k390_two_wheel_batch_vs_c_oracle(native):
    """The k = 390 configuration's launch shape: both recorded wheels (two inner words, pair
    tables) as two plans of one persistent launch, with the learned-style deeper inner stage
    too; 2^22 positions of each at an odd offset, against the C oracle."""
    import es_gb300
    import es_oracle as O
    N = native
    g = golden("scan_k390_sample.json")["wheels"]
    plans = [es_gb300.Plan(390, None, g[r]["wheel"]) for r in ("primary", "confirmation")]
    ctxs = [N.Context(p, _tune(N)) for p in plans]
    items = [(i, i, 0, 424242 + 7 * i, 424242 + 7 * i + (1 << 22) // p.radix[0]) for i, p in enumerate(plans)]
    want = [O.scan_c(p, 0, o_range=(it[3], it[4]))[:2] for p, it in zip(plans, items)]
    for F, strip in ((4, 2), (5, 4)):
        b = N.Batch(ctxs, items, _tune(N, layout=2, mask_filters=F, strip=strip))
        b.run(use_graph=True)
        b.sync()
        surv = b.survivors()
        for i, (ws, wc) in enumerate(want):
            assert sorted(int(r["idx"]) for r in surv if r["item"] == i) == ws, (F, i)
            assert [int(x) for x in b.item_counts(i)] == wc, (F, i)
        b.close()


def test_batch64_prefixes(native):
    """64 seeded instances (k in 150..400) in one persistent launch: per-item golden counts."""
    import es_gb300
    N = native
    g = golden("scan_batch64.json")["instances"]
    ctxs, items = [], []
    for i, inst in enumerate(g):
        plan = es_gb300.Plan(inst["k"])
        assert [[p, T] for p, T in plan.wheel] == inst["plan"]["wheel"]
        ctxs.append(N.Context(plan, _tune(N)))
        items.append((i, i, 0, 0, inst["prefix_outer"]))
    # the plans differ in inner-ring width: one launch per width class; with layout 2 the one-
    # and two-word classes use pair tables and the three-word class the 16-byte-row word masks;
    # layout 5 lets the library choose per class (staged word masks where they fit at F = 4)
    for graph, layout, F in ((False, 0, 6), (True, 0, 6), (False, 2, 6), (True, 5, 6), (False, 5, 4)):
        b = N.Batch(ctxs, items, _tune(N, layout=layout, mask_filters=F, strip=2))
        b.run(use_graph=graph)
        b.sync()
        surv = b.survivors()
        for i, inst in enumerate(g):
            assert [int(x) for x in b.item_counts(i)] == inst["counts"], i
            got = sorted(int(r["idx"]) for r in surv if r["item"] == i)
            assert got == inst["survivors"], i
        b.close()


def test_batch64_config_items_match_c_oracle(native):
    """Config 3 as the measurement runs it (one persistent launch over the 64 seeded instances,
    each with its full range): every instance of at most 2^24 positions, survivors and per-stage
    counts, against the C oracle of the reference path."""
    import es_configs
    import es_gb300
    import es_oracle as O
    res = es_configs.batch64(autotune=False, reps=1)
    assert res["instances"] == 64 and len(res["small_items"]) >= 16
    for it in res["small_items"]:
        ws, wc, _ = O.scan_c(es_gb300.Plan(it["k"]), 0, o_range=tuple(it["o_range"]))
        assert it["survivors"] == ws, it["item"]
        assert it["counts"] == wc, it["item"]


def test_search_matches_bfile(native, bfile):
    """Drop-in search() reproduces g(k) for k = 1..240 (harness/gate.py semantics, extended past
    its k <= 140 gate; about 4e11 positions in all)."""
    import es_gb300
    for k in range(1, 241):
        res = es_gb300.GpuSieve(es_gb300.Plan(k)).search(None)
        assert res["status"] == "FOUND" and res["g"] == bfile[k], (k, res)


def test_run_k_driver_loop(native, bfile):
    """The block loop of harness/run_k.py:99-182 driven through the GpuSieve attribute surface."""
    import es_gb300
    from es_plan import is_admissible
    for k in (33, 60, 97, 120, 150):
        plan = es_gb300.Plan(k, {"chunk_log2": 12})
        sieve = es_gb300.GpuSieve(plan)
        assert sieve.R_outer * sieve.r0 == plan.R
        t = 0
        while True:
            for j, q in enumerate(sieve.rest_q):
                sieve.tconst_h[j] = ((t % q) * sieve.rest_Mmodq[j]) % q
            sieve.tconst.set(sieve.tconst_h)
            surv, done = [], 0
            while done < sieve.R_outer:
                cnt = min(sieve.ochunk, sieve.R_outer - done)
                sieve.out_n.fill(0)
                sieve._launch(done, cnt)
                nsv = int(sieve.out_n.get()[0])
                assert nsv <= sieve.out_cap
                if nsv:
                    surv.extend(int(x) for x in sieve.out[:nsv].get())
                done += cnt
            cands = sorted(plan.idx_to_n(i, t) for i in surv)
            good = [n for n in cands if is_admissible(n, k)]
            assert not [n for n in cands if n > k + 1 and n not in good]
            if good:
                assert good[0] == bfile[k]
                break
            t += 1


def test_min_survivor_and_overflow(native):
    import es_gb300
    N = native
    plan = es_gb300.Plan(40)
    ctx = N.Context(plan, _tune(N))
    # g(40) lies in block 0 of this plan; device min equals the host min of good survivors
    s, _ = _scan(N, ctx, 0, 0, ctx.n_outer)
    ns = sorted(plan.idx_to_n(i, 0) for i in s)
    good = [n for n in ns if n > 41]
    m = ctx.min_survivor()
    assert m is not None and m[0] * plan.M + m[1] == good[0]
    # capacity 1 with several survivors -> count exceeds capacity, reading raises
    ctx.set_capacity(1)
    ctx.reset()
    ctx.launch(0, ctx.n_outer)
    assert ctx.count() == len(s) > 1
    with pytest.raises(N.EsError):
        ctx.survivors()


def test_edge_ranges(native):
    """Empty ranges, ranges inside one ring-1 cycle, ranges that start and end inside a ring-2
    row (a warp-unit spans 32 rows, so its first lanes may start later than the rest),
    duplicates in a list, range checks."""
    import es_gb300
    import es_oracle as O
    N = native
    plan = es_gb300.Plan(200)
    r1, r2 = plan.radix[1], plan.radix[2]
    row = r1 * r2   # outer indices per ring-2 row
    ranges = ((0, 0), (5, 6), (r1 - 1, r1 + 1), (3 * r1 + 2, 7 * r1 + 5), (row - 1, row + 1),
              (5 * row + 3 * r1 + 1, 40 * row + 7), (2 * row, 70 * row), (33 * row - 5, 33 * row + r1 * 3))
    for strip in (4, 64):
        ctx = N.Context(plan, _tune(N, strip=strip))
        for ob, oe in ranges + ((ctx.n_outer - 3, ctx.n_outer),):
            s, c = _scan(N, ctx, 2, ob, oe)
            ws, wc, _ = O.scan_c(plan, 2, o_range=(ob, oe))
            assert s == ws and c == wc, (strip, ob, oe)
        ctx.close()
    ctx = N.Context(plan, _tune(N))
    lst = np.array([9, 9, 1, 12345, 9], dtype=np.uint64)
    ctx.set_block(1)
    ctx.reset()
    ctx.reset_counts()
    ctx.launch_list(lst)
    ws, wc, _ = O.scan_c(plan, 1, outer=lst)
    assert sorted(int(x) for x in ctx.survivors()) == ws
    assert [int(x) for x in ctx.stage_counts()] == wc
    with pytest.raises(N.EsError):
        ctx.launch(ctx.n_outer, 1)


def test_k390_autotuned_config_vs_c_oracle(native):
    """The k = 390 configuration as the measurement runs it: both recorded wheels in one
    persistent launch, with the launch shape the batch autotuner picks for them, in the reference
    (analytic) cascade orders and in the learned planner's orders; 2^26 positions of each wheel
    at an odd offset, survivors and per-stage counts against the C oracle."""
    import es_autotune
    import es_configs
    import es_gb300
    import es_learned
    import es_oracle as O
    N = native
    model = es_learned.CostModel.load(es_learned.MODEL_PATH)
    for arm in ("analytic", "learned"):
        plans = []
        for wheel in es_configs.K390_WHEELS.values():
            P = es_gb300.Plan(390, None, wheel)
            if arm == "learned":
                P = P.with_order(es_learned.learned_order(model, P)[1])
            plans.append(P)
        F = es_autotune.DEFAULT["mask_filters"]
        start = dict(es_autotune.DEFAULT, layout=N.layout_for_plan(plans[0], F))
        ctxs = [N.Context(p, N.make_tune(**start)) for p in plans]
        probe = [(i, i, 0, 0, min(c.n_outer, (1 << 30) // c.r0)) for i, c in enumerate(ctxs)]
        tune, _ = es_autotune.tune_batch(ctxs, probe, start=start)
        assert all(tune[key] in vals for key, vals in es_autotune.SPACE.items()), tune
        n = (1 << 26) // plans[0].radix[0]
        items = [(i, i, 0, 777777 + 5 * i, 777777 + 5 * i + n) for i in range(len(plans))]
        b = N.Batch(ctxs, items, N.make_tune(**dict(tune, count_stages=1)))
        b.run(use_graph=True)
        b.sync()
        surv = b.survivors()
        for i, (P, it) in enumerate(zip(plans, items)):
            ws, wc, _ = O.scan_c(P, 0, o_range=(it[3], it[4]))
            assert sorted(int(r["idx"]) for r in surv if r["item"] == i) == ws, (arm, i, tune)
            assert [int(x) for x in b.item_counts(i)] == wc, (arm, i, tune)
        b.close()
        for c in ctxs:
            c.close()


def test_autotune_plan_shape_is_exact(native, tmp_path):
    """es_autotune.tune_plan on a small plan: every field of the shape it returns is the start
    shape's (the default with the layout rule's layout) or a value of the search space, the shape
    is cached (a second call returns it without timing), and the survivors and per-stage counts
    under it equal the C oracle's."""
    import es_autotune
    import es_gb300
    import es_oracle as O
    N = native
    plan = es_gb300.Plan(250)
    cache = str(tmp_path / "tune.json")
    space = {"strip": [1, 2, 4], "mask_filters": [3, 4, 5], "layout": [0, 2, 1], "threads": [256, 512]}
    tune = es_autotune.tune_plan(plan, probe_log2=26, cache=cache, space=space)
    start = dict(es_autotune.DEFAULT, layout=N.layout_for_plan(plan, es_autotune.DEFAULT["mask_filters"]))
    assert all(tune[key] in vals or tune[key] == start[key] for key, vals in space.items()), tune
    assert es_autotune.tune_plan(plan, probe_log2=26, cache=cache, space=space) == tune
    ctx = N.Context(plan, N.make_tune(**dict(tune, count_stages=1)))
    ob = 31337
    n = (1 << 24) // plan.radix[0]
    s, c = _scan(N, ctx, 0, ob, ob + n)
    ws, wc, _ = O.scan_c(plan, 0, o_range=(ob, ob + n))
    assert s == ws and c == wc, tune
    ctx.close()


def test_whole_recorded_block_replay(native):
    """One whole recorded frontier block: k = 379, primary wheel, block 0 (7.17e14 positions, a
    few minutes), every position through the drop-in scan_block; the reference driver's block
    audit built from its survivors must equal the recorded one field by field (positions, kernel
    survivors, survivors with n > k+1, survivors passing the exact test, sha256 of the sorted
    survivors).  The record comes from the reference project's evidence/through400/runs.json."""
    import es_configs
    g = golden("replay_blocks.json")
    case = next(c for c in g["cases"] if c["k"] == 379 and c["role"] == "primary" and c["audit"]["t"] == 0)
    res = es_configs.replay([case])
    assert res["all_match"], res["cases"][0]["fields"]
    assert res["cases"][0]["audit"]["passed_ref_is_good"] == 1
