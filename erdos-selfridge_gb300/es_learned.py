#!/usr/bin/env python3
"""Learned planner: an MLP cost model that stands in for the knapsack planner's analytic estimate.

The reference planner (sieve/gpu_sieve_v9.py:187-227) ranks wheels by expected residue checks
R / (1 - e^{-M/E}) and orders filters by conditional pass rate (v9:230-237); it assumes every plan
scans at the same rate.  On the GPU the rate is not constant: it depends on the inner radix, on
whether the first filters' word-mask tables stay in L1, on how fast the first filters reject, on
the number of rings.  This module

1. enumerates ~40 candidate plans per k: wheels from the reference's own sweep grids
   (harness/plan_sweep.py:33-49: planner, n_mult, cost_scale, m_cap_bits) and banned-prime
   re-plans (harness/plan_sweep.py:52-58), each with several filter orders;
2. probes each on the GPU: 2^28 positions of block 0 -> Gcand/s and per-filter pass fractions;
3. trains a 3-layer FP32 MLP (64 hidden, ReLU) with this library's own CUDA kernels
   (es_mlp_*) to predict log throughput and the log-error of the analytic estimate of expected
   positions to the first survivor (the planner's expected-checks formula is a good start; the
   network learns what it misses, which needs far less data than learning positions outright);
4. chooses, per k, the plan with the least predicted time = positions / throughput, and compares
   it on held-out k with the analytic choice (least expected checks, reference filter order).

The analytic planner stays the fallback (no model, or a k outside the trained range) and the judge
of the model's error: both predictions are scored against the measured outcome.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import multiprocessing as mp
import os
import statistics
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)

import es_plan  # noqa: E402

N_FIRST = 6          # filters described individually in the features
MODEL_PATH = os.path.join(HERE, "data", "cost_model.json")   # trained on 160 k of 100..400
FEATURE_DIM = 16 + 3 * N_FIRST
PROBE_LOG2 = 28


# ------------------------------------------------------------------ the GPU MLP (ctypes)
class MLP:
    """3-layer FP32 MLP on the GPU (es_mlp_* kernels): in -> 64 -> 64 -> out, ReLU."""

    def __init__(self, in_dim: int, out_dim: int = 2, hidden: int = 64, seed: int = 0):
        import es_native as N
        L = N.lib()
        f32p, u64 = C.POINTER(C.c_float), C.c_uint64
        for name, args in (("es_mlp_create", [C.c_uint32, C.c_uint32, C.c_uint32, u64, C.POINTER(C.c_void_p)]),
                           ("es_mlp_destroy", [C.c_void_p]),
                           ("es_mlp_num_params", [C.c_void_p, C.POINTER(u64)]),
                           ("es_mlp_get_params", [C.c_void_p, f32p, u64]),
                           ("es_mlp_set_params", [C.c_void_p, f32p, u64]),
                           ("es_mlp_forward", [C.c_void_p, f32p, u64, f32p]),
                           ("es_mlp_loss_grad", [C.c_void_p, f32p, f32p, u64, f32p, f32p]),
                           ("es_mlp_train", [C.c_void_p, f32p, f32p, u64, C.c_uint32, C.c_uint32, C.c_float, u64, f32p])):
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = C.c_int
        L.es_mlp_last_error.restype = C.c_char_p
        self.L = L
        self.in_dim, self.out_dim, self.hidden = in_dim, out_dim, hidden
        h = C.c_void_p()
        self._check(L.es_mlp_create(in_dim, hidden, out_dim, seed, C.byref(h)))
        self.h = h
        n = C.c_uint64()
        self._check(L.es_mlp_num_params(h, C.byref(n)))
        self.n_params = n.value

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError(f"es_mlp error {rc}: {self.L.es_mlp_last_error().decode()}")

    @staticmethod
    def _f32(a):
        return np.ascontiguousarray(a, dtype=np.float32)

    def close(self):
        if getattr(self, "h", None):
            self.L.es_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self) -> np.ndarray:
        out = np.zeros(self.n_params, dtype=np.float32)
        self._check(self.L.es_mlp_get_params(self.h, out.ctypes.data_as(C.POINTER(C.c_float)), self.n_params))
        return out

    def set_params(self, p) -> None:
        p = self._f32(p)
        self._check(self.L.es_mlp_set_params(self.h, p.ctypes.data_as(C.POINTER(C.c_float)), self.n_params))

    def forward(self, X) -> np.ndarray:
        X = self._f32(X)
        Y = np.zeros((X.shape[0], self.out_dim), dtype=np.float32)
        fp = C.POINTER(C.c_float)
        self._check(self.L.es_mlp_forward(self.h, X.ctypes.data_as(fp), X.shape[0], Y.ctypes.data_as(fp)))
        return Y

    def loss_grad(self, X, T) -> tuple[float, np.ndarray]:
        X, T = self._f32(X), self._f32(T)
        g = np.zeros(self.n_params, dtype=np.float32)
        loss = C.c_float()
        fp = C.POINTER(C.c_float)
        self._check(self.L.es_mlp_loss_grad(self.h, X.ctypes.data_as(fp), T.ctypes.data_as(fp), X.shape[0],
                                            C.byref(loss), g.ctypes.data_as(fp)))
        return loss.value, g

    def train(self, X, T, epochs: int = 400, batch: int = 256, lr: float = 1e-3, seed: int = 0) -> float:
        X, T = self._f32(X), self._f32(T)
        loss = C.c_float()
        fp = C.POINTER(C.c_float)
        self._check(self.L.es_mlp_train(self.h, X.ctypes.data_as(fp), T.ctypes.data_as(fp), X.shape[0],
                                        epochs, batch, lr, seed, C.byref(loss)))
        return loss.value


# ------------------------------------------------------------------ features and targets
def _log2(x: float) -> float:
    return math.log2(x) if x > 0 else 0.0


def features(plan) -> np.ndarray:
    """Description of a plan (wheel + cascade order) for the cost model."""
    k = plan.k
    r0 = plan.radix[0] if plan.radix else 1
    r1 = plan.radix[1] if len(plan.radix) > 1 else 1
    W = (r0 + 31) // 32
    rates = plan.conditional_pass_rates()
    qs = [plan.info[p][0] for p in plan.rest]
    log2E = -math.log2(plan.density_all) if plan.density_all > 0 else 0.0
    first_tab = sum(q * W * 4 for q in qs[:4])
    f = [k / 400.0, log2E / 128.0, _log2(plan.M) / 128.0, _log2(plan.R) / 64.0, _log2(r0) / 8.0,
         _log2(r1) / 8.0, len(plan.radix) / 20.0, len(plan.rest) / 80.0, W / 4.0,
         _log2(first_tab) / 24.0,
         sum(_log2(r) for r in rates[:4]) / -16.0,
         sum(_log2(r) for r in rates) / -64.0,
         _log2(plan._true_cost()) / 64.0,
         (r0 % 32) / 32.0]
    # the table layout the engine picks for the inner stage (es_native.layout_for, F = 4): staged
    # in shared memory, pair tables or word masks through L1 -- a step in throughput the table
    # bytes alone describe only through a sharp threshold
    import es_native
    lay = es_native.layout_for(r0, qs, 4)
    f += [1.0 if lay == es_native.LAYOUT_SMEM else 0.0, 1.0 if lay == es_native.LAYOUT_PAIR else 0.0]
    for j in range(N_FIRST):
        if j < len(qs):
            f += [_log2(qs[j]) / 20.0, rates[j], _log2(qs[j] * W * 4) / 24.0]
        else:
            f += [0.0, 1.0, 0.0]
    assert len(f) == FEATURE_DIM
    return np.array(f, dtype=np.float32)


def expected_positions(plan, counts, n_probe: int, min_count: int = 200) -> float:
    """Expected positions the block-ordered search scans before it ends: R / (1 - e^{-R p}),
    p = survivor probability per position from the probe's measured pass fractions (analytic
    conditional rates where a stage saw fewer than min_count candidates)."""
    rates = plan.conditional_pass_rates()
    logp, prev = 0.0, n_probe
    for j, r in enumerate(rates):
        c = counts[j] if j < len(counts) else 0
        if prev >= min_count and c > 0:
            logp += math.log(c / prev)
        else:
            logp += math.log(r)
        prev = c
    Rp = plan.R * math.exp(logp)
    if Rp < 1e-12:
        return math.exp(-logp)           # 1/p: far fewer than one survivor per block
    return plan.R / -math.expm1(-Rp)


# ------------------------------------------------------------------ candidate plans
WHEEL_TUNES = [
    None,                                            # the reference default (truecost)
    {"planner": "knapsack", "n_mult": 1.0},
    {"planner": "knapsack", "n_mult": 0.25},
    {"planner": "knapsack", "n_mult": 4.0},
    {"m_cap_bits": 100},
    {"m_cap_bits": 80},
    {"cost_scale": 64},
]


def _orders(plan, rng, shuffles: int = 2, unique: bool = True) -> list[tuple[str, list[int]]]:
    """Cascade-order families: the reference order, orders that trade rejection against the
    word-mask table footprint (several L1 budgets, two of them sized for pair tables),
    small-q-first heads, and random heads."""
    ref = list(plan.rest)
    out = [("reference", ref)]
    W = ((plan.radix[0] if plan.radix else 1) + 31) // 32
    rates = dict(zip(ref, plan.conditional_pass_rates()))
    size = {p: plan.info[p][0] * W * 4 for p in ref}

    def rest_after(head):
        hs = set(head)
        return head + [p for p in ref if p not in hs]
    # rejection per unit of table footprint, at three penalty scales
    for name, scale in (("table-aware-16k", 16384.0), ("table-aware", 65536.0), ("table-aware-256k", 262144.0)):
        head = sorted(ref, key=lambda p: (1.0 - rates[p]) / (1.0 + size[p] / scale), reverse=True)[:N_FIRST]
        out.append((name, rest_after(head)))
    # greedy: most rejection among the first four within an L1 budget, the rest by pass rate; the
    # two smallest budgets keep the pair tables (twice the bytes, one load per filter) in L1 too
    for name, budget in (("l1-96k", 96 * 1024), ("l1-160k", 160 * 1024), ("l1-pair-48k", 48 * 1024),
                         ("l1-pair-88k", 88 * 1024)):
        head, used = [], 0
        for p in sorted(ref, key=lambda p: rates[p]):
            if len(head) < 4 and used + size[p] <= budget:
                head.append(p)
                used += size[p]
        out.append((name, rest_after(head)))
    out.append(("small-q-first", sorted(ref[:8], key=lambda p: plan.info[p][0]) + ref[8:]))
    out.append(("small-q-first-4", sorted(ref[:4], key=lambda p: plan.info[p][0]) + ref[4:]))
    for i in range(shuffles):
        perm = ref[:8]
        rng.shuffle(perm)
        out.append((f"shuffle{i}", perm + ref[8:]))
    if not unique:
        return out
    seen, uniq = set(), []
    for name, o in out:
        key = tuple(o)
        if key not in seen:
            seen.add(key)
            uniq.append((name, o))
    return uniq


def candidate_specs(k: int, seed: int = 0) -> list[dict]:
    """Candidate (wheel, order) specs for k; deterministic for a seed."""
    rng = np.random.default_rng(seed * 1000003 + k)
    specs, wheels = [], set()
    base = es_plan.Plan(k)
    log2E = -math.log2(base.density_all)
    wheel_list = []
    for tun in WHEEL_TUNES:
        P = base if tun is None else es_plan.Plan(k, tun)
        wheel_list.append(("default" if tun is None else json.dumps(tun, sort_keys=True), P))
    for ban in sorted({p for p, _ in base.wheel})[:2]:
        ps = [p for p in es_plan.primes_upto(k) if p != ban]
        w = es_plan.plan_wheel(k, ps, log2E, dict(es_plan.TUNABLES))
        wheel_list.append((f"ban{ban}", es_plan.Plan(k, None, [[p, T] for p, T in w])))
    for wname, P in wheel_list:
        key = tuple(sorted(P.wheel))
        if key in wheels or not P.wheel:
            continue
        wheels.add(key)
        for oname, order in _orders(P, rng):
            specs.append({"k": k, "wheel": [[p, T] for p, T in P.wheel], "order": order,
                          "wheel_name": wname, "order_name": oname})
    return specs


def _materialise(spec) -> dict:
    """Worker side: build the plan, its device arrays and its analytic description."""
    import es_native as N
    P = es_plan.Plan(spec["k"], None, spec["wheel"]).with_order(spec["order"])
    A = N.PlanArrays(P)
    return {"spec": spec, "features": features(P), "R": P.R, "M_bits": P.M.bit_length(),
            "true_cost": P._true_cost(), "rates": P.conditional_pass_rates(),
            "arrays": (P.k, A.radix, A.term_lo, A.term_hi, A.q, A.allowed, P.M), "r0": P.radix[0],
            "ref_order": spec["order_name"] == "reference"}


def _specs_for(k):
    return candidate_specs(k)


# ------------------------------------------------------------------ GPU probes
def probe(item: dict, tune=None, log2_pos: int | None = None, reps: int = 3) -> dict:
    """Time 2^log2_pos positions of block 0 (median of reps) and take stage counts once."""
    import es_native as N
    log2_pos = PROBE_LOG2 if log2_pos is None else log2_pos
    k, radix, lo, hi, q, allowed, M = item["arrays"]
    A = N.PlanArrays.from_arrays(k, radix, lo, hi, q, allowed, M)
    tune = dict(tune or {})
    if "layout" not in tune:   # the engine's default choice for this plan
        tune["layout"] = N.layout_for(int(radix[0]) if len(radix) else 1, q, tune.get("mask_filters", 4))
    t = N.make_tune(**dict(tune, count_stages=1))
    ctx = N.Context.from_arrays(A, t, len(q))
    try:
        r0 = int(radix[0]) if len(radix) and radix[0] else 1
        n_outer = max(1, min(ctx.n_outer, (1 << log2_pos) // r0))
        ctx.set_block(0, np.zeros(len(q), dtype=np.uint32))
        ctx.reset_counts()
        ctx.reset()
        ctx.launch(0, n_outer)
        counts = [int(x) for x in ctx.stage_counts()]
        t_run = N.make_tune(**dict(tune, count_stages=0))
        ctx.set_tune(t_run)
        n_pos = n_outer * r0
        blocks = 1
        if n_pos < (1 << log2_pos) and n_outer >= ctx.n_outer:
            # the whole block is shorter than the probe: time consecutive blocks in one graph-
            # replayed launch, the way the block-ordered search issues them, so that a short
            # block's launch overhead is not taken for its scan rate
            blocks = int(min(64, -(-(1 << log2_pos) // n_pos)))
        if blocks > 1:
            items = [(0, b, b, 0, n_outer) for b in range(blocks)]   # one group per block: none skipped
            bt = N.Batch([ctx], items, t_run)
            try:
                bt.run(use_graph=True)
                bt.sync()
                ms = []
                for _ in range(reps):
                    bt.run(use_graph=True)
                    ms.append(bt.sync())
            finally:
                bt.close()
        else:
            ctx.reset()
            ctx.launch_timed(0, n_outer)
            ms = []
            for _ in range(reps):
                ctx.reset()
                ms.append(ctx.launch_timed(0, n_outer))
        m = statistics.median(ms)
    finally:
        ctx.close()
    return {"gcand": blocks * n_pos / m / 1e6, "ms": m, "positions": n_pos, "blocks": blocks, "counts": counts}


class _PlanLike:
    """Minimal plan view for expected_positions from a materialised record."""

    def __init__(self, rec):
        self.R = rec["R"]
        self._rates = rec["rates"]

    def conditional_pass_rates(self):
        return self._rates


def collect(ks, procs: int | None = None, log=None, tune=None) -> list[dict]:
    """Candidates for every k built in a process pool, probed one by one on the GPU."""
    ctx = mp.get_context("spawn")
    rows = []
    with ctx.Pool(procs or os.cpu_count() or 4) as pool:
        all_specs = [s for specs in pool.map(_specs_for, ks) for s in specs]
        for rec in pool.imap(_materialise, all_specs, chunksize=4):
            pr = probe(rec, tune)
            epos = expected_positions(_PlanLike(rec), pr["counts"], pr["positions"])
            row = {"k": rec["spec"]["k"], "wheel_name": rec["spec"]["wheel_name"],
                   "order_name": rec["spec"]["order_name"], "ref_order": rec["ref_order"],
                   "features": [float(x) for x in rec["features"]], "gcand": pr["gcand"],
                   "log_tp": math.log(pr["gcand"]), "log_pos": math.log(epos),
                   "true_cost": rec["true_cost"], "M_bits": rec["M_bits"], "R": rec["R"],
                   "counts": pr["counts"][:8], "probe_positions": pr["positions"],
                   "rates": [float(x) for x in rec["rates"]],
                   "wheel": rec["spec"]["wheel"], "order": rec["spec"]["order"]}
            rows.append(row)
            if log and len(rows) % 200 == 0:
                log(f"probed {len(rows)}/{len(all_specs)}")
    return rows


# ------------------------------------------------------------------ model fit and choice
class CostModel:
    """MLP on standardised features/targets.  Outputs: log throughput (Gcand/s) and the log-error
    of the analytic expected-positions estimate, log(positions) - log(true_cost); a plan's
    predicted log time is log(true_cost) + output[1] - output[0] (``log_time``)."""

    TARGETS = "log_tp, log_pos - log(true_cost)"

    def __init__(self, seed: int = 0, hidden: int = 64):
        self.seed, self.hidden = seed, hidden
        self.mlp = None

    def fit(self, rows, epochs: int = 600, batch: int = 256, lr: float = 2e-3) -> float:
        X = np.array([r["features"] for r in rows], dtype=np.float64)
        Y = np.array([[r["log_tp"], r["log_pos"] - math.log(r["true_cost"])] for r in rows], dtype=np.float64)
        self.xm, self.xs = X.mean(0), X.std(0) + 1e-6
        self.ym, self.ys = Y.mean(0), Y.std(0) + 1e-6
        self.mlp = MLP(X.shape[1], 2, self.hidden, self.seed)
        return self.mlp.train((X - self.xm) / self.xs, (Y - self.ym) / self.ys, epochs, batch, lr, self.seed)

    def predict(self, feats) -> np.ndarray:
        X = (np.asarray(feats, dtype=np.float64) - self.xm) / self.xs
        return self.mlp.forward(X).astype(np.float64) * self.ys + self.ym

    def log_time(self, feats, true_costs) -> list[float]:
        """Predicted log time-to-completion (up to a constant) of plans with these features and
        analytic expected checks."""
        pred = self.predict(feats)
        return [math.log(tc) + p[1] - p[0] for tc, p in zip(true_costs, pred)]

    def save(self, path: str) -> None:
        json.dump({"feature_dim": FEATURE_DIM, "targets": self.TARGETS, "hidden": self.hidden, "seed": self.seed,
                   "xm": self.xm.tolist(), "xs": self.xs.tolist(), "ym": self.ym.tolist(),
                   "ys": self.ys.tolist(), "params": self.mlp.params().tolist()}, open(path, "w"))

    @classmethod
    def load(cls, path: str) -> "CostModel":
        d = json.load(open(path))
        assert d["feature_dim"] == FEATURE_DIM, "model was trained on another feature set"
        assert d.get("targets") == cls.TARGETS, "model was trained on other targets"
        m = cls(d["seed"], d["hidden"])
        m.xm, m.xs = np.array(d["xm"]), np.array(d["xs"])
        m.ym, m.ys = np.array(d["ym"]), np.array(d["ys"])
        m.mlp = MLP(FEATURE_DIM, 2, d["hidden"], d["seed"])
        m.mlp.set_params(np.array(d["params"], dtype=np.float32))
        return m


def split_ks(ks, held_out: int = 40, seed: int = 0):
    rng = np.random.default_rng(seed)
    ks = sorted(ks)
    test = sorted(int(x) for x in rng.choice(ks, size=held_out, replace=False))
    return [k for k in ks if k not in test], test


# The analytic veto: the learned planner departs from the analytic planner's choice only when the
# network predicts at least this much less time for its own choice (log scale, 5 %); otherwise the
# analytic choice stands.
VETO_LOG_MARGIN = math.log(1.05)


def _analytic_evals(rates) -> float:
    """Expected filter evaluations per candidate of a cascade with these conditional pass rates
    (the analytic per-candidate cost: W = 10 + 8 * evaluations int32 ops, sieve/gpu_sieve_v9.py:25)."""
    total, alive = 0.0, 1.0
    for r in rates:
        total += alive
        alive *= r
    return total


def evaluate(rows, model: CostModel, test_ks, margin: float = VETO_LOG_MARGIN) -> dict:
    """Held-out comparison of the learned and the analytic planner, with an ablation of what the
    network adds over fixed order families."""
    by_k = {}
    for r in rows:
        if r["k"] in test_ks:
            by_k.setdefault(r["k"], []).append(r)
    # the analytic model's rate: the geometric-mean throughput of the model's training set
    mean_tp = math.exp(float(model.ym[0]))
    per_k, err_l, err_a, speed, plan_family = {}, [], [], [], {}
    for k, cand in sorted(by_k.items()):
        actual = [c["log_pos"] - c["log_tp"] for c in cand]            # ln(time) up to a constant
        pred_l = model.log_time([c["features"] for c in cand], [c["true_cost"] for c in cand])
        pred_a = [math.log(c["true_cost"]) - math.log(mean_tp) for c in cand]
        for a, pl, pa in zip(actual, pred_l, pred_a):
            err_l.append(abs(pl - a))
            err_a.append(abs(pa - a))
        ref = [i for i, c in enumerate(cand) if c["ref_order"]]
        ia = min(ref, key=lambda i: cand[i]["true_cost"])             # analytic planner's choice
        il = min(range(len(cand)), key=lambda i: pred_l[i])           # learned choice
        if pred_l[il] > pred_l[ia] - margin:                          # analytic veto
            il = ia
        ib = min(range(len(cand)), key=lambda i: actual[i])           # best measured
        s = math.exp(actual[ia] - actual[il])
        speed.append(s)
        # ablation of the plan choice: the analytic planner's wheel run with each fixed order
        # family (the family's order of that wheel, found among the probes by its order)
        aw = cand[ia]["wheel"]
        by_order = {tuple(c["order"]): i for i, c in enumerate(cand) if c["wheel"] == aw}
        for name, order in _orders(es_plan.Plan(k, None, aw), np.random.default_rng(0), shuffles=0, unique=False):
            j = by_order.get(tuple(order))
            if j is not None:
                plan_family.setdefault(name, {})[k] = math.exp(actual[ia] - actual[j])
        per_k[k] = {"analytic": f"{cand[ia]['wheel_name']}/{cand[ia]['order_name']}",
                    "learned": f"{cand[il]['wheel_name']}/{cand[il]['order_name']}",
                    "best": f"{cand[ib]['wheel_name']}/{cand[ib]['order_name']}",
                    "time_ratio_analytic_over_learned": s,
                    "time_ratio_analytic_over_best": math.exp(actual[ia] - actual[ib]),
                    "analytic_gcand": cand[ia]["gcand"], "learned_gcand": cand[il]["gcand"]}
    geo = math.exp(statistics.fmean(math.log(x) for x in speed)) if speed else None
    # fixed-scope scans (fixed positions, the default wheel): the learned order's measured
    # throughput against the reference order's; positions are equal, so time ratio = rate ratio.
    # Ablation: every order family on its own (the same family for every k), the family the
    # analytic model prefers (fewest expected filter evaluations per candidate), and the best
    # family in hindsight, against the network's per-k choice.
    fixed, family = [], {}
    for k, cand in sorted(by_k.items()):
        dw = [c for c in cand if c["wheel_name"] == "default"]
        ref = [c for c in dw if c["ref_order"]]
        if not dw or not ref:
            continue
        pred = model.predict([c["features"] for c in dw])
        ir = dw.index(ref[0])
        il = max(range(len(dw)), key=lambda i: pred[i][0])
        if pred[il][0] < pred[ir][0] + margin:                        # analytic veto
            il = ir
        fixed.append(dw[il]["gcand"] / ref[0]["gcand"])
        per_k[k]["fixed_scope_learned_order"] = dw[il]["order_name"]
        per_k[k]["fixed_scope_time_ratio"] = fixed[-1]
        # each named family's order for this wheel (families that coincide with an earlier one
        # were probed once, under the earlier name) mapped to the probe of that order
        by_order = {tuple(c["order"]): c for c in dw}
        P = es_plan.Plan(k, None, dw[0]["wheel"])
        for name, order in _orders(P, np.random.default_rng(0), shuffles=0, unique=False):
            c = by_order.get(tuple(order))
            if c is not None:
                family.setdefault(name, {})[k] = c["gcand"] / ref[0]["gcand"]
        if "rates" in dw[0]:
            ia = min(range(len(dw)), key=lambda i: _analytic_evals(dw[i]["rates"]))
            family.setdefault("analytic-model-choice", {})[k] = dw[ia]["gcand"] / ref[0]["gcand"]
    geo_fixed = math.exp(statistics.fmean(math.log(x) for x in fixed)) if fixed else None
    n_fixed = len(fixed)

    def geomean(v):
        return math.exp(statistics.fmean(math.log(x) for x in v)) if v else None
    families = {name: geomean(list(v.values())) for name, v in family.items() if len(v) == n_fixed}
    fixed_only = {n: g for n, g in families.items() if n != "analytic-model-choice"}
    best_family = max(fixed_only, key=fixed_only.get) if fixed_only else None
    plan_families = {name: geomean(list(v.values())) for name, v in plan_family.items() if len(v) == len(speed)}
    best_plan_family = max(plan_families, key=plan_families.get) if plan_families else None
    return {"held_out_k": sorted(by_k), "n_candidates": sum(len(v) for v in by_k.values()),
            "fixed_scope_geomean_time_ratio_reference_over_learned_order": geo_fixed,
            "fixed_scope_ablation": {
                "geomean_time_ratio_reference_over_family": families,
                "best_fixed_family": best_family,
                "network_over_best_fixed_family": (geo_fixed / fixed_only[best_family]
                                                   if best_family and geo_fixed else None),
                "network_over_analytic_model_choice": (geo_fixed / families["analytic-model-choice"]
                                                       if geo_fixed and families.get("analytic-model-choice")
                                                       else None)},
            "plan_choice_ablation": {
                "geomean_time_ratio_analytic_over_analytic_wheel_with_family": plan_families,
                "best_fixed_family": best_plan_family,
                "network_over_best_fixed_family": (geo / plan_families[best_plan_family]
                                                   if best_plan_family and geo else None)},
            "veto_log_margin": margin,
            "mae_log_time_learned": statistics.fmean(err_l) if err_l else None,
            "mae_log_time_analytic": statistics.fmean(err_a) if err_a else None,
            "geomean_time_ratio_analytic_over_learned": geo,
            "min_time_ratio": min(speed) if speed else None, "per_k": per_k}


def learned_order(model: CostModel, plan, seed: int = 0, margin: float = VETO_LOG_MARGIN) -> tuple[str, list[int]]:
    """Cascade order of one wheel with the least predicted time among the order families the
    model was trained on (a fixed-scope scan has fixed positions, so this is the fastest order).
    The analytic (reference) order stands unless the network predicts at least ``margin`` (log)
    more throughput for its choice."""
    rng = np.random.default_rng(seed)
    cands = [(n, o) for n, o in _orders(plan, rng, shuffles=0)]
    pred = model.predict([features(plan.with_order(o)) for _, o in cands])
    best = max(range(len(cands)), key=lambda i: pred[i][0])   # same wheel: same positions
    ref = next(i for i, (n, _) in enumerate(cands) if n == "reference")
    if pred[best][0] < pred[ref][0] + margin:
        best = ref
    return cands[best]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n-k", type=int, default=200)
    ap.add_argument("--held-out", type=int, default=40)
    ap.add_argument("--dataset", default=None, help="probe rows (JSON); collected when missing")
    ap.add_argument("--out", default=None)
    ap.add_argument("--epochs", type=int, default=600)
    ap.add_argument("--save-model", default=None, help="write the trained model (JSON) here")
    ap.add_argument("--eval-model", default=None,
                    help="score this trained model on the held-out k only (probes just those k)")
    a = ap.parse_args()
    rng = np.random.default_rng(0)
    ks = sorted(int(x) for x in rng.choice(np.arange(100, 401), size=a.n_k, replace=False))
    t0 = time.time()
    if a.eval_model:
        _, test_ks = split_ks(ks, a.held_out)
        rows = collect(test_ks, log=lambda s: print(s, file=sys.stderr, flush=True))
        if a.dataset:
            json.dump(rows, open(a.dataset, "w"))
        rep = evaluate(rows, CostModel.load(a.eval_model), set(test_ks))
        rep.update({"rows": len(rows), "probe_s": time.time() - t0, "model": a.eval_model})
        s = json.dumps(rep)
        if a.out:
            open(a.out, "w").write(s + "\n")
        print(s)
        return
    if a.dataset and os.path.exists(a.dataset):
        rows = json.load(open(a.dataset))
    else:
        rows = collect(ks, log=lambda s: print(s, file=sys.stderr, flush=True))
        if a.dataset:
            json.dump(rows, open(a.dataset, "w"))
    t_probe = time.time() - t0
    train_ks, test_ks = split_ks(ks, a.held_out)
    model = CostModel(0)
    t1 = time.time()
    loss = model.fit([r for r in rows if r["k"] in set(train_ks)], epochs=a.epochs)
    t_train = time.time() - t1
    rep = evaluate(rows, model, set(test_ks))
    if a.save_model:
        model.save(a.save_model)
    rep.update({"rows": len(rows), "probe_s": t_probe, "train_s": t_train, "train_loss": loss,
                "epochs": a.epochs, "k_range": [min(ks), max(ks)]})
    s = json.dumps(rep)
    if a.out:
        open(a.out, "w").write(s + "\n")
    print(s)


if __name__ == "__main__":
    main()
