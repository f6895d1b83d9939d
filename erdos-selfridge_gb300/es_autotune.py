"""Autotuner for the scan kernel's launch shape and table layout.

Chooses, per plan (or per batch), the fastest of: threads per CTA, strip depth (at most `strip`
ring-1 cycles per lane per work unit: one balanced window of ring-2 digits), the table layout
(word masks or pair tables, through L1 or staged in shared memory, or scalar) and the number of
filters evaluated in the inner-ring stage.  None of
these changes which candidates pass; the tuner only times.  Search: coordinate descent from the
default shape over one parameter at a time, each candidate timed with CUDA events on a probe
range (median of a few launches).  Results are cached in a JSON file keyed by the plan (k,
wheel, filter order) and the engine (a hash of the library's bytes, the device's name and SM
count), so a plan is tuned once per library build and GPU model.
"""
from __future__ import annotations

import hashlib
import json
import os
import statistics

import es_native as N

SPACE = {
    "threads": [256, 384, 512],
    "strip": [2, 4, 8, 16],
    "mask_filters": [2, 3, 4, 5, 6],
    "layout": [N.LAYOUT_WORDMASK, N.LAYOUT_PAIR, N.LAYOUT_SMEM, N.LAYOUT_SMEM_PAIR, N.LAYOUT_AUTO, N.LAYOUT_SCALAR],
}
DEFAULT = dict(layout=N.LAYOUT_WORDMASK, mask_filters=4, threads=512, strip=8, smem_kb=0,
               ctas_per_sm=4, count_stages=0)


def engine_signature() -> str:
    """What a cached shape was measured on: the engine library's bytes and the device's name and
    SM count.  A rebuilt kernel or another GPU model gets its own cache entries."""
    h = hashlib.sha256()
    with open(N.LIB_PATH, "rb") as f:
        for chunk in iter(lambda: f.read(1 << 20), b""):
            h.update(chunk)
    info = N.device_info()
    return f"{h.hexdigest()[:16]}|{info.get('name', '?')}|{info['sm_count']}"


def plan_signature(plan) -> str:
    """Cache key of a plan's tuned shape: the plan (k, wheel, cascade order) and the engine."""
    key = json.dumps({"k": plan.k, "wheel": [[p, T] for p, T in plan.wheel], "rest": plan.rest,
                      "engine": engine_signature()})
    return hashlib.sha256(key.encode()).hexdigest()[:16]


def default_cache_path() -> str:
    base = os.environ.get("XDG_CACHE_HOME") or os.path.join(os.path.expanduser("~"), ".cache")
    return os.path.join(base, "es_gb300", "tune.json")


def _load(path):
    try:
        with open(path) as f:
            return json.load(f)
    except Exception:
        return {}


def _save(path, data):
    os.makedirs(os.path.dirname(path), exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(data, f, indent=1)
    os.replace(tmp, path)


def time_ctx(ctx: N.Context, tune: dict, n_outer: int, reps: int = 3) -> float:
    """Median ms of `reps` launches over outer indices [0, n_outer) with this shape."""
    ctx.set_tune(N.make_tune(**tune))
    ctx.reset()
    ctx.launch_timed(0, n_outer)          # warm-up (tables into L1/L2)
    ms = []
    for _ in range(reps):
        ctx.reset()
        ms.append(ctx.launch_timed(0, n_outer))
    return statistics.median(ms)


def tune_plan(plan, ctx: N.Context | None = None, probe_log2: int = 28, cache: str | None = None,
              space: dict | None = None, log=None) -> dict:
    """Best shape for one plan (coordinate descent, cached)."""
    cache = cache or default_cache_path()
    sig = plan_signature(plan)
    data = _load(cache)
    if sig in data:
        return dict(data[sig]["tune"])
    own = ctx is None
    start = dict(DEFAULT, layout=N.layout_for_plan(plan, DEFAULT["mask_filters"]))
    if own:
        ctx = N.Context(plan, N.make_tune(**start))
    r0 = plan.radix[0] if plan.radix else 1
    n_outer = max(1, min(ctx.n_outer, (1 << probe_log2) // r0))
    ctx.set_block(0)
    best = dict(start)
    best_ms = time_ctx(ctx, best, n_outer)
    tried = {json.dumps(best, sort_keys=True): best_ms}
    space = space or SPACE
    improved = True
    while improved:
        improved = False
        for key, values in space.items():
            for v in values:
                cand = dict(best, **{key: v})
                if cand["layout"] == N.LAYOUT_SCALAR and cand["mask_filters"] > 4:
                    continue
                ck = json.dumps(cand, sort_keys=True)
                if ck in tried:
                    continue
                ms = time_ctx(ctx, cand, n_outer)
                tried[ck] = ms
                if log:
                    log(f"tune {plan.k}: {cand} {ms:.3f} ms")
                if ms < best_ms * 0.98:
                    best, best_ms, improved = cand, ms, True
    ctx.set_tune(N.make_tune(**best))
    data[sig] = {"tune": best, "ms": best_ms, "probe_positions": n_outer * r0, "k": plan.k}
    _save(cache, data)
    if own:
        ctx.close()
    return best


def tune_batch(ctxs, items, space: dict | None = None, reps: int = 3, log=None,
               start: dict | None = None) -> tuple[dict, float]:
    """Best shape for one persistent batch, timing the batch itself (graph replay), by coordinate
    descent from `start` (DEFAULT when not given)."""
    space = space or SPACE
    best, best_ms = dict(start or DEFAULT), None
    tried = {}

    def run(t):
        b = N.Batch(ctxs, items, N.make_tune(**t))
        try:
            b.run(use_graph=True)
            b.sync()
            ms = []
            for _ in range(reps):
                b.run(use_graph=True)
                ms.append(b.sync())
            return statistics.median(ms)
        finally:
            b.close()

    best_ms = run(best)
    tried[json.dumps(best, sort_keys=True)] = best_ms
    improved = True
    while improved:
        improved = False
        for key, values in space.items():
            for v in values:
                cand = dict(best, **{key: v})
                if cand["layout"] == N.LAYOUT_SCALAR and cand["mask_filters"] > 4:
                    continue
                ck = json.dumps(cand, sort_keys=True)
                if ck in tried:
                    continue
                ms = run(cand)
                tried[ck] = ms
                if log:
                    log(f"tune batch: {cand} {ms:.3f} ms")
                if ms < best_ms * 0.98:
                    best, best_ms, improved = cand, ms, True
    return best, best_ms
