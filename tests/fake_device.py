"""CPU stand-ins for the device half of the engine (es_native.Context / es_native.Batch), backed
by the C oracle, so that the host logic of es_gb300 -- and the reference's own drivers on top of
it -- run without a GPU.  Test infrastructure only: the product path never imports this."""
import numpy as np


class FakeCtx:
    """Stands in for es_native.Context; every launch scans its outer range with the C oracle."""

    def __init__(self, plan, capacity=1 << 20, plant=None):
        import es_oracle as O
        self.plan, self.capacity, self.plant = plan, capacity, plant
        self.T = O.CTables(plan)
        self.r0 = plan.radix[0] if plan.radix else 1
        self.n_outer = plan.R // self.r0
        self.n_filters = len(plan.rest)
        self.t, self.surv = 0, []
        self.launches = 0

    def set_block(self, t, tconst=None):
        self.t = int(t)

    def reset(self):
        self.surv = []

    def launch(self, ostart, ocount):
        import es_oracle as O
        if ostart + ocount > self.n_outer:
            raise ValueError("outer range outside [0, R/r0)")
        s, _, _ = O.scan_c(self.T, self.t, o_range=(ostart, ostart + ocount), threads=2)
        self.surv.extend(s)
        self.launches += 1
        if self.plant is not None and ostart == 0:
            self.surv.append(self.plant)

    def count(self):
        return len(self.surv)

    def survivors(self, n=None):
        if len(self.surv) > self.capacity:
            raise RuntimeError("overflow")
        out = np.array(self.surv, dtype=np.uint64)
        return out if n is None else out[:n]


class FakeBatch:
    """Stands in for es_native.Batch: the blocks of one search group, least good (t, s)."""

    def __init__(self, ctxs, items, tune=None):
        self.ctx, self.items = ctxs[0], items

    def run(self, use_graph=False):
        from es_plan import is_admissible
        self.best = None
        for (_, _, t, ob, oe) in self.items:
            self.ctx.set_block(t)
            self.ctx.reset()
            self.ctx.launch(ob, oe - ob)
            P = self.ctx.plan
            good = [n for n in (P.idx_to_n(int(i), t) for i in self.ctx.surv)
                    if n > P.k + 1 and is_admissible(n, P.k)]
            if good:
                self.best = (t, min(good) - t * P.M)
                return

    def group_min(self, g):
        return self.best

    def close(self):
        pass


def install(monkeypatch, plant=None, cap=None):
    """Route every es_gb300 device context and batch through the fakes; returns the list of
    contexts created, in order."""
    import es_gb300
    made = []

    def make_ctx(plan, tune=None, capacity=None):
        c = FakeCtx(plan, cap if cap is not None else (capacity or 1 << 20), plant)
        made.append(c)
        return c
    monkeypatch.setattr(es_gb300.N, "Context", make_ctx)
    monkeypatch.setattr(es_gb300.N, "Batch", FakeBatch)
    return made
