"""GPU: what the trained cost model gains over the analytic planner.

A seeded campaign (56 k in 100..400, every candidate plan probed on 2^26 positions of block 0)
is collected on the GPU, the MLP is trained by the library's CUDA kernels on 48 k, and on the
8 held-out k its time prediction error is compared with the analytic model's (expected checks
at the mean training rate).  The packaged model (trained on 160 k) is scored on k it was not
trained on, both for prediction error and for the measured time to completion of the plans it
chooses against the analytic planner's choices."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_learned_model_beats_analytic_on_held_out_k(native):
    import es_learned
    es_learned.PROBE_LOG2 = 26
    rng = np.random.default_rng(7)
    ks = sorted(int(x) for x in rng.choice(np.arange(100, 401), size=56, replace=False))
    rows = es_learned.collect(ks, procs=12)
    assert len(rows) > 56 * 20
    train, test = es_learned.split_ks(ks, held_out=8, seed=1)
    model = es_learned.CostModel(0)
    model.fit([r for r in rows if r["k"] in set(train)], epochs=600)
    rep = es_learned.evaluate(rows, model, set(test))
    # a model trained on 48 k already predicts time-to-completion better than the analytic
    # estimate; choosing plans reliably better needs the full campaign (next test)
    assert rep["mae_log_time_learned"] < 0.8 * rep["mae_log_time_analytic"], rep


def test_packaged_model_on_unseen_k(native):
    """The committed model (trained on 160 k of the seeded 100..400 campaign) on fresh probes of
    k from that campaign's held-out set: better time predictions than the analytic model, and
    plans that finish faster than the analytic planner's."""
    import es_learned
    es_learned.PROBE_LOG2 = 28
    model = es_learned.CostModel.load(es_learned.MODEL_PATH)
    held = [103, 186, 264, 311, 350, 384]          # held out of the packaged model's training
    rows = es_learned.collect(held, procs=12)
    rep = es_learned.evaluate(rows, model, set(held))
    assert rep["mae_log_time_learned"] < 0.7 * rep["mae_log_time_analytic"], rep
    # the campaign that trained the model measured 1.26x (geomean over these six k) for the
    # plans the network picks against the analytic planner's; 1.08 leaves room for probe noise
    assert rep["geomean_time_ratio_analytic_over_learned"] >= 1.08, rep


def test_packaged_model_orders_are_permutations(native):
    """The committed model loads, runs on the GPU and proposes valid cascade orders."""
    import os
    import es_gb300
    import es_learned
    path = os.path.join(os.path.dirname(es_learned.__file__), "data", "cost_model.json")
    model = es_learned.CostModel.load(path)
    for k in (150, 300, 390):
        P = es_gb300.Plan(k)
        name, order = es_learned.learned_order(model, P)
        assert sorted(order) == sorted(P.rest)
        pred = model.predict([es_learned.features(P)])
        assert np.all(np.isfinite(pred))
