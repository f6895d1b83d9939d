"""GPU: the learned planner's CUDA MLP kernels against the numpy float64 restatement
(oracle/es_mlp_ref.py): forward outputs, loss and full gradient, and that training descends."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("D,H,O,n", [(32, 64, 2, 300), (7, 32, 3, 65), (64, 64, 2, 1000)])
def test_forward_and_gradient_match_cpu(native, D, H, O, n):
    import es_learned
    import es_mlp_ref as R
    rng = np.random.default_rng(D * 1000 + n)
    X = rng.normal(size=(n, D)).astype(np.float32)
    T = rng.normal(size=(n, O)).astype(np.float32)
    m = es_learned.MLP(D, O, H, seed=5)
    P = m.params()
    Y = m.forward(X)
    Yr, _ = R.forward(P, X, D, H, O)
    np.testing.assert_allclose(Y, Yr, rtol=1e-4, atol=1e-4)        # FP32 vs float64 forward
    loss, g = m.loss_grad(X, T)
    lr, gr = R.loss_grad(P, X, T, D, H, O)
    assert abs(loss - lr) <= 1e-4 * max(1.0, abs(lr))
    # gradient: FP32 sums over n samples -> relative tolerance on the vector norm + per entry
    assert np.linalg.norm(g - gr) <= 1e-4 * np.linalg.norm(gr) + 1e-7
    np.testing.assert_allclose(g, gr, rtol=2e-3, atol=1e-6)


def test_gradient_matches_finite_differences(native):
    import es_learned
    import es_mlp_ref as R
    rng = np.random.default_rng(3)
    D, H, O, n = 5, 32, 2, 40
    X = rng.normal(size=(n, D)).astype(np.float32)
    T = rng.normal(size=(n, O)).astype(np.float32)
    m = es_learned.MLP(D, O, H, seed=1)
    P = m.params().astype(np.float64)
    _, g = m.loss_grad(X, T)
    for i in rng.choice(P.size, size=12, replace=False):
        e = np.zeros_like(P)
        e[i] = 1e-5
        fd = (R.loss_grad(P + e, X, T, D, H, O)[0] - R.loss_grad(P - e, X, T, D, H, O)[0]) / 2e-5
        assert abs(fd - g[i]) <= 1e-3 * max(1e-3, abs(fd)) + 1e-6, i


def test_training_fits_a_smooth_function(native):
    import es_learned
    rng = np.random.default_rng(11)
    X = rng.uniform(-1, 1, size=(2048, 6)).astype(np.float32)
    T = np.stack([np.sin(2 * X[:, 0]) + X[:, 1] * X[:, 2], np.abs(X[:, 3]) - X[:, 4]], 1).astype(np.float32)
    m = es_learned.MLP(6, 2, 64, seed=0)
    l0, _ = m.loss_grad(X, T)
    l1 = m.train(X, T, epochs=300, batch=128, lr=3e-3, seed=0)
    assert l1 < 0.1 * l0
    # deterministic: the same seed gives bit-identical parameters
    m2 = es_learned.MLP(6, 2, 64, seed=0)
    m2.train(X, T, epochs=300, batch=128, lr=3e-3, seed=0)
    np.testing.assert_array_equal(m.params(), m2.params())
