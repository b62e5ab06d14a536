"""GPU checks of the warm-start network's tensor-core kernels against the FP64
oracle (oracle/mlp.py): forward, parameter gradients, Adam, and training."""
import numpy as np
import pytest

from oracle import mlp as OM
from phybs_gb300.warmstart import MLPTrainer

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    from phybs_gb300.build import build
    build()


def _data(n, seed=0):
    rng = np.random.default_rng(seed)
    X = rng.normal(0.0, 1.0, (n, 24)).astype(np.float32)
    Y = np.stack([np.sin(X[:, 0]) + 0.5 * X[:, 1] * X[:, 2], np.tanh(X[:, 3] - X[:, 4]), 0.3 * X[:, 5] ** 2 - 0.2],
                 axis=1).astype(np.float32)
    return X, Y


def test_param_count_matches_oracle():
    t = MLPTrainer(seed=1)
    assert t.n_params == OM.N_PARAMS == 10115
    t.close()


def test_forward_matches_oracle():
    theta = OM.init_params(3).astype(np.float32)
    t = MLPTrainer(theta)
    X, _ = _data(1000, 1)
    y = t.forward(X)
    ref, _ = OM.forward(theta, X, round_bf16=True)
    ref64, _ = OM.forward(theta, X, round_bf16=False)
    scale = np.abs(ref).max()
    assert np.abs(y - ref).max() / scale < 2e-2
    # the BF16 network against the all-FP64 one, stated as a bound
    assert np.abs(y - ref64).max() / np.abs(ref64).max() < 5e-2
    t.close()


@pytest.mark.parametrize("n", [37, 300, 4096])
def test_gradient_matches_oracle(n):
    """Every parameter block's gradient against the FP64 backward with the
    kernels' BF16 operand rounding: relative error of the block norm < 5e-3
    (measured 2.2e-3 at most, on the 37-sample batch), cosine > 0.999."""
    theta = OM.init_params(5).astype(np.float32)
    t = MLPTrainer(theta)
    X, Y = _data(n, 2)
    loss, g = t.gradient(X, Y)
    lref, gref = OM.loss_and_grad(theta, X, Y, round_bf16=True)
    assert abs(loss - lref) / lref < 1e-2
    off = 0
    errs = []
    for o, i in OM.SIZES:
        for sz in (o * i, o):
            a, b = g[off:off + sz].astype(np.float64), gref[off:off + sz]
            off += sz
            nb = np.linalg.norm(b)
            errs.append(np.linalg.norm(a - b) / nb)
            assert np.linalg.norm(a - b) / nb < 5e-3, (off, np.linalg.norm(a - b) / nb)
            assert a @ b / (np.linalg.norm(a) * nb) > 0.999
    print(f"n={n}: per-block gradient error {[f'{e:.1e}' for e in errs]}")
    t.close()


def test_adam_step_matches_oracle():
    theta = OM.init_params(7).astype(np.float32)
    t = MLPTrainer(theta)
    X, Y = _data(512, 3)
    _, g = t.gradient(X, Y)
    t.set_data(X, Y)
    t.train(1, batch=512, lr=1e-3, seed=0)
    new = t.params.astype(np.float64)
    ref, _, _ = OM.adam(theta.astype(np.float64), np.zeros_like(new), np.zeros_like(new), g.astype(np.float64), 1, 1e-3)
    assert np.abs(new - ref).max() < 1e-6 + 1e-5 * np.abs(ref).max()
    t.close()


def test_weighted_adam_step_matches_oracle():
    """With per-sample loss weights, one full-batch Adam step moves every
    parameter by -lr * sign of the FP64 weighted gradient (Adam's first step),
    wherever that gradient is clearly non-zero."""
    theta = OM.init_params(9).astype(np.float32)
    t = MLPTrainer(theta)
    X, Y = _data(512, 5)
    W = np.random.default_rng(6).uniform(0.0, 4.0, 512).astype(np.float32)
    t.set_data(X, Y, W)
    lr = 1e-3
    t.train(1, batch=512, lr=lr, seed=0)
    step = t.params.astype(np.float64) - theta
    _, g = OM.loss_and_grad(theta, X, Y, round_bf16=True, W=W)
    clear = np.abs(g) > 1e-2 * np.abs(g).max()
    assert clear.sum() > 1000
    np.testing.assert_allclose(step[clear], -lr * np.sign(g[clear]), rtol=1e-2, atol=1e-6)
    _, g_unw = OM.loss_and_grad(theta, X, Y, round_bf16=True)
    assert (np.sign(g_unw[clear]) != np.sign(g[clear])).any()  # the weights changed the step
    t.close()


def test_training_reduces_loss():
    t = MLPTrainer(seed=11)
    X, Y = _data(20000, 4)
    t.set_data(X, Y)
    losses = t.train(400, batch=1024, lr=2e-3, seed=1)
    assert losses[-20:].mean() < 0.25 * losses[:5].mean(), (losses[:5], losses[-20:])
    t.close()
