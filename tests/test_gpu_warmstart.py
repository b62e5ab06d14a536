"""GPU tests of the learned warm start inside the descent step: features,
the energy judge / fallback, the unchanged residual bar, and the gain of a
trained network over the plain inertial guess."""
import os

import numpy as np
import pytest

from phybs_gb300 import meshes as M
from phybs_gb300.solver import DescentSolver
from phybs_gb300.train_warmstart import box_scenario, residual_params, mean_edge
from phybs_gb300.warmstart import DEFAULT_MODEL, WarmStartModel, MLPTrainer

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    from phybs_gb300.build import build
    build()


def _pull_case(seed=123, n=(10, 10, 16)):
    rng = np.random.default_rng(seed)
    return box_scenario(rng, *n)


def test_features_match_definition():
    """Feature columns against a numpy evaluation of their definition."""
    m, x0, boundary = _pull_case()
    s = DescentSolver(m, positions=x0, params=residual_params())
    xs = [s.positions().astype(np.float64)]
    for f in range(3):
        boundary(s, f)
        s.step()
        xs.append(s.positions().astype(np.float64))
    feats, xin, scale = s.warm_start_features()
    v, vo = s.velocities()
    ell = mean_edge(m)
    h = 1 / 30
    free = m.pin_mask() == 0
    # s = (1 - damping) |d1| + |d1 - d2| + 1e-4 l from the last two displacements
    # (pinned nodes are prescribed between steps, so only free nodes follow the
    # recorded history)
    d1, d2 = xs[3] - xs[2], xs[2] - xs[1]
    ref_scale = 0.01 * np.linalg.norm(d1, axis=1) + np.linalg.norm(d1 - d2, axis=1) + 1e-4 * ell
    # |d1 - d2| from read-back FP32 positions carries their rounding (~1e-8 m)
    np.testing.assert_allclose(scale[free], ref_scale[free], rtol=1e-2, atol=1e-7 + 1e-6 * ell)
    sc = scale[:, None]
    np.testing.assert_allclose(feats[free, 0:3], (v * h / sc)[free], rtol=1e-4, atol=1e-4)
    np.testing.assert_allclose(feats[free, 3:6], (d1 / sc)[free], rtol=1e-3, atol=1e-3)
    np.testing.assert_allclose(feats[free, 6:9], (d2 / sc)[free], rtol=1e-3, atol=1e-3)
    np.testing.assert_allclose(feats[free, 9:12], (0.2 * h * (v - vo) / sc)[free], rtol=1e-3, atol=1e-4)
    x = s.positions()
    np.testing.assert_allclose(xin, x + h * v + 0.2 * h * (v - vo), atol=2e-6)
    # mean incident J - 1 at x~ = x + h v
    xt = (x + h * v).astype(np.float64)
    J = M.signed_volumes(xt, m.tets) / M.signed_volumes(m.rest, m.tets)
    acc = np.zeros(m.n_nodes)
    cnt = np.zeros(m.n_nodes)
    for c in range(4):
        np.add.at(acc, m.tets[:, c], J - 1)
        np.add.at(cnt, m.tets[:, c], 1)
    np.testing.assert_allclose(feats[:, 23], acc / cnt, atol=2e-5)
    s.close()


def test_zero_network_keeps_plain_result():
    """A network whose output is zero reproduces the plain guess: the step
    result equals the plain run bit for bit, and the residual reference is the
    plain guess's either way."""
    m, x0, boundary = _pull_case()
    theta = np.zeros(MLPTrainer(seed=0).n_params, np.float32)
    model = WarmStartModel(theta, np.zeros(24, np.float32), np.ones(24, np.float32), np.ones(3, np.float32))
    a = DescentSolver(m, positions=x0, params=residual_params())
    b = DescentSolver(m, positions=x0, params=residual_params())
    b.set_warm_start(model)
    for f in range(3):
        boundary(a, f)
        boundary(b, f)
        ia, ib = a.step(), b.step()
        assert ia == ib
        assert b.stats()["warm_start_used"] == 1
    assert np.array_equal(a.positions(), b.positions())
    a.close()
    b.close()


def test_zero_network_on_extrapolation_base_is_the_extrapolation():
    """With the extrapolation base (warm-start mode 2), a zero network's
    candidate is u0 + 2 d1 - d2.  After three plain steps, the next step equals
    the plain solver's started from that guess (pbs_set_guess) when the judge
    keeps it, and the plain step when the judge (energy not higher and, for
    this base, a smaller gradient norm) rejects it."""
    m, x0, boundary = _pull_case()
    theta = np.zeros(MLPTrainer(seed=0).n_params, np.float32)
    model = WarmStartModel(theta, np.zeros(24, np.float32), np.ones(24, np.float32), np.ones(3, np.float32),
                           base="extrapolation")
    sv = [DescentSolver(m, positions=x0, params=residual_params()) for _ in range(3)]
    hist = [sv[0].positions().astype(np.float64)] * 3
    free = m.pin_mask() == 0
    for f in range(3):
        for s in sv:
            boundary(s, f)
            s.step()
        hist = hist[1:] + [sv[0].positions().astype(np.float64)]
    plain, guessed, learned = sv
    learned.set_warm_start(model)
    for s in sv:
        boundary(s, 3)
    _, xin, _ = guessed.warm_start_features()
    guess = xin.copy()
    extrap = hist[-1] + 2.0 * (hist[-1] - hist[-2]) - (hist[-2] - hist[-3])
    guess[free] = extrap[free]
    guessed.set_guess(guess.astype(np.float32))
    ip, ig, il = plain.step(), guessed.step(), learned.step()
    used = learned.stats()["warm_start_used"]
    ref, iref = (guessed, ig) if used else (plain, ip)
    if used:
        assert guessed.stats()["warm_start_used"] == 1
    assert abs(il - iref) <= 2, (used, il, iref)  # the two guesses agree to FP32 rounding
    assert np.abs(learned.positions() - ref.positions()).max() <= 1e-5 * m.bbox_diagonal()
    for s in sv:
        s.close()


def test_bad_prediction_falls_back():
    """A network that predicts a large wrong correction raises the energy; the
    judge rejects it and the step equals the plain one."""
    m, x0, boundary = _pull_case()
    theta = np.zeros(MLPTrainer(seed=0).n_params, np.float32)
    # constant output bias: every free node moved by 2e4 motion scales (at least
    # two edge lengths, the scale being >= 1e-4 edge)
    theta[-3:] = 2e4
    model = WarmStartModel(theta, np.zeros(24, np.float32), np.ones(24, np.float32), np.ones(3, np.float32))
    a = DescentSolver(m, positions=x0, params=residual_params())
    b = DescentSolver(m, positions=x0, params=residual_params())
    b.set_warm_start(model)
    for f in range(2):
        boundary(a, f)
        boundary(b, f)
        assert a.step() == b.step()
        assert b.stats()["warm_start_used"] == 0
    assert np.array_equal(a.positions(), b.positions())
    a.close()
    b.close()


@pytest.mark.skipif(not os.path.exists(DEFAULT_MODEL), reason="no trained model committed")
def test_trained_network_gains_over_plain():
    """On a held-out pull scenario (a mesh seed not used in training; 51,200
    tets) the trained network cuts the iterations to the same residual bar by
    at least 8% over frames 2-11 (measured 1.125x: 4,571 against 5,143), is
    kept on at least half the frames, and both runs end within 1e-3 of the
    bbox diagonal of each other.  The step is bit-reproducible, so the gain
    is a fixed number for the committed model."""
    model = WarmStartModel.load(DEFAULT_MODEL)
    m, x0, boundary = _pull_case(seed=987654, n=(20, 20, 32))
    a = DescentSolver(m, positions=x0, params=residual_params())
    b = DescentSolver(m, positions=x0, params=residual_params())
    b.set_warm_start(model)
    ia, ib, used = [], [], 0
    for f in range(12):
        boundary(a, f)
        boundary(b, f)
        ia.append(a.step())
        ib.append(b.step())
        assert a.stats()["converged"] == 1 and b.stats()["converged"] == 1
        used += b.stats()["warm_start_used"]
    gain = sum(ia[2:]) / sum(ib[2:])
    print(f"held-out pull: iterations plain {ia}, warm-started {ib}; gain {gain:.3f}x on frames 2-11, "
          f"learned guess kept on {used} of 12")
    assert gain >= 1.08, (ia, ib)
    assert used >= 6
    assert np.abs(a.positions() - b.positions()).max() / m.bbox_diagonal() < 1e-3
    a.close()
    b.close()
