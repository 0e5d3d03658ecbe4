"""Host side of the inverse fitter: its Adam is the reference optimizer's
rule (ohao/inverse/optimizer.hpp:26-39: beta1 0.9, beta2 0.999, eps 1e-8,
bias-corrected moments, projection onto the parameter box after each step).
No GPU: the gradient is supplied directly."""
import math

import numpy as np

from ohao_engine_gb300.fit import Adam


def scalar_adam(theta, grads, lr, lo, hi, b1=0.9, b2=0.999, eps=1e-8):
    """The update written out per coordinate, one step per gradient."""
    theta = list(theta)
    m = [0.0] * len(theta)
    v = [0.0] * len(theta)
    for t, g in enumerate(grads, start=1):
        for i in range(len(theta)):
            m[i] = b1 * m[i] + (1 - b1) * g[i]
            v[i] = b2 * v[i] + (1 - b2) * g[i] * g[i]
            mh = m[i] / (1 - b1 ** t)
            vh = v[i] / (1 - b2 ** t)
            theta[i] = min(max(theta[i] - lr * mh / (math.sqrt(vh) + eps), lo[i]), hi[i])
    return np.array(theta)


def test_adam_matches_the_scalar_rule():
    rng = np.random.default_rng(3)
    n = 17
    theta0 = rng.uniform(0.2, 0.8, n)
    lo, hi = np.zeros(n), np.ones(n)
    grads = [rng.normal(0, 10 ** rng.uniform(-4, 1), n) for _ in range(12)]
    a = Adam(n)
    th = theta0.copy()
    for g in grads:
        th = a.step(th, g, 0.02, lo, hi)
    assert np.allclose(th, scalar_adam(theta0, grads, 0.02, lo, hi), rtol=0, atol=1e-12)
    assert a.t == len(grads)


def test_first_step_moves_by_lr_against_the_gradient_sign():
    a = Adam(4)
    th = a.step(np.full(4, 0.5), np.array([3.0, -2e-3, 1e-2, -50.0]), 0.05, np.zeros(4), np.ones(4))
    assert np.allclose(th, [0.45, 0.55, 0.45, 0.55], atol=1e-6)


def test_projection_onto_the_box():
    a = Adam(3)
    lo, hi = np.array([0.05, 0.0, 0.0]), np.array([1.0, 1.0, 0.3])
    th = np.array([0.06, 0.99, 0.29])
    for _ in range(20):
        th = a.step(th, np.array([1.0, -1.0, -1.0]), 0.1, lo, hi)
        assert np.all(th >= lo) and np.all(th <= hi)
    assert np.array_equal(th, [0.05, 1.0, 0.3])


def test_converges_on_a_quadratic():
    target = np.array([0.3, 0.5, 0.7, 0.9])
    a = Adam(4)
    th = np.full(4, 0.5)
    for _ in range(400):
        th = a.step(th, 2 * (th - target), 0.01, np.full(4, 0.05), np.ones(4))
    assert np.abs(th - target).max() < 2e-3
