"""The NumPy denoiser oracle's backward pass against finite differences of
its own forward pass (exact FP64, BF16 rounding switched off)."""
import numpy as np

import dn_ref as R


def test_oracle_backward_matches_finite_differences():
    R.ROUND = False
    try:
        rng = np.random.default_rng(0)
        specs, tensors = R.layer_specs()
        convs = [s for s in specs if s[0] == "conv"]
        params = []
        for s in convs:
            cin, cout = s[5], s[7]
            params.append((rng.normal(0, np.sqrt(2.0 / (9 * cin)), (cout, 9, cin)), rng.normal(0, 0.05, cout)))
        x = np.zeros((1, 16, 16, 16))
        x[..., :10] = rng.random((1, 16, 16, 10))
        r = rng.normal(size=(1, 16, 16, 8))
        r[..., 3:] = 0.0

        def loss(ps):
            return float((R.forward(x, ps)[-1] * r).sum())

        T = R.forward(x, params)
        grads, _ = R.backward(T, params, r)
        for li, kind, idx in [(0, "W", (3, 4, 2)), (5, "W", (7, 1, 20)), (9, "b", (11,)), (12, "W", (5, 8, 100)),
                              (16, "W", (1, 0, 50)), (18, "W", (2, 7, 31)), (18, "b", (1,))]:
            h = 1e-6
            pp = [(W.copy(), b.copy()) for W, b in params]
            pm = [(W.copy(), b.copy()) for W, b in params]
            (pp[li][0] if kind == "W" else pp[li][1])[idx] += h
            (pm[li][0] if kind == "W" else pm[li][1])[idx] -= h
            fd = (loss(pp) - loss(pm)) / (2 * h)
            an = (grads[li][0] if kind == "W" else grads[li][1])[idx]
            assert abs(fd - an) <= 1e-5 * max(abs(an), 1e-3), (li, kind, idx, fd, an)
    finally:
        R.ROUND = True


def test_oracle_loss_gradient_and_demodulation():
    """The training loss's gradient in the network's output (demodulated
    log1p radiance) against central differences, and pack/unpack as inverse
    albedo modulations."""
    rng = np.random.default_rng(1)
    h, w = 6, 5
    aov = rng.random((1, h, w, 12))
    aov[..., 7] = (rng.random((1, h, w)) < 0.7).astype(np.float64)
    tgt = rng.exponential(0.6, (1, h, w, 3))
    out = np.zeros((1, h, w, 8))
    out[..., :3] = rng.uniform(0.05, 1.5, (1, h, w, 3))
    l0, g = R.l1_loss_grad(out, tgt, aov)
    for idx in [(0, 1, 2, 0), (0, 3, 4, 1), (0, 5, 0, 2), (0, 2, 2, 1)]:
        e = 1e-7
        op, om = out.copy(), out.copy()
        op[idx] += e
        om[idx] -= e
        fd = (R.l1_loss_grad(op, tgt, aov)[0] - R.l1_loss_grad(om, tgt, aov)[0]) / (2 * e)
        assert abs(fd - g[idx]) <= 1e-4 * abs(g[idx]) + 1e-9, (idx, fd, g[idx])
    rad = np.zeros((h, w, 4))
    rad[..., :3] = rng.exponential(0.6, (h, w, 3))
    m = R.demod(aov[0])
    assert np.all(m[aov[0, ..., 7] <= 0.5] == 1.0)
    R.ROUND = False
    try:
        x = R.pack(rad, aov[0])
        y = np.zeros((h, w, 8))
        y[..., :3] = x[..., :3]
        assert np.allclose(R.unpack(y, aov[0]), rad[..., :3], rtol=1e-12, atol=1e-12)
    finally:
        R.ROUND = True
