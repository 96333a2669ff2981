"""Pins of the radiance-cache oracle (oracle/nrc.py) on the CPU: the spherical harmonics
are orthonormal over the sphere, trilinear corner weights sum to one, BF16 rounding is
round-to-nearest-even, and with BF16 rounding switched off the oracle's analytic weight
gradient matches central finite differences of its loss."""
import numpy as np

from oracle import nrc as ON


def test_sh_orthonormal():
    rng = np.random.default_rng(0)
    d = rng.normal(size=(400000, 3))
    y = ON.sh16(d.astype(np.float32)).astype(np.float64)
    gram = y.T @ y * (4 * np.pi / len(d))
    assert np.allclose(gram, np.eye(16), atol=2e-2)


def test_corner_weights_and_bf16():
    rng = np.random.default_rng(1)
    p = rng.uniform(0, 1, (1000, 3)).astype(np.float32)
    res, strides = ON.levels()
    for l in (0, 7, 15):
        idx, w = ON.corners(p, l, res, strides)
        assert np.allclose(w.sum(1), 1, atol=1e-5)
        assert (idx >= l * ON.TABLE).all() and (idx < (l + 1) * ON.TABLE).all()
    # ulp(1) = 2^-7 in BF16: halfway cases go to the even mantissa
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 0.75 * 2 ** -7, 1.0078125 + 2 ** -9, 1.0078125 + 2 ** -8], np.float32)
    assert list(ON.bf16(x)) == [1.0, 1.0, 1.0078125, 1.0078125, 1.015625]


def test_oracle_gradient_matches_finite_differences(monkeypatch):
    # without BF16 rounding the analytic weight gradient is the derivative of the loss with
    # the denominator y^2 + eps held at its current value (the loss's stop-gradient)
    monkeypatch.setattr(ON, "bf16", lambda x: np.asarray(x, np.float32))
    rng = np.random.default_rng(2)
    n = 64
    s = np.zeros((n, 16), np.float32)
    s[:, 0:3] = rng.uniform(-1, 1, (n, 3))
    s[:, 3:9] = rng.normal(size=(n, 6))
    s[:, 9:16] = rng.uniform(0, 1, (n, 7))
    w = rng.uniform(-0.3, 0.3, 22528).astype(np.float32)
    h = rng.uniform(-0.5, 0.5, ON.LEVELS * ON.TABLE * 2).astype(np.float32)
    lo, hi = [-1, -1, -1], [1, 1, 1]
    _, gw, _, y0 = ON.loss_and_grads(s, w, h, lo, hi)
    x0, _ = ON.encode(s[:, :13], h, lo, hi)
    den = 1.0 / (y0[:, :3].astype(np.float64) ** 2 + float(ON.REL_EPS))

    def frozen_loss(wv):
        _, y = ON.forward(x0, wv)
        d = y[:, :3].astype(np.float64) - s[:, 13:16]
        return float(np.sum(d * d * den) / n)
    for i in rng.choice(np.flatnonzero(np.abs(gw) > 1e-2), 8, replace=False):
        e = 1e-3
        wp, wm = w.copy(), w.copy()
        wp[i] += e
        wm[i] -= e
        fd = (frozen_loss(wp) - frozen_loss(wm)) / (float(wp[i]) - float(wm[i]))
        assert abs(fd - gw[i]) < 2e-2 * abs(gw[i]) + 1e-4, (i, fd, gw[i])
