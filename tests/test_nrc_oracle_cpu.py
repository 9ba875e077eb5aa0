"""The radiance-cache oracle checked on its own (no GPU): its analytic
gradients equal central finite differences of its loss (with the loss's
stop-gradient denominator held at the base point), for weights of every
layer and for hash-table entries, and its grid follows the level schedule
(16 -> 2048, dense levels while the grid fits the table)."""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import nrc as ref  # noqa: E402


def _setup(n=64, seed=0):
    rng = np.random.default_rng(seed)
    rec = np.zeros((n, 16))
    rec[:, 0:3] = rng.random((n, 3)) * 2 - 1
    d = rng.normal(size=(n, 3))
    rec[:, 3:6] = d / np.linalg.norm(d, axis=1, keepdims=True)
    nn = rng.normal(size=(n, 3))
    rec[:, 6:9] = nn / np.linalg.norm(nn, axis=1, keepdims=True)
    rec[:, 9:13] = rng.random((n, 4))
    rec[:, 13:16] = rng.random((n, 3))
    w = rng.uniform(-1, 1, ref.NUM_W) * np.sqrt(6.0 / 128.0)
    t = rng.uniform(-0.5, 0.5, ref.LEVELS * ref.T * ref.FEAT)
    return rec.astype(np.float32), w, t, ref.make_grid((-1, -1, -1), (1, 1, 1))


def test_grid_schedule():
    g = ref.make_grid((0, 0, 0), (2, 1, 1))
    assert abs(g["inv_extent"] - 0.5) < 1e-7
    assert abs(g["scales"][0] - 15.0) < 1e-5 and abs(g["scales"][-1] - 2047.0) < 1e-2
    assert g["dense"][0] == 17 and g["dense"][-1] == 0
    assert all(np.diff(g["scales"]) > 0)


def test_oracle_gradients_equal_finite_differences():
    rec, w, t, grid = _setup()
    loss, gw, gt = ref.loss_and_gradients(rec, grid, w, t)
    o3 = ref.forward(rec, grid, w, t)[0]
    den = o3 * o3 + 0.01

    def L(wx, tx):
        return ref.loss_and_gradients(rec, grid, wx, tx, den=den)[0]
    rng = np.random.default_rng(1)
    eps = 1e-6
    for l in range(5):
        lo = l * 4096
        hi = lo + (4096 if l < 4 else 1024)
        idx = rng.choice(np.arange(lo, hi)[np.abs(gw[lo:hi]) > 1e-9], 3, replace=False)
        for i in idx:
            wp, wm = w.copy(), w.copy()
            wp[i] += eps
            wm[i] -= eps
            fd = (L(wp, t) - L(wm, t)) / (2 * eps)
            assert abs(fd - gw[i]) < 1e-4 * max(1.0, abs(gw[i])) + 1e-7, (l, i, fd, gw[i])
    touched = np.nonzero(gt)[0]
    for i in rng.choice(touched, 4, replace=False):
        tp, tm = t.copy(), t.copy()
        tp[i] += eps
        tm[i] -= eps
        fd = (L(w, tp) - L(w, tm)) / (2 * eps)
        assert abs(fd - gt[i]) < 1e-4 * max(1.0, abs(gt[i])) + 1e-7, (i, fd, gt[i])
