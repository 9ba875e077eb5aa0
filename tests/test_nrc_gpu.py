"""Neural radiance cache kernels against the float64 oracle (oracle/nrc.py).

The fused kernels run the MLP in BF16 on the tensor cores with FP32
accumulation and keep activations in BF16; the oracle runs the same model in
float64 on the same parameters (weights BF16-representable, table entries
FP16-representable) and the same grid cells.  So: inference outputs agree to
a few percent of their scale, gradients of every weight matrix and of the
touched table entries agree in direction (cosine > 0.995) and norm (within
5 %), the losses within 2 %; and training on a smooth radiance field lowers
the loss by more than 10x."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import nrc as ref  # noqa: E402

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _records(n, seed, target=None):
    rng = np.random.default_rng(seed)
    rec = np.zeros((n, 16), np.float32)
    rec[:, 0:3] = rng.random((n, 3)) * 2.0 - 1.0
    d = rng.normal(size=(n, 3))
    rec[:, 3:6] = d / np.linalg.norm(d, axis=1, keepdims=True)
    nn = rng.normal(size=(n, 3))
    rec[:, 6:9] = nn / np.linalg.norm(nn, axis=1, keepdims=True)
    rec[:, 9] = rng.random(n)
    rec[:, 10:13] = rng.random((n, 3))
    if target is not None:
        rec[:, 13:16] = target(rec)
    return rec


def _bf16(a):
    return (np.asarray(a, np.float32).view(np.uint32) & np.uint32(0xffff0000)).view(np.float32)


def _cache(b200_device, seed=3):
    import ospray_gb300 as og
    c = og.RadianceCache(b200_device, (-1, -1, -1), (1, 1, 1), learning_rate=1e-2, seed=seed)
    rng = np.random.default_rng(seed)
    w = _bf16(rng.uniform(-1, 1, ref.NUM_W) * np.sqrt(6.0 / 128.0))
    t = rng.uniform(-0.5, 0.5, ref.LEVELS * ref.T * ref.FEAT).astype(np.float16).astype(np.float32)
    c.set_params(w, t)
    return c, w, t


def _target(rec):
    p, d = rec[:, 0:3], rec[:, 3:6]
    return np.stack([0.6 + 0.4 * np.sin(3 * p[:, 0]) * np.cos(2 * p[:, 1]),
                     0.5 + 0.3 * np.cos(2 * p[:, 2] + d[:, 1]),
                     0.4 + 0.3 * p[:, 1] * d[:, 2]], axis=1).astype(np.float32)


def test_inference_matches_oracle(b200_device):
    c, w, t = _cache(b200_device)
    rec = _records(2000, 1)
    q = torch.from_numpy(rec).cuda()
    out = torch.zeros((len(rec), 3), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    c.infer(q.data_ptr(), len(rec), out.data_ptr())
    b200_device.sync()
    got = out.cpu().numpy()
    g, r = c.grid(), ref.make_grid((-1, -1, -1), (1, 1, 1))
    np.testing.assert_allclose(g["scales"], r["scales"], rtol=1e-6)
    np.testing.assert_array_equal(g["dense"], r["dense"])
    assert g["inv_extent"] == r["inv_extent"]
    exp, _, _ = ref.forward(rec, g, w, t)
    scale = np.abs(exp).max()
    assert np.abs(got - exp).max() < 0.03 * scale
    assert np.linalg.norm(got - exp) < 0.02 * np.linalg.norm(exp)


def test_gradients_match_oracle(b200_device):
    c, w, t = _cache(b200_device, seed=5)
    rec = _records(512, 2, _target)
    s = torch.from_numpy(rec).cuda()
    wg = torch.zeros(ref.NUM_W, dtype=torch.float32, device="cuda")
    tg = torch.zeros(ref.LEVELS * ref.T * ref.FEAT, dtype=torch.float32, device="cuda")
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    c.gradients(s.data_ptr(), len(rec), wg.data_ptr(), tg.data_ptr(), loss.data_ptr())
    b200_device.sync()
    rloss, rw, rt = ref.loss_and_gradients(rec, c.grid(), w, t)
    assert abs(float(loss.item()) - rloss) < 0.02 * rloss
    gw = wg.cpu().numpy().astype(np.float64)
    offs = [0, 4096, 8192, 12288, 16384, ref.NUM_W]
    for l in range(5):
        a, b = gw[offs[l]:offs[l + 1]], rw[offs[l]:offs[l + 1]]
        cos = a @ b / (np.linalg.norm(a) * np.linalg.norm(b))
        assert cos > 0.995, (l, cos)
        assert abs(np.linalg.norm(a) / np.linalg.norm(b) - 1.0) < 0.05, l
    gt = tg.cpu().numpy().astype(np.float64)
    touched = rt != 0
    assert touched.sum() > 1000
    a, b = gt[touched], rt[touched]
    assert a @ b / (np.linalg.norm(a) * np.linalg.norm(b)) > 0.995
    assert abs(np.linalg.norm(a) / np.linalg.norm(b) - 1.0) < 0.05
    assert np.all(gt[~touched] == 0.0)


def test_training_reduces_loss(b200_device):
    import ospray_gb300 as og
    c = og.RadianceCache(b200_device, (-1, -1, -1), (1, 1, 1), learning_rate=1e-2, seed=7)
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    losses = []
    for step in range(300):
        rec = _records(16384, 100 + step, _target)
        s = torch.from_numpy(rec).cuda()
        torch.cuda.synchronize()
        c.train(s.data_ptr(), len(rec), loss.data_ptr())
        b200_device.sync()
        losses.append(float(loss.item()))
    assert np.isfinite(losses).all()
    assert np.mean(losses[-20:]) < 0.1 * np.mean(losses[:5])
