"""Oracle (test infrastructure only): float64 restatement of the neural
radiance cache's encoding, forward pass, relative L2 loss and gradients, used
to check the fused GPU kernels' inference output and gradients.

The model follows the published methods the GPU code states (Mueller et al.
2021, neural radiance caching: relative L2 loss (o - y)^2 / (sg(o)^2 + 0.01);
Mueller et al. 2022, multiresolution hash encoding with primes 1,
2654435761, 805459861 and trilinear interpolation), with this project's
configuration: 16 levels x 2 features, 2^19 entries per level, encoding
columns [hash grid 0..31 | SH degree 3 of the direction 32..47 | normal
48..50 | roughness 51 | albedo 52..54 | 1 at 55 | 0], 4 hidden 64-wide ReLU
layers and a 16-wide output layer (3 used), no biases.

The grid cell of a position is computed in float32 with one rounding per
operation, as the GPU does, so both sides interpolate the same table entries;
everything after that is float64.
"""
import numpy as np

LEVELS, FEAT, T = 16, 2, 1 << 19
WIDTH, HIDDEN, OUT_PAD = 64, 4, 16
NUM_W = HIDDEN * WIDTH * WIDTH + WIDTH * OUT_PAD
OUT_OFF = HIDDEN * WIDTH * WIDTH


def split_weights(w):
    """[W0..W3 (64x64), W4 (64x16)], each [in][out], float64."""
    w = np.asarray(w, np.float64)
    mats = [w[l * WIDTH * WIDTH:(l + 1) * WIDTH * WIDTH].reshape(WIDTH, WIDTH) for l in range(HIDDEN)]
    mats.append(w[OUT_OFF:].reshape(WIDTH, OUT_PAD))
    return mats


def sh_encode(d):
    x, y, z = d[:, 0], d[:, 1], d[:, 2]
    xx, yy, zz = x * x, y * y, z * z
    return np.stack([
        np.full_like(x, 0.28209479177387814),
        -0.48860251190291987 * y, 0.48860251190291987 * z, -0.48860251190291987 * x,
        1.0925484305920792 * x * y, -1.0925484305920792 * y * z, 0.94617469575755997 * zz - 0.31539156525251999,
        -1.0925484305920792 * x * z, 0.54627421529603959 * (xx - yy),
        0.59004358992664352 * y * (-3.0 * xx + yy), 2.8906114426405538 * x * y * z,
        0.45704579946446572 * y * (1.0 - 5.0 * zz), 0.3731763325901154 * z * (5.0 * zz - 3.0),
        0.45704579946446572 * x * (1.0 - 5.0 * zz), 1.4453057213202769 * z * (xx - yy),
        0.59004358992664352 * x * (-xx + 3.0 * yy)], axis=1)


def cells(rec, grid, level):
    """corner table indices (n, 8) and trilinear weights (n, 8) at a level."""
    p = np.asarray(rec[:, :3], np.float32)
    lo = np.asarray(grid["lo"], np.float32)
    inv = np.float32(grid["inv_extent"])
    u = np.clip((p - lo) * inv, np.float32(0), np.float32(1)).astype(np.float32)
    q = (u * np.float32(grid["scales"][level])).astype(np.float32) + np.float32(0.5)
    q = q.astype(np.float32)
    c0 = np.floor(q)
    f = (q - c0).astype(np.float64)
    c0 = c0.astype(np.uint64)
    side = int(grid["dense"][level])
    idx = np.zeros((len(rec), 8), np.uint64)
    wts = np.zeros((len(rec), 8))
    for k in range(8):
        dx, dy, dz = k & 1, (k >> 1) & 1, k >> 2
        x, y, z = c0[:, 0] + dx, c0[:, 1] + dy, c0[:, 2] + dz
        if side:
            idx[:, k] = x + side * (y + side * z)
        else:
            m = np.uint64(0xffffffff)
            h = (x * np.uint64(1)) & m ^ (y * np.uint64(2654435761)) & m ^ (z * np.uint64(805459861)) & m
            idx[:, k] = h & np.uint64(T - 1)
        wx = f[:, 0] if dx else 1.0 - f[:, 0]
        wy = f[:, 1] if dy else 1.0 - f[:, 1]
        wz = f[:, 2] if dz else 1.0 - f[:, 2]
        wts[:, k] = wx * wy * wz
    return idx, wts


def encode(rec, grid, table):
    """encoding (n, 64) and the per-level (indices, weights) for the backward."""
    n = len(rec)
    tab = np.asarray(table, np.float64).reshape(LEVELS, T, FEAT)
    X = np.zeros((n, WIDTH))
    geo = []
    for l in range(LEVELS):
        idx, wts = cells(rec, grid, l)
        geo.append((idx, wts))
        feats = tab[l][idx.astype(np.int64)]  # (n, 8, 2)
        X[:, 2 * l:2 * l + 2] = np.einsum("nk,nkf->nf", wts, feats)
    X[:, 32:48] = sh_encode(np.asarray(rec[:, 3:6], np.float64))
    X[:, 48:51] = rec[:, 6:9]
    X[:, 51] = rec[:, 9]
    X[:, 52:55] = rec[:, 10:13]
    X[:, 55] = 1.0
    return X, geo


def forward(rec, grid, weights, table):
    X, geo = encode(rec, grid, table)
    W = split_weights(weights)
    acts = [X]
    a = X
    for l in range(HIDDEN):
        a = np.maximum(a @ W[l], 0.0)
        acts.append(a)
    out = a @ W[HIDDEN]
    return out[:, :3], acts, geo


def loss_and_gradients(rec, grid, weights, table, den=None):
    """mean relative L2 loss over the 3 channels and its gradients:
    (loss, weight gradient (NUM_W,), table gradient (LEVELS*T*FEAT,)).
    The denominator sg(o)^2 + 0.01 is a constant of the gradient; `den`
    freezes it (n x 3) to evaluate the same surrogate at other parameters."""
    n = len(rec)
    o3, acts, geo = forward(rec, grid, weights, table)
    W = split_weights(weights)
    y = np.asarray(rec[:, 13:16], np.float64)
    if den is None:
        den = o3 * o3 + 0.01
    diff = o3 - y
    loss = float(np.sum(diff * diff / den) / (3 * n))
    dO = np.zeros((n, OUT_PAD))
    dO[:, :3] = 2.0 * diff / den / (3 * n)
    grads = [None] * (HIDDEN + 1)
    grads[HIDDEN] = acts[HIDDEN].T @ dO
    dA = dO @ W[HIDDEN].T
    for l in range(HIDDEN - 1, -1, -1):
        dZ = dA * (acts[l + 1] > 0)
        grads[l] = acts[l].T @ dZ
        dA = dZ @ W[l].T
    wgrad = np.concatenate([g.reshape(-1) for g in grads])
    tgrad = np.zeros((LEVELS, T, FEAT))
    for l in range(LEVELS):
        idx, wts = geo[l]
        d = dA[:, 2 * l:2 * l + 2]
        for k in range(8):
            np.add.at(tgrad[l], idx[:, k].astype(np.int64), wts[:, k:k + 1] * d)
    return loss, wgrad, tgrad.reshape(-1)


def make_grid(lo, hi, base_res=16, max_res=2048.0):
    """the grid parameters for a bounding box: levels N_l = base * b^l up to
    max_res, scale N_l - 1, dense side ceil(N_l) + 1 when its cube fits T."""
    lo = np.asarray(lo, np.float32)
    ext = float(np.max(np.asarray(hi, np.float32) - lo))
    b = np.exp(np.log(max_res / base_res) / (LEVELS - 1))
    scales = np.zeros(LEVELS, np.float32)
    dense = np.zeros(LEVELS, np.uint32)
    for l in range(LEVELS):
        N = base_res * b ** l
        scales[l] = np.float32(N - 1.0)
        side = np.ceil(N) + 1.0
        dense[l] = np.uint32(side) if side ** 3 <= T else 0
    return dict(lo=lo, inv_extent=float(np.float32(1.0) / np.float32(ext)), scales=scales, dense=dense)
