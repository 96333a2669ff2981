"""Oracle for the neural radiance cache (test infrastructure, not the product).

Restates the cache's mathematics in NumPy so that the GPU forward pass, loss and
gradients can be checked: the multiresolution hash-grid encoding (Instant-NGP's spatial
hash and trilinear interpolation over FP16 features), real spherical harmonics of bands
0..3, and the 80 -> 5 x 64 -> 16 ReLU MLP with the GPU's rounding points (BF16 weights,
BF16 layer inputs and BF16 pre-activation gradients, FP32 products accumulated in FP64
here), the relative L2 loss (y - t)^2 / (y^2 + 0.01) averaged over the batch, and the
weight / hash-feature gradients.
"""
from __future__ import annotations

import numpy as np

LEVELS, FEATURES, TABLE = 16, 2, 1 << 19
IN, WIDTH, OUT, LAYERS = 80, 64, 16, 6
REL_EPS = np.float32(1e-2)


def layer_shapes():
    return [(IN if l == 0 else WIDTH, OUT if l == LAYERS - 1 else WIDTH) for l in range(LAYERS)]


def split_weights(w: np.ndarray) -> list[np.ndarray]:
    out, o = [], 0
    for k, n in layer_shapes():
        out.append(w[o:o + k * n].reshape(k, n))
        o += k * n
    return out


def bf16(x: np.ndarray) -> np.ndarray:
    """Round float32 to bfloat16 (nearest, ties to even), returned as float32."""
    x = np.ascontiguousarray(x, np.float32)
    b = x.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32)


def levels():
    b = np.exp((np.log(4096.0) - np.log(16.0)) / (LEVELS - 1))
    res = [float(np.floor(16.0 * b ** l)) for l in range(LEVELS)]
    strides = [int(r) + 2 if (int(r) + 2) ** 3 <= TABLE else 0 for r in res]
    return np.array(res, np.float32), strides


def bbox_transform(lo, hi):
    lo, hi = np.asarray(lo, np.float32), np.asarray(hi, np.float32)
    ext = (hi - lo).astype(np.float32)
    bmin = (lo - np.float32(1e-3) * ext).astype(np.float32)
    inv = np.where(ext > 0, np.float32(1) / (ext * np.float32(1.002)), np.float32(1)).astype(np.float32)
    return bmin, inv


def corners(p: np.ndarray, l: int, res, strides):
    """Table indices (N, 8) and trilinear weights (N, 8) of level l."""
    x = (p * res[l]).astype(np.float32)
    f = np.floor(x)
    t = (x - f).astype(np.float32)
    i = f.astype(np.uint64)
    idx = np.zeros((len(p), 8), np.uint64)
    w = np.zeros((len(p), 8), np.float32)
    for c in range(8):
        cx, cy, cz = i[:, 0] + (c & 1), i[:, 1] + ((c >> 1) & 1), i[:, 2] + ((c >> 2) & 1)
        if strides[l]:
            s = np.uint64(strides[l])
            h = (cx + cy * s + cz * s * s) & np.uint64(0xFFFFFFFF)
        else:
            h = ((cx * np.uint64(1)) ^ ((cy * np.uint64(2654435761)) & np.uint64(0xFFFFFFFF)) ^
                 ((cz * np.uint64(805459861)) & np.uint64(0xFFFFFFFF)))
        idx[:, c] = (h & np.uint64(TABLE - 1)) + np.uint64(l * TABLE)
        wx = t[:, 0] if c & 1 else np.float32(1) - t[:, 0]
        wy = t[:, 1] if (c >> 1) & 1 else np.float32(1) - t[:, 1]
        wz = t[:, 2] if (c >> 2) & 1 else np.float32(1) - t[:, 2]
        w[:, c] = (wx * wy).astype(np.float32) * wz
    return idx, w


def sh16(d: np.ndarray) -> np.ndarray:
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    x, y, z = d[:, 0], d[:, 1], d[:, 2]
    xx, yy, zz = x * x, y * y, z * z
    return np.stack([
        np.full_like(x, 0.28209479177387814), -0.48860251190291987 * y, 0.48860251190291987 * z,
        -0.48860251190291987 * x, 1.0925484305920792 * x * y, -1.0925484305920792 * y * z,
        0.94617469575755997 * zz - 0.31539156525251999, -1.0925484305920792 * x * z,
        0.54627421529603959 * (xx - yy), 0.59004358992664352 * y * (-3 * xx + yy),
        2.8906114426405538 * x * y * z, 0.45704579946446572 * y * (1 - 5 * zz),
        0.3731763325901154 * z * (5 * zz - 3), 0.45704579946446572 * x * (1 - 5 * zz),
        1.4453057213202769 * z * (xx - yy), 0.59004358992664352 * x * (-xx + 3 * yy)], 1).astype(np.float32)


def encode(q: np.ndarray, hash_params: np.ndarray, lo, hi):
    """Inputs (N, 80) before BF16 rounding, plus the per-level corners for the gradient."""
    res, strides = levels()
    bmin, inv = bbox_transform(lo, hi)
    p = np.clip((q[:, 0:3] - bmin) * inv, 0, 1).astype(np.float32)
    table = hash_params.reshape(-1, 2).astype(np.float16).astype(np.float32)
    x = np.zeros((len(q), IN), np.float32)
    cs = []
    for l in range(LEVELS):
        idx, w = corners(p, l, res, strides)
        cs.append((idx, w))
        f = np.zeros((len(q), 2), np.float32)
        for c in range(8):
            f = (f + w[:, c:c + 1] * table[idx[:, c]]).astype(np.float32)
        x[:, 2 * l:2 * l + 2] = f
    x[:, 32:48] = sh16(q[:, 3:6])
    x[:, 48:64] = sh16(q[:, 6:9])
    x[:, 64:68] = q[:, 9:13]
    x[:, 68] = 1.0
    return x, cs


def forward(x0: np.ndarray, w: np.ndarray):
    """Layer inputs X_0..X_5 (BF16-rounded) and the FP32 outputs (N, 16)."""
    ws = [bf16(m).astype(np.float64) for m in split_weights(w)]
    xs = [bf16(x0)]
    for l in range(LAYERS):
        y = (xs[-1].astype(np.float64) @ ws[l]).astype(np.float32)
        if l < LAYERS - 1:
            xs.append(bf16(np.maximum(y, 0)))
        else:
            return xs, y


def loss_and_grads(samples: np.ndarray, w: np.ndarray, hash_params: np.ndarray, lo, hi):
    """Mean relative L2 loss, dW (flat, like the weights) and the dense hash gradient."""
    n = len(samples)
    x0, cs = encode(samples[:, :13], hash_params, lo, hi)
    xs, y = forward(x0, w)
    ws = [bf16(m).astype(np.float64) for m in split_weights(w)]
    t = samples[:, 13:16]
    den = (np.float32(1) / (y[:, :3] * y[:, :3] + REL_EPS)).astype(np.float32)
    diff = y[:, :3] - t
    loss = float(np.sum(diff * diff * den) / n)
    dy = np.zeros((n, OUT), np.float32)
    dy[:, :3] = np.float32(2) * diff * den * np.float32(1.0 / n)
    dy = bf16(dy)
    dws = [None] * LAYERS
    for l in range(LAYERS - 1, -1, -1):
        dws[l] = xs[l].astype(np.float64).T @ dy.astype(np.float64)
        dx = (dy.astype(np.float64) @ ws[l].T).astype(np.float32)
        if l > 0:
            dy = bf16(np.where(xs[l] > 0, dx, np.float32(0)))
        else:
            dx0 = dx
    dhash = np.zeros((LEVELS * TABLE, 2), np.float64)
    for l in range(LEVELS):
        idx, wt = cs[l]
        g = dx0[:, 2 * l:2 * l + 2].astype(np.float64)
        for c in range(8):
            np.add.at(dhash, idx[:, c].astype(np.int64), wt[:, c:c + 1].astype(np.float64) * g)
    return loss, np.concatenate([d.reshape(-1) for d in dws]), dhash.reshape(-1), y
