"""FP64 numpy restatement of the rotation-proposal network (test infrastructure).

Checker only: tests and the smoke check compare the library's CUDA forward,
backward and input-binning kernels (emc_gb300/csrc/proposal.cu) against
these functions; nothing in the library calls them.  The reference has no
counterpart (parity unpinned by construction); the functions restate the
network from its mathematics:

* inputs: counts summed over b x b pixel blocks inside the mask (b = side /
  64, negative counts as 0), scaled so the pattern sums to 4096, log1p;
* four 3x3 convolutions, stride 2, padding 1, 64 channels, ReLU
  (64 -> 32 -> 16 -> 8 -> 4 pixels), weights [co][ci][3][3];
* linear head 1024 -> 6 over the [64][4][4] activations in memory order;
* loss per pattern min(|o - t|^2, |o + t|^2), t the first two columns of
  the label's rotation matrix, mean over the batch.

Parameters are one flat vector in the library's order: w0, b0, w1, b1, w2,
b2, w3, b3, fw, fb.
"""
from __future__ import annotations

import numpy as np

D, CH, NCONV, OUT = 64, 64, 4, 6
FC_IN = CH * 16


def cin(l):
    return 1 if l == 0 else CH


def layout():
    """(offset, shape) of every parameter block, in order."""
    out, o = [], 0
    for l in range(NCONV):
        for shape in ((CH, cin(l), 3, 3), (CH,)):
            out.append((o, shape))
            o += int(np.prod(shape))
    for shape in ((OUT, FC_IN), (OUT,)):
        out.append((o, shape))
        o += int(np.prod(shape))
    return out, o


def unpack(params):
    lay, total = layout()
    assert params.size == total
    return [np.asarray(params[o:o + int(np.prod(s))], np.float64).reshape(s) for o, s in lay]


def inputs(images, mask, side, stats=None):
    """[n][s*s] counts, [s*s] mask -> [n][64*64] network inputs (before the
    per-pixel standardisation when stats is None; else (X - mean) * inv)."""
    b = side // D
    im = np.where((mask[None, :] > 0) & (images > 0), images, 0).astype(np.float64)
    v = im.reshape(-1, D, b, D, b).sum(axis=(2, 4)).reshape(-1, D * D)
    scale = 4096.0 / np.maximum(v.sum(1, keepdims=True), 1.0)
    X = np.log1p(v * scale)
    if stats is not None:
        X = (X - stats[0][None, :]) * stats[1][None, :]
    return X


def input_stats(X):
    """Per-pixel mean and 1 / sqrt(var + 1e-4) of raw inputs X [n][4096]."""
    m = X.mean(0)
    var = np.maximum((X * X).mean(0) - m * m, 0.0)
    return np.stack([m, 1.0 / np.sqrt(var + 1e-4)])


def _cols(x):
    """x [B][C][H][H] -> im2col [B][C*9][Ho*Ho] for stride 2, padding 1."""
    B, C, H, _ = x.shape
    Ho = H // 2
    xp = np.zeros((B, C, H + 2, H + 2))
    xp[:, :, 1:-1, 1:-1] = x
    cols = np.empty((B, C, 9, Ho, Ho))
    for ky in range(3):
        for kx in range(3):
            cols[:, :, ky * 3 + kx] = xp[:, :, ky:ky + 2 * Ho:2, kx:kx + 2 * Ho:2]
    return cols.reshape(B, C * 9, Ho * Ho)


def _uncols(dc, C, H):
    """Adjoint of _cols: [B][C*9][Ho*Ho] -> [B][C][H][H]."""
    B = dc.shape[0]
    Ho = H // 2
    dc = dc.reshape(B, C, 9, Ho, Ho)
    xp = np.zeros((B, C, H + 2, H + 2))
    for ky in range(3):
        for kx in range(3):
            xp[:, :, ky:ky + 2 * Ho:2, kx:kx + 2 * Ho:2] += dc[:, :, ky * 3 + kx]
    return xp[:, :, 1:-1, 1:-1]


def forward(params, X):
    """X [B][4096] -> (o [B][6], cache)."""
    p = unpack(params)
    B = X.shape[0]
    a = X.reshape(B, 1, D, D).astype(np.float64)
    cache = []
    for l in range(NCONV):
        W, bias = p[2 * l], p[2 * l + 1]
        H = a.shape[2]
        cols = _cols(a)
        z = np.einsum("ok,bkn->bon", W.reshape(CH, -1), cols) + bias[None, :, None]
        out = np.maximum(z, 0.0)
        cache.append((a, cols, out))
        a = out.reshape(B, CH, H // 2, H // 2)
    h = a.reshape(B, FC_IN)
    o = h @ p[8].T + p[9]
    cache.append(h)
    return o, cache


def quat_to_6d(q):
    """Library convention (rotated = M p): first two columns of M."""
    a, b, c, d = (np.asarray(q, np.float64)[..., i] for i in range(4))
    m0 = a * a + b * b - c * c - d * d
    m1 = 2 * (b * c - a * d)
    m3 = 2 * (b * c + a * d)
    m4 = a * a - b * b + c * c - d * d
    m6 = 2 * (b * d - a * c)
    m7 = 2 * (c * d + a * b)
    return np.stack([m0, m3, m6, m1, m4, m7], -1)


def loss(o, t):
    dp = ((o - t) ** 2).sum(1)
    dm = ((o + t) ** 2).sum(1)
    s = np.where(dp <= dm, 1.0, -1.0)
    B = o.shape[0]
    return float(np.minimum(dp, dm).mean()), (2.0 / B) * (o - s[:, None] * t)


def loss_and_grads(params, X, quats):
    """Mean loss and d loss / d params (flat, library order)."""
    p = unpack(params)
    o, cache = forward(params, X)
    L, go = loss(o, quat_to_6d(quats))
    h = cache[-1]
    grads = [None] * len(p)
    grads[8] = go.T @ h
    grads[9] = go.sum(0)
    g = (go @ p[8]).reshape(X.shape[0], CH, 16)  # d loss / d act of the last conv
    for l in range(NCONV - 1, -1, -1):
        a, cols, out = cache[l]
        d = g.reshape(out.shape) * (out > 0)
        W = p[2 * l]
        grads[2 * l] = np.einsum("bon,bkn->ok", d, cols).reshape(W.shape)
        grads[2 * l + 1] = d.sum(axis=(0, 2))
        if l > 0:
            dc = np.einsum("ok,bon->bkn", W.reshape(CH, -1), d)
            g = _uncols(dc, a.shape[1], a.shape[2])
    return L, np.concatenate([gr.ravel() for gr in grads])


def six_d_to_quat(o):
    """Gram-Schmidt of [n][6] outputs to rotation quaternions (w >= 0)."""
    out = np.empty((o.shape[0], 4))
    for i, v in enumerate(np.asarray(o, np.float64)):
        a = v[:3] / np.linalg.norm(v[:3])
        b = v[3:] - (a @ v[3:]) * a
        b /= np.linalg.norm(b)
        c = np.cross(a, b)
        M = np.stack([a, b, c], 1)  # columns
        w = np.sqrt(max(0.0, 1.0 + np.trace(M))) / 2.0
        x = np.sqrt(max(0.0, 1.0 + M[0, 0] - M[1, 1] - M[2, 2])) / 2.0
        y = np.sqrt(max(0.0, 1.0 - M[0, 0] + M[1, 1] - M[2, 2])) / 2.0
        z = np.sqrt(max(0.0, 1.0 - M[0, 0] - M[1, 1] + M[2, 2])) / 2.0
        x = np.copysign(x, M[2, 1] - M[1, 2])
        y = np.copysign(y, M[0, 2] - M[2, 0])
        z = np.copysign(z, M[1, 0] - M[0, 1])
        q = np.array([w, x, y, z])
        out[i] = q / np.linalg.norm(q)
    return out


def turn(X, k):
    """[n][4096] inputs turned in-plane by k quarter turns, the way the
    library's batch gather does it: one turn takes out[y][x] = in[63 - x][y]."""
    img = np.asarray(X).reshape(-1, D, D)
    return np.rot90(img, -k, axes=(1, 2)).reshape(-1, D * D)


def turn_6d(t, k):
    """6D labels composed with Rz(-90 deg) k times: (c1, c2) -> (-c2, c1) per turn."""
    t = np.asarray(t, np.float64).copy()
    for _ in range(k % 4):
        t = np.concatenate([-t[..., 3:], t[..., :3]], -1)
    return t


def friedel_mate(q):
    """q (x) (0, 0, 0, 1): the rotation followed by a half turn about the beam axis."""
    q = np.asarray(q, np.float64)
    m = np.stack([-q[..., 3], q[..., 2], -q[..., 1], q[..., 0]], -1)
    return np.where(m[..., :1] < 0, -m, m)
