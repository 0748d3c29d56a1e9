"""ORACLE — test infrastructure only.

FP64 numpy restatement of the learned multilevel preconditioner network
(architecture in include/sfx_learned.h): forward pass, loss and the gradient
with respect to every parameter, used to check the project's BF16
tensor-core training and inference kernels.  Only tests/ import this module.

Volumes are numpy arrays (nz, ny, nx, C); parameters follow the library's
flat layout: per convolution W[cout][27][cin] then b[cout];
tap = (dz + 1) * 9 + (dy + 1) * 3 + (dx + 1).
"""
from __future__ import annotations

import numpy as np

SPEC = [(16, 16, True), (16, 16, True), (16, 32, True), (32, 32, True), (32, 48, True), (48, 48, True),
        (48, 48, True), (48, 32, True), (32, 16, True), (16, 16, True), (16, 16, False)]
A0, B0L, A1, B1L, A2, B2L, A3, U2, U1, U0, OUTL = range(11)
TAPS = [(t % 3 - 1, (t // 3) % 3 - 1, t // 9 - 1) for t in range(27)]  # (dx, dy, dz)


def num_params():
    return sum(co * 27 * ci + co for ci, co, _ in SPEC)


def unpack(p):
    out, off = [], 0
    for ci, co, _ in SPEC:
        W = p[off:off + co * 27 * ci].reshape(co, 27, ci)
        off += co * 27 * ci
        b = p[off:off + co]
        off += co
        out.append((W.astype(np.float64), b.astype(np.float64)))
    return out


def _shift(x, dx, dy, dz):
    """y[z, y, x] = x[z + dz, y + dy, x + dx] with zeros outside."""
    nz, ny, nx = x.shape[:3]
    y = np.zeros_like(x)
    zs, ze = max(0, -dz), min(nz, nz - dz)
    ys, ye = max(0, -dy), min(ny, ny - dy)
    xs, xe = max(0, -dx), min(nx, nx - dx)
    y[zs:ze, ys:ye, xs:xe] = x[zs + dz:ze + dz, ys + dy:ye + dy, xs + dx:xe + dx]
    return y


def conv(x, W, b):
    y = np.zeros(x.shape[:3] + (W.shape[0],))
    for t, (dx, dy, dz) in enumerate(TAPS):
        y += _shift(x, dx, dy, dz) @ W[:, t, :].T
    return y + b


def conv_bwd(x, W, gz):
    """Gradients of y = conv(x) given gz = dL/dy: (gx, gW, gb)."""
    gx = np.zeros_like(x)
    gW = np.zeros_like(W)
    gzf = gz.reshape(-1, gz.shape[-1])
    for t, (dx, dy, dz) in enumerate(TAPS):
        xs = _shift(x, dx, dy, dz)
        gW[:, t, :] = gzf.T @ xs.reshape(-1, xs.shape[-1])
        gx += _shift(gz @ W[:, t, :], -dx, -dy, -dz)
    return gx, gW, gz.sum(axis=(0, 1, 2))


def _r1(m_fine):
    m = (m_fine + 1) // 2
    R = np.zeros((m, m_fine))
    for X in range(m):
        R[X, 2 * X] = 1.0
        if 2 * X - 1 >= 0:
            R[X, 2 * X - 1] = 0.5
        if 2 * X + 1 < m_fine:
            R[X, 2 * X + 1] = 0.5
    return R


def restrict(f, scale=0.125):
    Rz, Ry, Rx = _r1(f.shape[0]), _r1(f.shape[1]), _r1(f.shape[2])
    return scale * np.einsum("Zz,Yy,Xx,zyxc->ZYXc", Rz, Ry, Rx, f, optimize=True)


def prolong(c, fine_shape, scale=1.0):
    Rz, Ry, Rx = _r1(fine_shape[0]), _r1(fine_shape[1]), _r1(fine_shape[2])
    return scale * np.einsum("Zz,Yy,Xx,ZYXc->zyxc", Rz, Ry, Rx, c, optimize=True)


def relu(x):
    return np.maximum(x, 0.0)


def pack(r, feat, shape):
    """Input volume and scale s from byNODES residual r (3N) and features (2N)."""
    N = int(np.prod(shape))
    s = np.sqrt(np.sum(r.astype(np.float64) ** 2) / (3 * N))
    s = s if s > 0 else 1.0
    x = np.zeros(tuple(shape) + (16,))
    for c in range(3):
        x[..., c] = r[c * N:(c + 1) * N].reshape(shape) / s
    x[..., 3] = feat[:N].reshape(shape)
    x[..., 4] = feat[N:].reshape(shape)
    return x, s


def forward(params, x):
    P = unpack(params)
    a = {}
    a["A0"] = relu(conv(x, *P[A0]))
    a["B0"] = relu(conv(a["A0"], *P[B0L]))
    a["C1"] = restrict(a["B0"])
    a["A1"] = relu(conv(a["C1"], *P[A1]))
    a["B1"] = relu(conv(a["A1"], *P[B1L]))
    a["C2"] = restrict(a["B1"])
    a["A2"] = relu(conv(a["C2"], *P[A2]))
    a["B2"] = relu(conv(a["A2"], *P[B2L]))
    a["C3"] = restrict(a["B2"])
    a["A3"] = relu(conv(a["C3"], *P[A3]))
    a["D2"] = prolong(a["A3"], a["B2"].shape[:3]) + a["B2"]
    a["E2"] = relu(conv(a["D2"], *P[U2]))
    a["D1"] = prolong(a["E2"], a["B1"].shape[:3]) + a["B1"]
    a["E1"] = relu(conv(a["D1"], *P[U1]))
    a["D0"] = prolong(a["E1"], a["B0"].shape[:3]) + a["B0"]
    a["E0"] = relu(conv(a["D0"], *P[U0]))
    a["OUT"] = conv(a["E0"], *P[OUTL])
    return a


def loss_and_grad(params, r, target, feat, shape):
    """Normalised loss and its gradient w.r.t. the flat parameter vector."""
    x, s = pack(r, feat, shape)
    N = int(np.prod(shape))
    P = unpack(params)
    a = forward(params, x)
    mask = feat[N:].reshape(shape) > 0.5
    t = np.stack([target[c * N:(c + 1) * N].reshape(shape) / s for c in range(3)], axis=-1)
    t[mask] = 0.0
    tt = np.sum(t ** 2)
    d = a["OUT"][..., :3] - t
    d[mask] = 0.0
    loss = np.sum(d ** 2) / tt
    g = {k: None for k in range(11)}
    gOUT = np.zeros_like(a["OUT"])
    gOUT[..., :3] = 2.0 * d / tt

    def back(layer, xin, y, gy, relu_on=True):
        gz = gy * (y > 0) if relu_on else gy
        gx, gW, gb = conv_bwd(xin, P[layer][0], gz)
        g[layer] = (gW, gb)
        return gx

    gE0 = back(OUTL, a["E0"], None, gOUT, relu_on=False)
    gD0 = back(U0, a["D0"], a["E0"], gE0)
    gB0 = gD0.copy()
    gE1 = restrict(gD0, scale=1.0)
    gD1 = back(U1, a["D1"], a["E1"], gE1)
    gB1 = gD1.copy()
    gE2 = restrict(gD1, scale=1.0)
    gD2 = back(U2, a["D2"], a["E2"], gE2)
    gB2 = gD2.copy()
    gA3 = restrict(gD2, scale=1.0)
    gC3 = back(A3, a["C3"], a["A3"], gA3)
    gB2 += prolong(gC3, a["B2"].shape[:3], scale=0.125)
    gA2 = back(B2L, a["A2"], a["B2"], gB2)
    gC2 = back(A2, a["C2"], a["A2"], gA2)
    gB1 += prolong(gC2, a["B1"].shape[:3], scale=0.125)
    gA1 = back(B1L, a["A1"], a["B1"], gB1)
    gC1 = back(A1, a["C1"], a["A1"], gA1)
    gB0 += prolong(gC1, a["B0"].shape[:3], scale=0.125)
    gA0 = back(B0L, a["A0"], a["B0"], gB0)
    back(A0, x, a["A0"], gA0)
    flat = np.concatenate([np.concatenate([g[l][0].ravel(), g[l][1].ravel()]) for l in range(11)])
    return loss, flat, a, s


def apply(params, r, feat, shape):
    """z = s NN(r/s) with zeros on masked nodes (byNODES, 3N)."""
    x, s = pack(r, feat, shape)
    N = int(np.prod(shape))
    out = forward(params, x)["OUT"]
    mask = (feat[N:] > 0.5)
    z = np.zeros(3 * N)
    for c in range(3):
        zc = s * out[..., c].ravel()
        zc[mask] = 0.0
        z[c * N:(c + 1) * N] = zc
    return z
