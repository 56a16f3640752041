"""FP64 numpy restatement of the learned-coefficient network's forward pass,
operator-space loss and gradient, used to check the GPU training kernels.

TEST INFRASTRUCTURE ONLY.  Parameter layout (flat, as the GPU keeps it):
W1[64][3], b1[64], W2[64][64], b2[64], W3[16][64], b3[16]; tanh hidden
layers; inputs normalised as (x - in_mean)/in_scale; outputs are normalised
coefficients (c - out_mean)/out_scale; the loss compares operators (FD
symbols), see loss_and_grad.
"""
from __future__ import annotations

import numpy as np

NI, NH, NO = 3, 64, 16


def unpack(p):
    p = np.asarray(p, np.float64)
    o = 0
    out = []
    for shape in ((NH, NI), (NH,), (NH, NH), (NH,), (NO, NH), (NO,)):
        k = int(np.prod(shape))
        out.append(p[o:o + k].reshape(shape))
        o += k
    return out


def loss_and_grad(params, norm, x, c):
    """(loss, flat gradient) in FP64.  norm = (in_mean, in_scale, out_mean,
    out_scale); x [n,3] with x[:,1] = kh_max, x[:,2] = M; c [n,16].

    Loss: mean over samples and over kh = u*bb (u = 1/8..1), theta in
    {0, pi/12, pi/6, pi/4} of ((S_net - S_opt) / (kh^2/4))^2 with the FD symbol
    S = sum_{l<=M} c_l (sin^2(l kh cos th/2) + sin^2(l kh sin th/2))."""
    W1, b1, W2, b2, W3, b3 = unpack(params)
    in_mean, in_scale, out_mean, out_scale = [np.asarray(a, np.float64) for a in norm]
    x = np.asarray(x, np.float64)
    t = (np.asarray(c, np.float64) - out_mean) / out_scale
    n = len(x)
    M = np.minimum(x[:, 2].astype(int), NO)
    bb = x[:, 1]
    mask = (np.arange(NO)[None, :] < M[:, None]).astype(np.float64)
    xi = (x - in_mean) / in_scale
    h1 = np.tanh(xi @ W1.T + b1)
    h2 = np.tanh(h1 @ W2.T + b2)
    y = h2 @ W3.T + b3
    dc = (y - t) * out_scale * mask                     # [n, NO]
    u = np.arange(1, 9) / 8.0
    th = np.arange(4) * (np.pi / 4) / 3
    kh = bb[:, None, None] * u[None, :, None]           # [n, 8, 1]
    l = np.arange(1, NO + 1)
    cs = (np.cos(th)[None, None, :] * kh / 2)[..., None] * l     # [n, 8, 4, NO]
    sn = (np.sin(th)[None, None, :] * kh / 2)[..., None] * l
    g = (np.sin(cs) ** 2 + np.sin(sn) ** 2) * mask[:, None, None, :]
    w = 4.0 / kh ** 2                                   # [n, 8, 1]
    e = (g * dc[:, None, None, :]).sum(-1)              # [n, 8, 4]
    r = w * e
    P = 32.0
    loss = (r ** 2).sum() / P / n
    dcoef = (2 * (r * w)[..., None] * g).sum((1, 2)) / P / n   # dL/dc  [n, NO]
    dy = dcoef * out_scale
    dz2 = (dy @ W3) * (1 - h2 * h2)
    dz1 = (dz2 @ W2) * (1 - h1 * h1)
    grads = [dz1.T @ xi, dz1.sum(0), dz2.T @ h1, dz2.sum(0), dy.T @ h2, dy.sum(0)]
    return loss, np.concatenate([a.ravel() for a in grads])
