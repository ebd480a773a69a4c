"""ORACLE -- test infrastructure only.

CPU (numpy, FP64) restatement of the learned absorbing boundary's pieces in
fletcher_petrobras_gb300/csrc/abc_learned.cu, used by the tests to check the
GPU kernels:

* `forward` / `loss_and_grad`: the 40 -> 32 -> 32 -> 2 tanh network with the
  same roundings as the GPU path (weights, inputs and hidden activations
  rounded to FP16, biases and accumulation unrounded) and its analytic
  gradient (roundings treated as the identity);
* `features_targets`: the inputs and target of a layer cell, restated from
  the update of original/sample.h:32-89 (Der2 original/derivatives.h:37-41,
  DerCross :22-31) evaluated on the field beyond the layer.

Only the tests import this module; the library never does.
"""
from __future__ import annotations

import numpy as np

N_IN, N_HID, N_OUT = 40, 32, 2
OFF = {}
_o = 0
for _name, _size in (("W1", N_HID * N_IN), ("b1", N_HID), ("W2", N_HID * N_HID), ("b2", N_HID),
                     ("W3", N_OUT * N_HID), ("b3", N_OUT)):
    OFF[_name] = (_o, _size)
    _o += _size
N_PARAMS = _o  # 2434

K = np.array([-205.0 / 72.0, 8.0 / 5.0, -1.0 / 5.0, 8.0 / 315.0, -1.0 / 560.0])   # Der2 weights
L = np.array([0.0, 4.0 / 5.0, -1.0 / 5.0, 4.0 / 105.0, -1.0 / 280.0])               # Der1 weights


def unpack(P):
    P = np.asarray(P, np.float64)
    out = {}
    for k, (o, s) in OFF.items():
        out[k] = P[o:o + s]
    out["W1"] = out["W1"].reshape(N_HID, N_IN)
    out["W2"] = out["W2"].reshape(N_HID, N_HID)
    out["W3"] = out["W3"].reshape(N_OUT, N_HID)
    return out


def _h16(a, on=True):
    return np.asarray(a, np.float32).astype(np.float16).astype(np.float64) if on else np.asarray(a, np.float64)


def forward(P, X, rounding=True):
    """Raw outputs (n, 2) and the intermediates."""
    w = unpack(P)
    W1, W2, W3 = (_h16(w[k], rounding) for k in ("W1", "W2", "W3"))
    x = _h16(X, rounding)
    a1 = np.tanh(x @ W1.T + w["b1"])
    h1 = _h16(a1, rounding)
    a2 = np.tanh(h1 @ W2.T + w["b2"])
    h2 = _h16(a2, rounding)
    y = h2 @ W3.T + w["b3"]
    return y, dict(x=x, a1=a1, h1=h1, a2=a2, h2=h2, W2=W2, W3=W3)


def loss_and_grad(P, X, T, rounding=True):
    """loss = sum (y - t)^2 / (2 n) and d loss / d P (length 2434)."""
    n = X.shape[0]
    y, c = forward(P, X, rounding)
    e = y - np.asarray(T, np.float64)
    loss = float(np.sum(e * e) / (2.0 * n))
    dy = e / n
    dz2 = (dy @ c["W3"]) * (1.0 - c["a2"] ** 2)
    dz1 = (dz2 @ c["W2"]) * (1.0 - c["a1"] ** 2)
    g = np.zeros(N_PARAMS)
    parts = {"W1": dz1.T @ c["x"], "b1": dz1.sum(0), "W2": dz2.T @ c["h1"], "b2": dz2.sum(0),
             "W3": dy.T @ c["h2"], "b3": dy.sum(0)}
    for k, (o, s) in OFF.items():
        g[o:o + s] = parts[k].ravel()
    return loss, g


def _outside(box_lo, box_hi, c):
    return bool(np.any(np.asarray(c) < box_lo) or np.any(np.asarray(c) >= box_hi))


def features_targets(cur, prev, coef, in_lo, in_hi, layer, cells, d_xyz, dt, return_scale=False):
    """cur, prev: (p, q) pairs as arrays (2, sz, sy, sx); coef: (10, sz, sy, sx)
    in the reference order ch1dxx ch1dyy ch1dzz ch1dxy ch1dyz ch1dxz v2px v2pz
    v2sz v2pn; cells: (x, y, z) list.  Returns features (n, 40), targets
    (n, 2), both divided by the stencils' largest magnitude s as the GPU does
    (and s, with return_scale)."""
    in_lo = np.asarray(in_lo)
    in_hi = np.asarray(in_hi)
    k_lo, k_hi = in_lo - layer, in_hi + layer
    cur = np.asarray(cur, np.float64)
    prev = np.asarray(prev, np.float64)
    feats, tgts, scales = [], [], []

    def at(F, x, y, z):
        return F[:, z, y, x]

    def outer(x, y, z):
        return at(cur, x, y, z) if _outside(k_lo, k_hi, (x, y, z)) else np.zeros(2)

    for (x, y, z) in cells:
        c = np.array([x, y, z])
        dist = np.maximum(np.maximum(in_lo - c, c - (in_hi - 1)), 0)
        d = int(dist.max())
        a = int(np.argmax(dist))
        sgn = 1 if c[a] - (in_hi[a] - 1) > 0 else -1
        st = []
        for F in (cur, prev):
            vals = []
            for j in range(-4, 5):
                u = c.copy()
                u[a] += sgn * j
                vals.append(at(F, *u) if not _outside(k_lo, k_hi, u) else np.zeros(2))
            vals = np.array(vals)  # (9, 2)
            st += [vals[:, 0], vals[:, 1]]
        st = np.concatenate(st)
        s = np.abs(st).max()
        scales.append(s)
        v2px, v2pz, v2pn = coef[6, z, y, x], coef[7, z, y, x], coef[9, z, y, x]
        med = [np.sqrt(v2pz) / 4000.0, 0.5 * (v2px / v2pz - 1.0), 0.5 * (v2pn / v2pz - 1.0), d / layer]
        feats.append(np.concatenate([st / s, med]))
        # dt^2 * rhs of the field beyond the layer.
        e = np.eye(3, dtype=int)
        d2 = []
        for ax in range(3):
            acc = np.zeros(2)
            for k in range(1, 5):
                acc += K[k] * (outer(*(c + k * e[ax])) + outer(*(c - k * e[ax])))
            d2.append(acc / d_xyz[ax] ** 2)
        dc = []
        for (p1, p2) in ((0, 1), (1, 2), (0, 2)):
            acc = np.zeros(2)
            for i in range(1, 5):
                for j in range(1, 5):
                    o1, o2 = i * e[p1], j * e[p2]
                    acc += L[i] * L[j] * (outer(*(c + o1 + o2)) - outer(*(c + o1 - o2)) - outer(*(c - o1 + o2))
                                          + outer(*(c - o1 - o2)))
            dc.append(acc / (d_xyz[p1] * d_xyz[p2]))
        (pxx, qxx), (pyy, qyy), (pzz, qzz) = d2
        (pxy, qxy), (pyz, qyz), (pxz, qxz) = dc
        cxx, cyy, czz, cxy, cyz, cxz = (coef[k, z, y, x] for k in range(6))
        v2sz = coef[8, z, y, x]
        h1p = cxx * pxx + cyy * pyy + czz * pzz + cxy * pxy + cyz * pyz + cxz * pxz
        h1q = cxx * qxx + cyy * qyy + czz * qzz + cxy * qxy + cyz * qyz + cxz * qxz
        h2p, h2q = pxx + pyy + pzz - h1p, qxx + qyy + qzz - h1q
        rhsp = v2px * h2p + v2pz * h1q + v2sz * (h1p - h1q)
        rhsq = v2pn * h2p + v2pz * h1q - v2sz * (h2p - h2q)
        tgts.append(np.array([rhsp, rhsq]) * dt * dt / s)
    if return_scale:
        return np.array(feats), np.array(tgts), np.array(scales)
    return np.array(feats), np.array(tgts)
