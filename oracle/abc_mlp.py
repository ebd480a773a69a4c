"""ORACLE -- test infrastructure only.

CPU (numpy, FP64) restatement of the learned absorbing boundary's pieces in
fletcher_petrobras_gb300/csrc/abc_learned.cu, used by the tests to check the
GPU kernels:

* `forward` / `loss_and_grad`: the 40 -> 32 -> 32 -> 2 tanh network with the
  same roundings as the GPU path (weights, inputs, hidden pre-activations
  and activations rounded to FP16, biases and accumulation unrounded), the
  loss
  sum_c (sigmoid(y_c) a_c - b_c)^2 / (2 n) and its analytic gradient
  (roundings treated as the identity);
* `ghost_cells`: the ghost zone's cells in the library's order (faces z-,
  z+, y-, y+, x-, x+; rays with the first transverse axis fastest; d
  fastest within a ray);
* `features_targets`: the inputs and targets (a, b) of ghost cells, with the
  plain update of original/sample.h:32-89 (Der2 original/derivatives.h:37-41,
  DerCross :22-31) giving the next values;
* `oneway_update`: the box-scheme update of the ghost zone after a step.

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
    a1 = np.tanh(_h16(x @ W1.T + w["b1"], rounding))
    h1 = _h16(a1, rounding)
    a2 = np.tanh(_h16(h1 @ W2.T + w["b2"], rounding))
    h2 = _h16(a2, rounding)
    y = h2 @ W3.T + w["b3"]
    return y, dict(x=x, a1=a1, h1=h1, a2=a2, h2=h2, W2=W2, W3=W3)


def sigmoid(y):
    return 1.0 / (1.0 + np.exp(-y))


def loss_and_grad(P, X, T, rounding=True):
    """T (n, 4) = a_p, a_q, b_p, b_q.  loss = sum_c (sigmoid(y_c) a_c -
    b_c)^2 / (2 n) and d loss / d P (length 2434)."""
    n = X.shape[0]
    y, c = forward(P, X, rounding)
    T = np.asarray(T, np.float64)
    a, b = T[:, :2], T[:, 2:]
    k = sigmoid(y)
    e = k * a - b
    loss = float(np.sum(e * e) / (2.0 * n))
    dy = e * a * k * (1.0 - k) / n
    dz2 = (dy @ c["W3"]) * (1.0 - c["a2"] ** 2)
    dz1 = (dz2 @ c["W2"]) * (1.0 - c["a1"] ** 2)
    g = np.zeros(N_PARAMS)
    parts = {"W1": dz1.T @ c["x"], "b1": dz1.sum(0), "W2": dz2.T @ c["h1"], "b2": dz2.sum(0),
             "W3": dy.T @ c["h2"], "b3": dy.sum(0)}
    for k_, (o, s_) in OFF.items():
        g[o:o + s_] = parts[k_].ravel()
    return loss, g


GHOST = 4  # the layer's outer cells


def face_axis(f):
    return 2 - f // 2


def face_sign(f):
    return 1 if f & 1 else -1


def ghost_cells(in_lo, in_hi, layer):
    """(x, y, z, face, d) of every ghost cell, in the library's order."""
    in_lo = np.asarray(in_lo)
    in_hi = np.asarray(in_hi)
    k_lo, k_hi = in_lo - layer, in_hi + layer
    out = []
    for f in range(6):
        a, sgn = face_axis(f), face_sign(f)
        t0, t1 = (1 if a == 0 else 0), (1 if a == 2 else 2)
        for v in range(k_lo[t1], k_hi[t1]):
            for u in range(k_lo[t0], k_hi[t0]):
                for d in range(layer - GHOST + 1, layer + 1):
                    c = [0, 0, 0]
                    c[t0], c[t1] = u, v
                    c[a] = in_lo[a] - d if sgn < 0 else in_hi[a] - 1 + d
                    out.append((int(c[0]), int(c[1]), int(c[2]), f, d))
    return out


def _outside(box_lo, box_hi, c):
    return bool(np.any(np.asarray(c) < box_lo) or np.any(np.asarray(c) >= box_hi))


def _rhs(cur, coef, c, d_xyz, dt):
    """dt^2 (rhsp, rhsq) of original/sample.h:32-89 at cell c of the field cur."""
    e = np.eye(3, dtype=int)

    def at(u):
        return cur[:, u[2], u[1], u[0]]

    d2 = []
    for ax in range(3):
        acc = K[0] * at(c)
        for k in range(1, 5):
            acc = acc + K[k] * (at(c + k * e[ax]) + at(c - k * e[ax]))
        d2.append(acc / d_xyz[ax] ** 2)
    dc = []
    for (p1, p2) in ((0, 1), (1, 2), (0, 2)):
        acc = np.zeros(2)
        for i in range(1, 5):
            for j in range(1, 5):
                o1, o2 = i * e[p1], j * e[p2]
                acc += L[i] * L[j] * (at(c + o1 + o2) - at(c + o1 - o2) - at(c - o1 + o2) + at(c - o1 - o2))
        dc.append(acc / (d_xyz[p1] * d_xyz[p2]))
    (pxx, qxx), (pyy, qyy), (pzz, qzz) = d2
    (pxy, qxy), (pyz, qyz), (pxz, qxz) = dc
    x, y, z = c
    cxx, cyy, czz, cxy, cyz, cxz = (coef[k, z, y, x] for k in range(6))
    v2px, v2pz, v2sz, v2pn = (coef[k, z, y, x] for k in range(6, 10))
    h1p = cxx * pxx + cyy * pyy + czz * pzz + cxy * pxy + cyz * pyz + cxz * pxz
    h1q = cxx * qxx + cyy * qyy + czz * qzz + cxy * qxy + cyz * qyz + cxz * qxz
    h2p, h2q = pxx + pyy + pzz - h1p, qxx + qyy + qzz - h1q
    rhsp = v2px * h2p + v2pz * h1q + v2sz * (h1p - h1q)
    rhsq = v2pn * h2p + v2pz * h1q - v2sz * (h2p - h2q)
    return np.array([rhsp, rhsq]) * dt * dt


def features_targets(cur, prev, coef, in_lo, in_hi, layer, cells, d_xyz, dt, return_scale=False, targets=True):
    """cur, prev: (p, q) pairs as arrays (2, sz, sy, sx); coef: (10, sz, sy, sx)
    in the reference order ch1dxx ch1dyy ch1dzz ch1dxy ch1dyz ch1dxz v2px v2pz
    v2sz v2pn; cells: (x, y, z, face, d) tuples.  Returns features (n, 40)
    and targets (n, 4) = (a_p, a_q, b_p, b_q), divided by the stencils'
    largest magnitude s as the GPU does (and s, with return_scale); with
    targets=False the targets are left at zero."""
    in_lo = np.asarray(in_lo)
    in_hi = np.asarray(in_hi)
    k_lo, k_hi = in_lo - layer, in_hi + layer
    cur = np.asarray(cur, np.float64)
    prev = np.asarray(prev, np.float64)
    feats, tgts, scales = [], [], []

    def at(F, u):
        return F[:, u[2], u[1], u[0]]

    for (x, y, z, f, d) in cells:
        c = np.array([x, y, z])
        a, sgn = face_axis(f), face_sign(f)
        st = []
        for F in (cur, prev):
            vals = []
            for j in range(-4, 5):
                u = c.copy()
                u[a] += sgn * j
                vals.append(at(F, u) if not _outside(k_lo, k_hi, u) else np.zeros(2))
            vals = np.array(vals)  # (9, 2)
            st += [vals[:, 0], vals[:, 1]]
        st = np.concatenate(st)
        s = np.abs(st).max()
        if not s > 1e-30:  # no wave: the GPU feeds zeros (its reciprocal would overflow)
            s = 0.0
        scales.append(s)
        inv = 1.0 / s if s > 0 else 0.0
        v2px, v2pz, v2pn = coef[6, z, y, x], coef[7, z, y, x], coef[9, z, y, x]
        med = [np.sqrt(v2pz) / 4000.0, 0.5 * (v2px / v2pz - 1.0), 0.5 * (v2pn / v2pz - 1.0), d / layer]
        feats.append(np.concatenate([st * inv, med]))
        if not targets:
            tgts.append(np.zeros(4))
            continue
        ci = c.copy()
        ci[a] -= sgn
        ug, ui = at(cur, c), at(cur, ci)
        ug1 = 2.0 * ug - at(prev, c) + _rhs(cur, coef, c, d_xyz, dt)
        ui1 = 2.0 * ui - at(prev, ci) + _rhs(cur, coef, ci, d_xyz, dt)
        tgts.append(np.concatenate([ug - ui1, ug1 - ui]) * inv)
    if return_scale:
        return np.array(feats), np.array(tgts), np.array(scales)
    return np.array(feats), np.array(tgts)


def oneway_update(cur, nxt, in_lo, in_hi, layer, k):
    """The ghost-zone update after a step: nxt (2, sz, sy, sx), updated in
    place and returned; k (n, 2) per ghost cell in ghost_cells order."""
    cells = ghost_cells(in_lo, in_hi, layer)
    for i, (x, y, z, f, d) in enumerate(cells):
        a, sgn = face_axis(f), face_sign(f)
        c = [x, y, z]
        ci = list(c)
        ci[a] -= sgn
        g = (slice(None), c[2], c[1], c[0])
        gi = (slice(None), ci[2], ci[1], ci[0])
        nxt[g] = cur[gi] + k[i] * (cur[g] - nxt[gi])
    return nxt
