"""CPU checks of the learned boundary's oracle (oracle/abc_mlp.py): its
analytic gradient against central finite differences (FP64, without the
FP16 roundings, whose derivative the GPU and the oracle both take as the
identity), and the parameter layout the C header declares."""
import re

import numpy as np

from conftest import ROOT


def test_parameter_count_matches_header():
    from oracle import abc_mlp

    hdr = open(f"{ROOT}/include/fletcher_gb300.h").read()
    assert int(re.search(r"#define FLETCHER_ABC_PARAMS (\d+)", hdr).group(1)) == abc_mlp.N_PARAMS == 2434


def test_oracle_gradient_vs_finite_differences():
    from oracle import abc_mlp

    g = np.random.default_rng(0)
    P = g.normal(0, 0.3, abc_mlp.N_PARAMS)
    X = g.uniform(-1, 1, (24, 40))
    T = g.normal(0, 1, (24, 4))
    _, grad = abc_mlp.loss_and_grad(P, X, T, rounding=False)
    idx = np.concatenate([g.choice(abc_mlp.N_PARAMS, 60, replace=False),
                          np.arange(abc_mlp.N_PARAMS - 66, abc_mlp.N_PARAMS)])
    h = 1e-6
    for i in idx:
        e = np.zeros(abc_mlp.N_PARAMS)
        e[i] = h
        fd = (abc_mlp.loss_and_grad(P + e, X, T, rounding=False)[0]
              - abc_mlp.loss_and_grad(P - e, X, T, rounding=False)[0]) / (2 * h)
        assert abs(fd - grad[i]) <= 1e-6 * max(1.0, abs(fd)), i


def test_oracle_rounding_matches_fp16():
    """With rounding the forward uses FP16 weights, inputs and activations."""
    from oracle import abc_mlp

    g = np.random.default_rng(1)
    P = g.normal(0, 0.3, abc_mlp.N_PARAMS)
    X = g.uniform(-1, 1, (8, 40))
    y, c = abc_mlp.forward(P, X)
    assert np.array_equal(c["h1"], c["h1"].astype(np.float16).astype(np.float64))
    y0, _ = abc_mlp.forward(P, X, rounding=False)
    assert np.max(np.abs(y - y0)) < 0.05 * np.max(np.abs(y0)) + 1e-3


def test_ghost_zone_enumeration():
    """The ghost zone is the layer's outer 4 cells on every face: each face
    holds one ray of 4 cells per transverse position of the kept box, and
    every cell lies d = L-3 .. L cells outside the interior along its face's
    axis."""
    from oracle import abc_mlp

    lo, hi, L = (12, 13, 14), (20, 23, 18), 8
    cells = abc_mlp.ghost_cells(lo, hi, L)
    ext = [h - l + 2 * L for l, h in zip(lo, hi)]
    want = 4 * 2 * (ext[0] * ext[1] + ext[0] * ext[2] + ext[1] * ext[2])
    assert len(cells) == want
    for (x, y, z, f, d) in cells[::37]:
        a, sgn = abc_mlp.face_axis(f), abc_mlp.face_sign(f)
        c = (x, y, z)
        dist = lo[a] - c[a] if sgn < 0 else c[a] - (hi[a] - 1)
        assert dist == d and L - 3 <= d <= L
        for b in range(3):
            assert lo[b] - L <= c[b] < hi[b] + L
    # rays: 4 consecutive cells, d = L-3 .. L, stepping outward
    for i in range(0, len(cells), 4 * 101):
        ray = cells[i:i + 4]
        assert [r[4] for r in ray] == [5, 6, 7, 8]
        a = abc_mlp.face_axis(ray[0][3])
        assert len({r[:3][b] for r in ray for b in range(3) if b != a}) <= 2


def test_oneway_update_transports_a_plane_wave():
    """With k = (1 - r) / (1 + r) the box-scheme update of the oracle carries a
    smooth outgoing profile u(x - c t) across the ghost zone with a small
    error, and it is exact for a profile constant in space."""
    from oracle import abc_mlp

    L, n = 8, 4
    lo, hi = (L + 4,) * 3, (L + 4 + n,) * 3
    S = n + 2 * (L + 4)
    r = 0.2
    k = (1 - r) / (1 + r)
    cells = abc_mlp.ghost_cells(lo, hi, L)
    x = np.arange(S, dtype=np.float64)
    prof = lambda t: np.exp(-((x - 24.0 - r * t) / 6.0) ** 2)  # moving along +x, r cells per step
    cur = np.zeros((2, S, S, S))
    nxt = np.zeros((2, S, S, S))
    cur[:] = prof(0)[None, None, None, :]
    nxt[:] = prof(1)[None, None, None, :]
    want = nxt.copy()
    kk = np.full((len(cells), 2), k)
    abc_mlp.oneway_update(cur, nxt, lo, hi, L, kk)
    # the x+ face away from the edges (there the y and z faces, applied
    # first, give the wave a wrong direction)
    xs = [c for c in cells if c[3] == 5 and lo[1] <= c[1] < hi[1] and lo[2] <= c[2] < hi[2]]
    err = max(abs(nxt[0, z, y, x_] - want[0, z, y, x_]) for (x_, y, z, f, d) in xs)
    assert err < 1e-3
    flat = np.ones((2, S, S, S))
    out = abc_mlp.oneway_update(flat, flat.copy(), lo, hi, L, kk)
    assert np.allclose(out, 1.0)


def test_boundary_arguments_are_checked_on_the_host(lib):
    """Host-side checks of part 4, before any CUDA call: the network interval
    must be positive, a boundary needs an initialised state, an unknown mode
    is refused."""
    lib.FLETCHER_SetErrorMode(1)
    lib.FLETCHER_ClearError()
    assert lib.FLETCHER_AbcSetInterval(0) != 0
    lib.FLETCHER_ClearError()
    assert lib.FLETCHER_AbcSetInterval(3) == 0
    assert lib.FLETCHER_AbcSetInterval(1) == 0
    assert lib.FLETCHER_SetBoundary(1, 8, 0.0) != 0  # no DRIVER_Initialize yet
    lib.FLETCHER_ClearError()
    assert lib.FLETCHER_SetBoundary(7, 8, 0.0) != 0
    lib.FLETCHER_ClearError()
    assert lib.FLETCHER_AbcLayerCells() == 0
