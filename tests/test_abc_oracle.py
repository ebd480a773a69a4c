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
    T = g.normal(0, 1, (24, 2))
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
