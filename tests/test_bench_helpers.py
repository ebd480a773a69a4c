"""Host-side helpers of bench.py (no GPU): the parity figure the C1 line
reports against the reference build's committed 1000-step fixture."""
import importlib.util
import os

import numpy as np

from conftest import ROOT, load_golden


def _bench():
    spec = importlib.util.spec_from_file_location("bench_module", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_reference_parity_reads_the_c1_fixture():
    from fletcher_petrobras_gb300 import C1

    bench = _bench()
    prob, meta, g = load_golden("c1")
    st = meta["stride"]
    full = {}
    for k in ("p", "q"):
        a = np.zeros((C1.sz, C1.sy, C1.sx), np.float32)
        view = a[::st, ::st, ::st]
        view[...] = g[k].reshape(view.shape)
        full[k] = a.ravel()
    same = bench.reference_parity(C1, 1000, "fp32", full["p"], full["q"])
    assert same["rel_l2_p"] == 0.0 and same["rel_l2_q"] == 0.0 and same["tolerance"] == 1e-4
    # a perturbed run reports its error
    off = bench.reference_parity(C1, 1000, "fp32", full["p"] * np.float32(1.001), full["q"])
    assert abs(off["rel_l2_p"] - 1e-3) < 1e-6 and off["rel_l2_q"] == 0.0
    # other runs have no fixture to compare with
    assert bench.reference_parity(C1, 999, "fp32", full["p"], full["q"]) is None
    assert bench.reference_parity(C1, 1000, "fp16x", full["p"], full["q"]) is None
    assert bench.reference_parity(C1.with_(name="other"), 1000, "fp32", full["p"], full["q"]) is None
