"""The Der1-Der1 numerics (FLETCHER_NUMERICS_D1D1) on the GPU, through the C
ABI, against the der1der1/ tree's own output.

The fixtures tests/golden/golden_d1d1_*.npz were written by the reference's
der1der1/ OpenMP build (oracle/_ref, gcc -O3 on x86-64, which never contracts
a multiply and an add).  The mode evaluates that tree's formulation in its
operation order (der1der1/sample.h:35-120), every operation rounded on its
own, so the bound is bit equality.  The default numerics, which fold the
inverse spacings differently and use fused multiply-adds, are only within
1e-5 of the same fixtures; the mode must be strictly closer.
"""
import numpy as np
import pytest

from conftest import gpu_available, load_golden, subsample
from fletcher_petrobras_gb300 import FletcherError, Problem, Propagator

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not gpu_available():
        pytest.fail("these tests need a CUDA GPU")


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def run(prob, model, numerics, zchunks=0):
    prop = Propagator(zchunks=zchunks, numerics=numerics)
    prop.initialize(prob.sx, prob.sy, prob.sz, prob.bord, prob.dx, prob.dy, prob.dz, prob.dt, model)
    src = prob.sources()
    for it in range(1, prob.steps + 1):  # the reference's loop, original/model.c:71-88
        prop.insert_source(it - 1, prob.i_source, src[it - 1])
        prop.propagate(it)
    out = [prop.field(k) for k in range(4)]
    prop.finalize()
    return out


@pytest.mark.parametrize("name", ["d1d1_tiny_layered", "d1d1_c0", "d1d1_tiny_aniso"])
def test_d1d1_numerics_bit_identical_to_der1der1_tree(name):
    prob, meta, g = load_golden(name)
    m = prob.model()
    p, q, _, _ = run(prob, m, "d1d1")
    fp, fq, _, _ = run(prob, m, "fast")
    s = meta["stride"]
    sp, sq = subsample(p, prob, s), subsample(q, prob, s)
    e_mode = max(rel_l2(sp, g["p"]), rel_l2(sq, g["q"]))
    e_fast = max(rel_l2(subsample(fp, prob, s), g["p"]), rel_l2(subsample(fq, prob, s), g["q"]))
    nd = int(np.count_nonzero(sp != g["p"]) + np.count_nonzero(sq != g["q"]))
    print(f"{name}: d1d1 numerics vs der1der1 tree rel L2 {e_mode:.3g} ({nd} cells differ); "
          f"default numerics {e_fast:.3g}")
    assert np.array_equal(sp, g["p"]) and np.array_equal(sq, g["q"])
    assert e_fast > 0.0  # the default numerics round differently


@pytest.mark.parametrize("zchunks", [-1, 3, -3])
def test_d1d1_numerics_independent_of_work_split(zchunks):
    """Whole tile columns, shared-out segments and uniform z-chunks give the
    same floats (three different spacings)."""
    prob = Problem("d1d1split", 40, 28, 24, absorb=4, dx=10.0, dy=12.5, dz=15.0, dt=0.0005, steps=23, fcut=45.0,
                   kind="layered", layers=3, seed=21, source=(20, 16, 9))
    m = prob.model()
    base = run(prob, m, "d1d1", zchunks=-1)
    got = run(prob, m, "d1d1", zchunks=zchunks)
    for a, b in zip(base, got):
        assert np.array_equal(a, b)


def test_d1d1_numerics_rejects_16bit_forms():
    prop = Propagator(form="fp16x", numerics="d1d1")
    prob = Problem("d1d1half", 20, 20, 20, absorb=4, dt=0.0006, steps=2, kind="layered", layers=2, seed=1)
    with pytest.raises(FletcherError, match="FP32 form"):
        prop.initialize(prob.sx, prob.sy, prob.sz, prob.bord, prob.dx, prob.dy, prob.dz, prob.dt, prob.model())
    Propagator(form="fp32", numerics="fast")


@pytest.mark.parametrize("case", ["odd_sizes", "bord6", "thin_z", "src_tile_edge", "src_in_border"])
def test_d1d1_numerics_edge_cases_bit_identical_to_oracle(case, orc):
    """The geometry and source edge cases of the default numerics' parity tests
    (grid not a multiple of the tile, a border wider than the stencil, a few
    planes only, a source on a tile corner and chunk edge, a source in the
    never-updated border), held to bit equality against the oracle's
    restatement of the der1der1/ tree -- given the same coefficients: the
    GPU's FP64 trigonometry can round a coefficient one unit differently from
    the host's, which is not what this test is about."""
    base = Problem("edge", 21, 13, 9, absorb=3, dt=0.0006, steps=20, fcut=45.0, kind="layered", layers=3, seed=4)
    zc = 0
    if case == "odd_sizes":
        prob = base
    elif case == "bord6":
        prob = base.with_(bord=6)
    elif case == "thin_z":
        prob, zc = base.with_(nz=1, nx=40, ny=37), 3
    elif case == "src_tile_edge":
        prob = Problem("edge2", 60, 40, 40, absorb=4, dt=0.0006, steps=20, fcut=45.0, seed=4)
        prob, zc = prob.with_(source=(4 + 32, 4 + 15, 4 + 13)), 3  # tile corner (16-row tiles), chunk edge
    else:
        prob = base.with_(source=(2, base.sy // 2, base.sz // 2))
    m = prob.model()
    prop = Propagator(zchunks=zc, numerics="d1d1")
    prop.initialize(prob.sx, prob.sy, prob.sz, prob.bord, prob.dx, prob.dy, prob.dz, prob.dt, m)
    src = prob.sources()
    for it in range(1, prob.steps + 1):
        prop.insert_source(it - 1, prob.i_source, src[it - 1])
        prop.propagate(it)
    got = [prop.field(k) for k in range(4)]
    coef = prop.coefficients()
    prop.finalize()
    Propagator(numerics="fast")
    want = orc.run_d1d1_f32(prob, m, coef=coef)
    assert np.abs(want[0]).max() > 0
    for g, w in zip(got, want):
        assert np.array_equal(g, w), rel_l2(g, w)
