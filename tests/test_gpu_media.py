"""The media-table coefficient layout on the GPU.

The FP32 step reads each cell's six angle coefficients from a table of at
most 256 (phi, theta) pairs (one id byte per cell) instead of six coefficient
planes; the floats used are the same, so every run must be bit-identical to
the plane layout: isotropic and three-spacing grids, grids that are not a
multiple of the tile, wide borders, thin grids, every built pipeline depth,
the segment-list plan and the multi-step entry point.  Models with more
pairs than the table holds fall back to the planes (auto) or are refused
(media requested).  The layout is also held to the oracle directly.
"""
import numpy as np
import pytest

from conftest import gpu_available
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


def run(prob, model, layout, tile=(0, 0, 0), use_run=False, steps=None):
    st = prob.steps if steps is None else steps
    prop = Propagator(*tile, coef_layout=layout)
    prop.initialize(prob.sx, prob.sy, prob.sz, prob.bord, prob.dx, prob.dy, prob.dz, prob.dt, model)
    got_layout = prop.coef_layout()
    src = prob.sources(st)
    if use_run:
        prop.run(st, prob.i_source, src)
        prop.synchronize()
    else:
        for it in range(1, st + 1):
            prop.insert_source(it - 1, prob.i_source, src[it - 1])
            prop.propagate(it)
    out = [prop.field(k) for k in range(4)]
    prop.finalize()
    Propagator()  # back to the default options
    return out, got_layout


BASE = Problem("media", 21, 13, 9, absorb=3, dt=0.0006, steps=20, fcut=45.0, kind="layered", layers=3, seed=4)
CASES = {
    "odd_sizes": (BASE, (0, 0, 0)),
    "bord6": (BASE.with_(bord=6), (0, 0, 0)),
    "thin_z": (BASE.with_(nz=1, nx=40, ny=37), (16, 5, 3)),
    "three_spacings": (Problem("media3", 40, 36, 30, absorb=6, dx=10.0, dy=12.5, dz=15.0, dt=0.0006, steps=24,
                               fcut=45.0, kind="layered", layers=5, seed=8), (0, 0, 0)),
    "layered_c1_like": (Problem("mediaC", 88, 88, 88, absorb=16, dt=0.0006, steps=16, fcut=40.0, kind="layered",
                                layers=8, seed=1), (0, 0, 0)),
    "homogeneous": (Problem("mediaH", 48, 40, 36, absorb=8, dt=0.001, steps=20, fcut=50.0), (0, 0, 0)),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_media_layout_bit_identical_to_planes(case):
    prob, tile = CASES[case]
    m = prob.model()
    planes, lp = run(prob, m, "planes", tile)
    media, lm = run(prob, m, "media", tile)
    assert (lp, lm) == ("planes", "media")
    assert np.abs(planes[0]).max() > 0
    for a, b in zip(media, planes):
        assert np.array_equal(a, b), rel_l2(a, b)


@pytest.mark.parametrize("stages", [5, 6, 7])
@pytest.mark.parametrize("zchunks", [0, 2, -1, -3])
def test_media_shapes_and_plans_bit_identical(stages, zchunks):
    """Every built depth through both work-item modes: segment lists
    (zchunks >= 0: this small grid has fewer items than CTAs, so the plan
    shares them out) and arithmetic round-robin items (zchunks < 0)."""
    prob = Problem("mediaS", 70, 27, 33, absorb=5, dt=0.0006, steps=24, fcut=45.0, kind="layered", layers=5,
                   seed=9)
    prob = prob.with_(source=(prob.sx // 2 + 1, prob.sy // 2, prob.sz // 2 + 2))
    m = prob.model()
    ref, _ = run(prob, m, "planes", (16, 5, zchunks))
    got, lay = run(prob, m, "media", (16, stages, zchunks))
    assert lay == "media"
    for a, b in zip(got, ref):
        assert np.array_equal(a, b)


def test_media_multi_step_entry_point():
    prob = CASES["layered_c1_like"][0]
    m = prob.model()
    a, _ = run(prob, m, "media")
    b, _ = run(prob, m, "media", use_run=True)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_auto_layout_choice_and_overflow():
    """A model with more than 256 (phi, theta) pairs: auto keeps the planes
    (and the same results as planes), media is refused.  On a layered model
    auto picks media."""
    prob = Problem("mediaO", 30, 28, 26, absorb=4, dt=0.0006, steps=10, fcut=45.0, kind="layered", layers=4,
                   seed=2)
    m = prob.model()
    _, lay = run(prob, m, "auto")
    assert lay == "media"
    rng = np.random.default_rng(0)
    m2 = m.copy()
    m2[4] = rng.uniform(0.0, 1.0, m.shape[1]).astype(np.float32)  # phi per cell: ~all distinct
    auto, lay = run(prob, m2, "auto")
    assert lay == "planes"
    planes, _ = run(prob, m2, "planes")
    for a, b in zip(auto, planes):
        assert np.array_equal(a, b)
    prop = Propagator(coef_layout="media")
    with pytest.raises(FletcherError, match=r"more than 256 distinct \(phi, theta\) pairs"):
        prop.initialize(prob.sx, prob.sy, prob.sz, prob.bord, prob.dx, prob.dy, prob.dz, prob.dt, m2)
    # Exactly 256 pairs still fit.
    m3 = m.copy()
    m3[4] = (np.arange(m.shape[1]) % 256).astype(np.float32) * 0.01
    m3[5] = np.float32(0.3)
    a3, lay = run(prob, m3, "auto")
    assert lay == "media"
    b3, _ = run(prob, m3, "planes")
    for a, b in zip(a3, b3):
        assert np.array_equal(a, b)
    Propagator()


def test_media_layout_refused_where_not_built():
    prob = Problem("mediaR", 20, 20, 20, absorb=4, dt=0.0006, steps=4, fcut=45.0, kind="layered", layers=3)
    m = prob.model()
    for kw in ({"form": "fp16x"}, {"numerics": "d1d1"}, {"tile_rows": 12, "stages": 5}):
        prop = Propagator(coef_layout="media", **kw)
        with pytest.raises(FletcherError, match=r"media-table layout"):
            prop.initialize(prob.sx, prob.sy, prob.sz, prob.bord, prob.dx, prob.dy, prob.dz, prob.dt, m)
    # auto with a plane-only shape or form: planes.
    for kw in ({"form": "fp16x"}, {"tile_rows": 12, "stages": 5}):
        prop = Propagator(coef_layout="auto", **kw)
        prop.initialize(prob.sx, prob.sy, prob.sz, prob.bord, prob.dx, prob.dy, prob.dz, prob.dt, m)
        assert prop.coef_layout() == "planes"
        prop.finalize()
    Propagator()


def test_media_layout_vs_oracle(orc):
    """The auto layout (media, on this layered model) against the oracle's
    restatement of the reference at the short-run tolerance 1e-5."""
    prob = CASES["three_spacings"][0]
    m = prob.model()
    got, lay = run(prob, m, "auto")
    assert lay == "media"
    want = orc.run_f32(prob, m)
    for g, w in zip(got, want):
        assert rel_l2(g, w) < 1e-5
