"""16-bit wavefield storage (FLETCHER_FORM_FP16 / FLETCHER_FORM_FP16X) on the
GPU, through the C ABI, against the FP64 oracle.

Both forms store (p, q) per cell with one power-of-two scale per z-plane and
compute in FP32.  FP16 keeps an 11-bit significand per value, FP16X a 19-bit
one (FP16 plus a residual byte).  The error vs the FP64 oracle (relative L2
of p and q over the compared cells) is bounded per form:

* 128^3 interior, 2000 steps (the 16-bit storage case): <= 1e-3 for both
  forms.  FP16X meets it.  FP16 does not, and its test is an expected
  failure (xfail, strict) that names the miss: its per-step rounding (2^-12
  of each value) accumulates through the leapfrog update
  (p_next = 2 p - p_prev + ...), whose near-zero-frequency modes integrate
  the rounding noise, and reaches 0.45 (p) / 0.58 (q) after 2000 steps.  A
  separate test only checks that FP16 stays finite and below 1 there.
* short runs (150 steps): FP16X <= 1e-4, FP16 <= 2e-2.

Results that do not depend on the launch shape (tile rows, stages,
z-chunks) must be bit-identical, as in the FP32 form.
"""
import numpy as np
import pytest

from conftest import gpu_available, load_golden, plane_sums, subsample
from fletcher_petrobras_gb300 import C2, FletcherError, Problem, Propagator

pytestmark = pytest.mark.gpu

TOL = {"fp16x": {"short": 1e-4, "c2": 1e-3}, "fp16": {"short": 2e-2, "c2": 1e-3}}
FP16_C2_MISS = ("FP16 storage (11-bit significand) misses the 1e-3 C2 bound: relative L2 0.45 (p) / 0.58 (q) "
                "after 2000 steps; FP16X is the 16-bit-storage form that meets it")


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not gpu_available():
        pytest.fail("these tests need a CUDA GPU")


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def run(prob, model, form, steps=None, tile=(0, 0, 0), fields=None):
    st = prob.steps if steps is None else steps
    prop = Propagator(*tile, form=form)
    kw = {} if fields is None else dict(zip(("pp", "pc", "qp", "qc"), fields))
    prop.initialize(prob.sx, prob.sy, prob.sz, prob.bord, prob.dx, prob.dy, prob.dz, prob.dt, model, **kw)
    if st:
        prop.run(st, prob.i_source, prob.sources(st))
        prop.synchronize()
    out = [prop.field(k) for k in range(4)]
    bpc = prop.bytes_per_cell()
    prop.finalize()
    return out, bpc


SMALL = Problem("half_small", 40, 36, 32, absorb=6, dt=0.0006, steps=150, fcut=45.0, kind="layered", layers=4,
                seed=12)


@pytest.mark.parametrize("form", ["fp16x", "fp16"])
def test_short_run_vs_fp64_oracle(form, orc):
    m = SMALL.model()
    (p, q, pp, qp), bpc = run(SMALL, m, form)
    op, oq = orc.run_f64(SMALL, m)
    ep, eq = rel_l2(p, op), rel_l2(q, oq)
    print(f"{form}: rel L2 vs FP64 p {ep:.3g} q {eq:.3g} ({bpc} B/cell)")
    assert ep < TOL[form]["short"] and eq < TOL[form]["short"]
    assert bpc == {"fp16": 52.0, "fp16x": 58.0}[form]
    # cells outside the updated region stay zero
    v = p.reshape(SMALL.sz, SMALL.sy, SMALL.sx)
    b = SMALL.bord
    assert not v[:b].any() and not v[-b:].any() and not v[:, :b].any() and not v[:, :, -b:].any()


ANISO = Problem("half_aniso", 40, 36, 32, absorb=6, dx=10.0, dy=12.5, dz=15.0, dt=0.0005, steps=150, fcut=45.0,
                kind="layered", layers=4, seed=13)


@pytest.mark.parametrize("form", ["fp16x", "fp16"])
def test_anisotropic_spacing_vs_fp64_oracle(form, orc):
    """dx, dy, dz all different: every derivative carries its own inverse
    spacing (the kernels' non-isotropic path); same bounds as the short run."""
    m = ANISO.model()
    (p, q, _, _), _ = run(ANISO, m, form)
    op, oq = orc.run_f64(ANISO, m)
    ep, eq = rel_l2(p, op), rel_l2(q, oq)
    print(f"{form} anisotropic: rel L2 vs FP64 p {ep:.3g} q {eq:.3g}")
    assert ep < TOL[form]["short"] and eq < TOL[form]["short"]
    (p32, _, _, _), _ = run(ANISO, m, "fp32")
    assert rel_l2(p32, op) < 1e-5


def c2_errors(form):
    prob, meta, g = load_golden("c2_f64")
    assert prob == C2
    (p, q, _, _), _ = run(prob, prob.model(), form)
    s = meta["stride"]
    ep, eq = rel_l2(subsample(p, prob, s), g["p"]), rel_l2(subsample(q, prob, s), g["q"])
    es = rel_l2(plane_sums(p, prob), g["psum"])
    print(f"{form} C2: rel L2 vs FP64 p {ep:.3g} q {eq:.3g}; plane energy {es:.3g}")
    return ep, eq


@pytest.mark.parametrize("form", ["fp16x", pytest.param("fp16", marks=pytest.mark.xfail(strict=True,
                                                                                        reason=FP16_C2_MISS))])
def test_c2_error_vs_fp64_oracle(form):
    """128^3 interior (200^3 grid), 2000 steps, vs the FP64 oracle fixture:
    the 16-bit storage contract, relative L2 <= 1e-3 for p and q."""
    ep, eq = c2_errors(form)
    assert ep < TOL[form]["c2"] and eq < TOL[form]["c2"]


def test_c2_fp16_stays_bounded():
    """FP16 on the same case: not within the contract (above), but finite
    and below 1."""
    ep, eq = c2_errors("fp16")
    assert np.isfinite(ep) and np.isfinite(eq) and ep < 1.0 and eq < 1.0


def test_c2_fp32_form_vs_fp64_oracle():
    """The FP32 form on the same case, for comparison (FP32 rounding only)."""
    prob, meta, g = load_golden("c2_f64")
    (p, q, _, _), _ = run(prob, prob.model(), "fp32")
    s = meta["stride"]
    ep, eq = rel_l2(subsample(p, prob, s), g["p"]), rel_l2(subsample(q, prob, s), g["q"])
    print(f"fp32 C2: rel L2 vs FP64 p {ep:.3g} q {eq:.3g}")
    assert ep < 1e-4 and eq < 1e-4


@pytest.mark.parametrize("tile", [(12, 4, 1), (12, 6, 3), (8, 6, 2), (12, 5, 5), (16, 5, 0)])
@pytest.mark.parametrize("form", ["fp16x", "fp16"])
def test_launch_shapes_bit_identical(form, tile):
    prob = Problem("hshape", 70, 27, 33, absorb=5, dt=0.0006, steps=24, fcut=45.0, kind="layered", layers=5, seed=9)
    prob = prob.with_(source=(prob.sx // 2 + 1, prob.sy // 2, prob.sz // 2 + 2))
    m = prob.model()
    base, _ = run(prob, m, form)
    got, _ = run(prob, m, form, tile=tile)
    for a, b in zip(base, got):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("form", ["fp16x", "fp16"])
def test_initial_fields_round_trip(form):
    """Encoding of initial fields: every value within the form's significand
    (relative 2^-11 for FP16, 2^-18 for FP16X, of the value itself)."""
    prob = Problem("hinit", 30, 26, 22, absorb=3, dt=0.0006, steps=0, kind="layered", layers=3, seed=5)
    g = np.random.default_rng(3)
    inner = np.zeros((prob.sz, prob.sy, prob.sx), bool)
    b = prob.bord
    inner[b:-b, b:-b, b:-b] = True
    fields = []
    for _ in range(4):
        f = (g.standard_normal(inner.shape) * np.exp(g.uniform(-20, 5, inner.shape))).astype(np.float32)
        f[~inner] = 0
        fields.append(f.ravel())
    (p, q, pp, qp), _ = run(prob, prob.model(), form, steps=0, fields=fields)
    # FP16X: 2^-19, or 2^-18 where a tie clamps the residual byte
    rel = 2.0 ** -11 if form == "fp16" else 2.0 ** -18
    for got, want in ((p, fields[1]), (q, fields[3]), (pp, fields[0]), (qp, fields[2])):
        plane_max = np.abs(want.reshape(prob.sz, -1)).max(axis=1)
        # values far below their plane's maximum fall into FP16's subnormals
        floor = (plane_max * 2.0 ** -37)[:, None] * np.ones((1, prob.sx * prob.sy))
        err = np.abs(got - want)
        assert np.all(err <= rel * np.abs(want) + floor.ravel())


def test_rejects_what_the_16_bit_forms_cannot_hold():
    prob = Problem("hrej", 20, 20, 20, absorb=3, dt=0.0006, steps=2, kind="layered", layers=2, seed=1)
    m = prob.model()
    bad = np.zeros(prob.n, np.float32)
    bad[0] = 1.0  # a border cell
    prop = Propagator(form="fp16")
    with pytest.raises(FletcherError):
        prop.initialize(prob.sx, prob.sy, prob.sz, prob.bord, prob.dx, prob.dy, prob.dz, prob.dt, m, pc=bad)
    prop.initialize(prob.sx, prob.sy, prob.sz, prob.bord, prob.dx, prob.dy, prob.dz, prob.dt, m)
    with pytest.raises(FletcherError):
        prop.insert_source(0, 1, 1.0)  # outside the updated region
    prop.insert_source(0, prob.i_source, 1.0)
    with pytest.raises(FletcherError):
        prop.insert_source(0, prob.i_source, 1.0)  # a second source before the step
    prop.finalize()
    Propagator(form="fp32")  # restores the default form


@pytest.mark.parametrize("form", ["fp16x", "fp16"])
def test_driver_loop_and_update_pointers(form, orc):
    """The reference's loop (InsertSource, Propagate, Update_pointers) in a
    16-bit form: pc after each step tracks the FP64 oracle."""
    prob = Problem("hloop", 24, 24, 24, absorb=4, dt=0.0006, steps=12, fcut=45.0, kind="layered", layers=3, seed=6)
    m = prob.model()
    prop = Propagator(form=form)
    prop.initialize(prob.sx, prob.sy, prob.sz, prob.bord, prob.dx, prob.dy, prob.dz, prob.dt, m)
    src = prob.sources()
    pc = np.zeros(prob.n, np.float32)
    for it in range(1, prob.steps + 1):
        prop.insert_source(it - 1, prob.i_source, src[it - 1])
        prop.propagate(it)
    prop.update_pointers(pc)
    prop.finalize()
    Propagator(form="fp32")
    op, _ = orc.run_f64(prob, m)
    assert rel_l2(pc, op) < TOL[form]["short"]
