"""GPU parity: the CUDA path, called through the C ABI, against the reference's
outputs (golden fixtures) and the oracle on the same seeded inputs.

Tolerances (relative L2 over the compared cells, stated per test): the GPU
kernel evaluates DerCross as D1(D1(.)) and folds the inverse spacings per
derivative, so its FP32 rounding differs from the reference's grouped sums;
1e-5 bounds short runs, and the 504^3 x 1000-step run is held to the 1e-4
target.  Results that do not depend on rounding order (tile shapes, chunking,
multi-step entry point) must be bit-identical.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, gpu_available, load_golden, plane_sums, subsample
from fletcher_petrobras_gb300 import C0, C1, Problem, Propagator

pytestmark = pytest.mark.gpu

TOL_SHORT = 1e-5
TOL_C1 = 1e-4


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not gpu_available():
        pytest.fail("these tests need a CUDA GPU")


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def gpu_run(prob, model, steps=None, tile=(0, 0, 0), use_run=False):
    """The reference's time loop (original/model.c:71-88) through DRIVER_*."""
    st = prob.steps if steps is None else steps
    prop = Propagator(*tile)
    prop.initialize(prob.sx, prob.sy, prob.sz, prob.bord, prob.dx, prob.dy, prob.dz, prob.dt, model)
    src = prob.sources(st)
    if use_run:
        prop.run(st, prob.i_source, src)
        prop.synchronize()
    else:
        for it in range(1, st + 1):
            prop.insert_source(it - 1, prob.i_source, src[it - 1])
            prop.propagate(it)
    out = [prop.field(k) for k in range(4)]
    launches = prop.kernel_launches()
    prop.finalize()
    assert launches >= st
    return out


def oracle_model(orc, prob):
    return orc.boundary(prob.sx, prob.sy, prob.sz, prob.nx, prob.ny, prob.nz, prob.bord, prob.absorb,
                        prob.raw_model(), prob.seed)


def test_coefficients_match_oracle(orc):
    """FP64 precompute on the GPU vs the host (original/precomp.h): identical
    floats except where a device/host double sin/cos differs at a float
    rounding boundary (then 1 ulp)."""
    prob = Problem("coef", 40, 36, 28, absorb=6, kind="layered", layers=6, seed=11)
    m = prob.model()
    rng = np.random.default_rng(5)
    # per-cell angles and anisotropy too, not only layer values
    m[2] = rng.uniform(0, 0.3, prob.n).astype(np.float32)
    m[3] = (m[2] * rng.uniform(0, 1, prob.n)).astype(np.float32)
    m[4] = rng.uniform(-np.pi, np.pi, prob.n).astype(np.float32)
    m[5] = rng.uniform(-np.pi / 2, np.pi / 2, prob.n).astype(np.float32)
    prop = Propagator()
    prop.initialize(prob.sx, prob.sy, prob.sz, prob.bord, prob.dx, prob.dy, prob.dz, prob.dt, m)
    got = prop.coefficients()
    prop.finalize()
    ref = orc.precompute(m)
    ulp = np.abs(got.view(np.int32).astype(np.int64) - ref.view(np.int32).astype(np.int64))
    assert ulp.max() <= 1
    assert np.count_nonzero(ulp) <= 1e-4 * ulp.size


@pytest.mark.parametrize("name", ["tiny_homog", "tiny_layered", "tiny_maintti", "tiny_aniso"])
def test_small_cases_vs_reference(name, orc):
    prob, meta, g = load_golden(name)
    if name == "tiny_maintti":
        import sys
        sys.path.insert(0, os.path.dirname(GOLDEN))
        from golden.make_golden import main_tti_model

        raw = main_tti_model(prob.nx, prob.absorb, prob.steps)[1]
        m = orc.boundary(prob.sx, prob.sy, prob.sz, prob.nx, prob.ny, prob.nz, prob.bord, prob.absorb, raw, prob.seed)
    else:
        m = prob.model()
    p, q, _, _ = gpu_run(prob, m)
    assert rel_l2(p, g["p"]) < TOL_SHORT
    assert rel_l2(q, g["q"]) < TOL_SHORT
    assert np.max(np.abs(p - g["p"])) < TOL_SHORT * np.max(np.abs(g["p"]))


def test_c0_vs_reference(orc):
    prob, meta, g = load_golden("c0")
    p, q, _, _ = gpu_run(prob, prob.model())
    s = meta["stride"]
    assert rel_l2(subsample(p, prob, s), g["p"]) < TOL_SHORT
    assert rel_l2(subsample(q, prob, s), g["q"]) < TOL_SHORT
    np.testing.assert_allclose(plane_sums(p, prob), g["psum"], rtol=1e-4, atol=1e-12 * g["psum"].max())


def test_previous_fields_match_oracle(orc):
    """The previous-field buffers (pp, qp) after a run, including the source
    cell that the fused injection leaves to the next read."""
    prob, meta, g = load_golden("tiny_layered")
    m = prob.model()
    p, q, pp, qp = gpu_run(prob, m)
    op, oq, opp, oqp = orc.run_f32(prob, m)
    assert rel_l2(pp, opp) < TOL_SHORT and rel_l2(qp, oqp) < TOL_SHORT
    i = prob.i_source
    assert abs(pp[i] - opp[i]) <= 1e-5 * np.abs(opp).max()


@pytest.mark.parametrize("tile", [(12, 4, 1), (12, 4, 3), (16, 5, 2), (16, 4, 0), (8, 5, 5), (12, 5, 0), (12, 6, 0),
                                  (8, 5, 2), (16, 5, -1), (12, 4, -3)])
def test_tile_shapes_bit_identical(tile, orc):
    """Every tile shape, stage count and z-chunking computes identical floats,
    through both work-item modes: segment lists (zchunks >= 0 here: the
    small grid has fewer items than CTAs, so the plan shares them out) and
    arithmetic round-robin items (zchunks < 0)."""
    prob = Problem("shapes", 70, 27, 33, absorb=5, dt=0.0006, steps=24, fcut=45.0, kind="layered", layers=5,
                   seed=9)
    prob = prob.with_(source=(prob.sx // 2 + 1, prob.sy // 2, prob.sz // 2 + 2))
    m = prob.model()
    base = gpu_run(prob, m)
    got = gpu_run(prob, m, tile=tile)
    for a, b in zip(base, got):
        assert np.array_equal(a, b)
    op, oq, _, _ = orc.run_f32(prob, m)
    assert rel_l2(base[0], op) < TOL_SHORT and rel_l2(base[1], oq) < TOL_SHORT


@pytest.mark.parametrize("tile", [(12, 5, -1), (8, 5, -1), (16, 4, -1), (16, 5, 0), (16, 5, 3), (12, 5, 2)])
def test_tile_shapes_three_spacings(tile, orc):
    """dx, dy, dz all different (every derivative scaled on its own): every
    tile height, stage count and z split of the tile columns gives identical
    floats, as with equal spacings, and all match the oracle at the
    short-run tolerance."""
    prob = Problem("shapes3", 40, 28, 24, absorb=4, dx=10.0, dy=12.5, dz=15.0, dt=0.0005, steps=23, fcut=45.0,
                   kind="layered", layers=3, seed=21, source=(20, 16, 9))
    m = prob.model()
    base = gpu_run(prob, m, tile=(16, 5, -1))
    got = gpu_run(prob, m, tile=tile)
    for a, b in zip(base, got):
        assert np.array_equal(a, b), rel_l2(a, b)
    op, oq, _, _ = orc.run_f32(prob, m)
    assert rel_l2(got[0], op) < TOL_SHORT and rel_l2(got[1], oq) < TOL_SHORT


def test_run_entry_point_matches_driver_loop():
    prob = Problem("run", 30, 30, 30, absorb=5, dt=0.0006, steps=30, fcut=45.0, kind="layered", layers=3, seed=2)
    m = prob.model()
    a = gpu_run(prob, m)
    b = gpu_run(prob, m, use_run=True)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("case", ["odd_sizes", "bord6", "thin_z", "src_tile_edge", "src_in_border"])
def test_geometry_and_source_edge_cases(case, orc):
    base = Problem("edge", 21, 13, 9, absorb=3, dt=0.0006, steps=20, fcut=45.0, kind="layered", layers=3, seed=4)
    tile = (0, 0, 0)
    if case == "odd_sizes":
        prob = base                                                     # sx = 35, not a multiple of 32
    elif case == "bord6":
        prob = base.with_(bord=6)                                       # wider border than the stencil
    elif case == "thin_z":
        prob = base.with_(nz=1, nx=40, ny=37)                           # a few planes only
        tile = (12, 4, 3)
    elif case == "src_tile_edge":
        prob = Problem("edge2", 60, 40, 40, absorb=4, dt=0.0006, steps=20, fcut=45.0, seed=4)
        prob = prob.with_(source=(4 + 32, 4 + 12, 4 + 13))              # on a tile corner and a chunk edge
        tile = (12, 4, 3)
    else:
        prob = base.with_(source=(2, base.sy // 2, base.sz // 2))       # never updated: stored directly
    m = prob.model()
    p, q, pp, qp = gpu_run(prob, m, tile=tile)
    op, oq, opp, oqp = orc.run_f32(prob, m)
    assert rel_l2(p, op) < TOL_SHORT and rel_l2(q, oq) < TOL_SHORT
    assert rel_l2(pp, opp) < TOL_SHORT and rel_l2(qp, oqp) < TOL_SHORT
    if case == "src_in_border":
        i = prob.i_source
        assert p[i] == op[i] and pp[i] == opp[i]  # accumulated sources, never updated


def test_driver_call_order_semantics(orc):
    """Two sources before one step; Update_pointers between InsertSource and
    Propagate shows the source (as the reference's back-ends do)."""
    prob = Problem("order", 24, 24, 24, absorb=4, dt=0.0006, steps=6, fcut=45.0, seed=3)
    m = prob.model()
    prop = Propagator()
    prop.initialize(prob.sx, prob.sy, prob.sz, prob.bord, prob.dx, prob.dy, prob.dz, prob.dt, m)
    i1, i2 = prob.i_source, prob.i_source + 3
    n = prob.n
    pc = np.zeros(n, np.float32)
    # oracle: by hand, with the same call order
    o = orc.load()
    coef = orc.precompute(m)
    opp, opc, oqp, oqc = (np.zeros(n, np.float32) for _ in range(4))
    for it in range(1, prob.steps + 1):
        s1, s2 = np.float32(0.5 * it), np.float32(-0.25 * it)
        prop.insert_source(it - 1, i1, s1)
        prop.insert_source(it - 1, i2, s2)
        opc[i1] += s1; oqc[i1] += s1
        opc[i2] += s2; oqc[i2] += s2
        prop.update_pointers(pc)
        if it == 1:
            assert np.array_equal(pc, opc)  # only the two sources so far
        else:
            assert rel_l2(pc, opc) < TOL_SHORT
        prop.propagate(it)
        o.orc_propagate_f32(prob.sx, prob.sy, prob.sz, prob.bord, prob.dx, prob.dy, prob.dz, prob.dt,
                            opp.ctypes.data_as(orc.FP), opc.ctypes.data_as(orc.FP), oqp.ctypes.data_as(orc.FP),
                            oqc.ctypes.data_as(orc.FP), coef.ctypes.data_as(orc.FP))
        opp, opc = opc, opp
        oqp, oqc = oqc, oqp
    assert rel_l2(prop.field(0), opc) < TOL_SHORT
    assert rel_l2(prop.field(3), oqp) < TOL_SHORT
    prop.finalize()


def test_model_loop_with_snapshots(orc, lib):
    """FLETCHER_Model: the reference's Model() sequence with snapshots every
    0.01 s of simulated time, against the oracle."""
    import ctypes as C
    from fletcher_petrobras_gb300._lib import fptr

    prob = Problem("model", 32, 32, 32, absorb=8, dt=0.001, steps=45, fcut=40.0, seed=1)
    m = prob.model()
    n = prob.n
    f = [np.zeros(n, np.float32) for _ in range(4)]
    stats = (C.c_double * 5)()
    rc = lib.FLETCHER_Model(prob.steps, prob.i_source, prob.fcut, 0.01, prob.sx, prob.sy, prob.sz, prob.bord,
                            prob.dx, prob.dy, prob.dz, prob.dt, *[fptr(x) for x in f], *[fptr(m[k]) for k in range(6)],
                            stats)
    assert rc == 0
    op, oq, _, _ = orc.run_f32(prob, m)
    assert rel_l2(f[1], op) < TOL_SHORT and rel_l2(f[3], oq) < TOL_SHORT
    assert stats[1] > 0 and stats[4] >= 4 * n * 4  # four snapshots + final fields


@pytest.mark.skipif(not os.path.exists(os.path.join(GOLDEN, "golden_c1.npz")), reason="C1 fixture not generated")
def test_c1_full_size_vs_reference():
    """504^3 interior (576^3 grid), 1000 steps: relative L2 <= 1e-4 against the
    reference's FP32 OpenMP run, on every 12th cell of each axis and on the
    per-plane energy."""
    prob, meta, g = load_golden("c1")
    assert prob == C1.with_(name=prob.name)
    p, q, _, _ = gpu_run(prob, prob.model(), use_run=True)
    s = meta["stride"]
    ep, eq = rel_l2(subsample(p, prob, s), g["p"]), rel_l2(subsample(q, prob, s), g["q"])
    es = rel_l2(np.sqrt(plane_sums(p, prob)), np.sqrt(g["psum"]))
    print(f"C1 504^3 x 1000 steps vs reference: rel L2 p {ep:.3e} q {eq:.3e} plane energy {es:.3e}")
    assert ep < TOL_C1 and eq < TOL_C1 and es < TOL_C1


@pytest.mark.parametrize("name", ["d1d1_tiny_layered", "d1d1_c0", "d1d1_tiny_aniso"])
def test_vs_der1der1_reference(name, orc):
    """The GPU path against the der1der1/ tree's output (the Der1-Der1
    formulation): the same 1e-5 bound as against original/.  The GPU's
    mixed derivatives are first derivatives of first derivatives too, so it
    is closer to this tree than to original/'s 64-point sums."""
    prob, meta, g = load_golden(name)
    m = prob.model()
    p, q, _, _ = gpu_run(prob, m)
    s = meta["stride"]
    e_d1d1 = rel_l2(subsample(p, prob, s), g["p"])
    op, _, _, _ = orc.run_f32(prob, m)
    e_orig = rel_l2(subsample(p, prob, s), subsample(op, prob, s))
    print(f"{name}: GPU vs der1der1 {e_d1d1:.3g}, vs original {e_orig:.3g}")
    assert e_d1d1 < TOL_SHORT
    assert rel_l2(subsample(q, prob, s), g["q"]) < TOL_SHORT


def test_host_access_and_copy_paths_identical():
    """DRIVER_Initialize and the read-backs through the GPU's direct access
    to the caller's host arrays (where the device has it) and through
    device buffers and copies give identical coefficients and fields."""
    prob = Problem("hostmem", 30, 28, 26, absorb=4, dt=0.0006, steps=12, fcut=45.0, kind="layered", layers=3, seed=2)
    m = prob.model()
    g = np.random.default_rng(4)
    init = [(1e-3 * g.standard_normal(prob.n)).astype(np.float32) for _ in range(4)]
    out, modes = [], []
    for mode in (1, 0):
        prop = Propagator()
        prop.lib.FLETCHER_SetHostAccess(mode)
        prop.initialize(prob.sx, prob.sy, prob.sz, prob.bord, prob.dx, prob.dy, prob.dz, prob.dt, m, *init)
        modes.append(prop.lib.FLETCHER_HostAccess())
        prop.run(prob.steps, prob.i_source, prob.sources())
        prop.synchronize()
        out.append([prop.field(k) for k in range(4)] + [prop.coefficients()])
        prop.finalize()
        prop.lib.FLETCHER_SetHostAccess(0)
    print("direct host access:", modes)
    assert modes[1] == 0
    for a, b in zip(out[0], out[1]):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("stop", [1, 13])
def test_checkpoint_and_resume_bit_identical(stop):
    """Checkpoint / resume: the four fields read back after `stop` steps
    (FLETCHER_GetField: current and previous p and q, as the reference's
    arrays hold them, the last step's source included) are the initial state
    of a new DRIVER_Initialize, and the run continues with the source of step
    stop + 1 on.  The FP32 result equals the uninterrupted run's bit for bit."""
    prob = Problem("ckpt", 30, 26, 22, absorb=4, dt=0.0006, steps=24, fcut=45.0, kind="layered", layers=3, seed=5)
    m = prob.model()
    src = prob.sources()
    full = gpu_run(prob, m)
    prop = Propagator()
    prop.initialize(prob.sx, prob.sy, prob.sz, prob.bord, prob.dx, prob.dy, prob.dz, prob.dt, m)
    for it in range(1, stop + 1):
        prop.insert_source(it - 1, prob.i_source, src[it - 1])
        prop.propagate(it)
    pc, qc, pp, qp = (prop.field(k) for k in range(4))
    prop.finalize()
    prop = Propagator()
    prop.initialize(prob.sx, prob.sy, prob.sz, prob.bord, prob.dx, prob.dy, prob.dz, prob.dt, m,
                    pp=pp, pc=pc, qp=qp, qc=qc)
    for it in range(stop + 1, prob.steps + 1):
        prop.insert_source(it - 1, prob.i_source, src[it - 1])
        prop.propagate(it)
    resumed = [prop.field(k) for k in range(4)]
    prop.finalize()
    for a, b in zip(resumed, full):
        assert np.array_equal(a, b), rel_l2(a, b)


@pytest.mark.parametrize("kw", [{}, {"numerics": "d1d1"}, {"coef_layout": "media"}, {"tile_rows": 12, "stages": 5}])
def test_pitch_padding_is_never_read(kw):
    """NaN written into the pitch padding of the field buffers and the
    coefficient block (columns sx .. pitch-1, FLETCHER_DebugPoisonPadding)
    changes no result: the kernels read only the grid's own cells."""
    prob = Problem("pad", 37, 21, 15, absorb=4, dt=0.0006, steps=18, fcut=45.0, kind="layered", layers=3, seed=7)
    assert prob.sx % 32 != 0
    m = prob.model()
    src = prob.sources()
    out = []
    for poison in (False, True):
        prop = Propagator(**kw)
        prop.initialize(prob.sx, prob.sy, prob.sz, prob.bord, prob.dx, prob.dy, prob.dz, prob.dt, m)
        if poison:
            assert prop.lib.FLETCHER_DebugPoisonPadding(float("nan")) == 0
        for it in range(1, prob.steps + 1):
            prop.insert_source(it - 1, prob.i_source, src[it - 1])
            prop.propagate(it)
        out.append([prop.field(k) for k in range(4)])
        prop.finalize()
    Propagator()
    for a, b in zip(*out):
        assert np.isfinite(b).all()
        assert np.array_equal(a, b)
