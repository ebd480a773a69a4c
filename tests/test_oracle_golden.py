"""The oracle (CPU restatement) against fixtures produced by the reference's
own OpenMP build: bit-identical boundary, coefficients, source and fields."""
import hashlib

import numpy as np
import pytest

from conftest import GOLDEN, load_golden, plane_sums, subsample

SMALL = ["tiny_homog", "tiny_layered", "tiny_maintti", "tiny_aniso"]  # tiny_aniso: dx, dy, dz all differ


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def raw_for(name, prob):
    if name == "tiny_maintti":
        from golden.make_golden import main_tti_model  # noqa

        return main_tti_model(prob.nx, prob.absorb, prob.steps)[1]
    return prob.raw_model()


@pytest.fixture(scope="module", autouse=True)
def _path():
    import sys

    sys.path.insert(0, GOLDEN.rsplit("/", 1)[0])


@pytest.mark.parametrize("name", SMALL + ["c0"])
def test_boundary_and_coefficients(name, orc):
    prob, meta, _ = load_golden(name)
    raw = raw_for(name, prob)
    if "raw_sha" in meta:
        assert sha(raw) == meta["raw_sha"]
    m = orc.boundary(prob.sx, prob.sy, prob.sz, prob.nx, prob.ny, prob.nz, prob.bord, prob.absorb, raw, prob.seed)
    assert sha(m[0]) == meta["vpz_sha"]
    assert sha(m[1]) == meta["vsv_sha"]
    assert sha(orc.precompute(m)) == meta["coef_sha"]


@pytest.mark.parametrize("name", SMALL)
def test_fields_bit_identical(name, orc):
    prob, meta, g = load_golden(name)
    raw = raw_for(name, prob)
    m = orc.boundary(prob.sx, prob.sy, prob.sz, prob.nx, prob.ny, prob.nz, prob.bord, prob.absorb, raw, prob.seed)
    p, q, _, _ = orc.run_f32(prob, m)
    assert meta["stride"] == 1
    assert np.array_equal(p, g["p"])
    assert np.array_equal(q, g["q"])
    assert np.max(np.abs(p)) > 1e-3  # the wave has been injected


def test_c0_full_run(orc):
    prob, meta, g = load_golden("c0")
    m = orc.boundary(prob.sx, prob.sy, prob.sz, prob.nx, prob.ny, prob.nz, prob.bord, prob.absorb,
                     prob.raw_model(), prob.seed)
    p, q, _, _ = orc.run_f32(prob, m)
    s = meta["stride"]
    assert np.array_equal(subsample(p, prob, s), g["p"])
    assert np.array_equal(subsample(q, prob, s), g["q"])
    np.testing.assert_allclose(plane_sums(p, prob), g["psum"], rtol=1e-12, atol=0)


def test_source_matches_reference(orc):
    ref = np.load(f"{GOLDEN}/golden_source_fcut40.npy")
    got = np.array([orc.source(np.float32(0.001), i, 40.0) for i in range(len(ref))], np.float32)
    assert np.array_equal(got, ref)


def test_fp64_oracle_close_to_fp32(orc):
    """The FP64 restatement and the FP32 path agree to FP32 rounding on a short run."""
    prob, meta, g = load_golden("tiny_layered")
    m = orc.boundary(prob.sx, prob.sy, prob.sz, prob.nx, prob.ny, prob.nz, prob.bord, prob.absorb,
                     prob.raw_model(), prob.seed)
    p64, q64 = orc.run_f64(prob, m)
    assert orc.rel_l2(g["p"], p64) < 1e-5
    assert orc.rel_l2(g["q"], q64) < 1e-5


@pytest.mark.parametrize("name", ["d1d1_tiny_layered", "d1d1_c0", "d1d1_tiny_aniso"])
def test_der1der1_restatement_bit_identical(name, orc):
    """The Der1-Der1 restatement (orc_propagate_d1d1_f32) against the
    der1der1/ tree's own OpenMP build: identical floats."""
    prob, meta, g = load_golden(name)
    m = orc.boundary(prob.sx, prob.sy, prob.sz, prob.nx, prob.ny, prob.nz, prob.bord, prob.absorb,
                     prob.raw_model(), prob.seed)
    assert sha(m[0]) == meta["vpz_sha"]
    p, q, _, _ = orc.run_d1d1_f32(prob, m)
    s = meta["stride"]
    assert np.array_equal(subsample(p, prob, s), g["p"])
    assert np.array_equal(subsample(q, prob, s), g["q"])
    # the two formulations differ by rounding only
    op, oq, _, _ = orc.run_f32(prob, m)
    d = np.linalg.norm(p.astype(np.float64) - op) / np.linalg.norm(op)
    assert 0.0 < d < 1e-5
