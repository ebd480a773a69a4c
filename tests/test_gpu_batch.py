"""Batched shots (one persistent launch per step for all running shots, CUDA
graph time loop) against single-shot runs of the same shots and the oracle.

The batched kernel evaluates every cell with the same operations as the
single-shot kernel, so each shot's fields must be bit-identical to its own
single-shot run, whatever the other shots in the batch and whether the loop
runs from a CUDA graph; the oracle bounds them at relative L2 1e-5.  The
same holds for the 16-bit storage forms: a shot's per-plane scales depend
only on its own field's maxima, so a batched FP16 or FP16X shot is
bit-identical to its single-shot run in that form."""
import numpy as np
import pytest

from conftest import gpu_available
from fletcher_petrobras_gb300 import Problem, Propagator
from fletcher_petrobras_gb300.batch import Batch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not gpu_available():
        pytest.fail("these tests need a CUDA GPU")


def rel_l2(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(np.asarray(b, np.float64)))


def single(prob, model, form="fp32"):
    prop = Propagator(form=form)
    prop.initialize(prob.sx, prob.sy, prob.sz, prob.bord, prob.dx, prob.dy, prob.dz, prob.dt, model)
    prop.run(prob.steps, prob.i_source, prob.sources())
    prop.synchronize()
    out = [prop.field(k) for k in range(4)]
    prop.finalize()
    return out


SHOTS = [
    Problem("b0", 40, 28, 24, absorb=4, dt=0.0006, steps=23, fcut=45.0, kind="layered", layers=3, seed=21,
            source=(20, 16, 9)),
    Problem("b1", 21, 33, 17, absorb=5, dt=0.0006, steps=31, fcut=45.0, kind="layered", layers=4, seed=22,
            source=(15, 20, 12)),
    Problem("b2", 64, 16, 40, absorb=3, dt=0.0006, steps=9, fcut=45.0, kind="layered", layers=2, seed=23,
            source=(30, 10, 20)),
]


@pytest.mark.parametrize("use_graph", [True, False])
def test_batch_matches_single_shot_runs(use_graph, orc):
    models = [p.model() for p in SHOTS]
    batch = Batch()
    for p, m in zip(SHOTS, models):
        batch.add(p, m)
    batch.run(use_graph=use_graph)
    got = [[batch.field(i, k) for k in range(4)] for i in range(len(SHOTS))]
    info = batch.info()
    batch.close()
    assert info["launches"] == max(p.steps for p in SHOTS)
    for i, (p, m) in enumerate(zip(SHOTS, models)):
        ref = single(p, m)
        for k in range(4):
            assert np.array_equal(got[i][k], ref[k]), (i, k)
        op, oq, _, _ = orc.run_f32(p, m)
        assert rel_l2(got[i][0], op) < 1e-5 and rel_l2(got[i][1], oq) < 1e-5


def test_batch_tile_shapes_and_rerun_identical():
    models = [p.model() for p in SHOTS]
    batch = Batch()
    for p, m in zip(SHOTS, models):
        batch.add(p, m)
    batch.run()
    a = [batch.field(i, 0) for i in range(len(SHOTS))]
    batch.reset()
    batch.set_tile(12, 5)  # the default is 16 x 5
    batch.run()
    b = [batch.field(i, 0) for i in range(len(SHOTS))]
    batch.close()
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("form", ["fp16", "fp16x"])
def test_half_batch_matches_single_shot_runs(form):
    models = [p.model() for p in SHOTS]
    batch = Batch(form=form)
    for p, m in zip(SHOTS, models):
        batch.add(p, m)
    batch.run()
    got = [[batch.field(i, k) for k in range(4)] for i in range(len(SHOTS))]
    info = batch.info()
    # Another tile shape and the loop without a graph give the same fields.
    batch.reset()
    batch.set_tile(12, 5)
    batch.run(use_graph=False)
    again = [batch.field(i, 0) for i in range(len(SHOTS))]
    batch.close()
    # Two launches per step: the plane scales of every running shot, then the step.
    assert info["launches"] == 2 * max(p.steps for p in SHOTS)
    for i, (p, m) in enumerate(zip(SHOTS, models)):
        ref = single(p, m, form)
        assert np.abs(ref[0]).max() > 0.0
        for k in range(4):
            assert np.array_equal(got[i][k], ref[k]), (form, i, k)
        assert np.array_equal(again[i], ref[0]), (form, i)


@pytest.mark.parametrize("form", ["fp32", "fp16x"])
def test_batch_with_three_spacings_matches_single_shot_runs(form, orc):
    """dx, dy, dz all different (the kernels' non-isotropic path): the rings
    and the exchange hold unscaled first derivatives and each cross
    derivative takes one combined factor, so a cell's floats do not depend
    on how its tile column is split in z -- batched shots equal their
    single-shot runs bit for bit, and the oracle bounds them."""
    sp = dict(dx=10.0, dy=12.5, dz=15.0, dt=0.0005)
    shots = [s.with_(**sp) for s in SHOTS[:2]]
    models = [p.model() for p in shots]
    batch = Batch(dx=sp["dx"], dy=sp["dy"], dz=sp["dz"], dt=sp["dt"], form=form)
    for p, m in zip(shots, models):
        batch.add(p, m)
    batch.run()
    got = [[batch.field(i, k) for k in range(4)] for i in range(len(shots))]
    batch.close()
    for i, (p, m) in enumerate(zip(shots, models)):
        ref = single(p, m, form)
        for k in range(4):
            assert np.array_equal(got[i][k], ref[k]), (form, i, k, rel_l2(got[i][k], ref[k]))
        op, oq, _, _ = orc.run_f32(p, m)
        tol = 1e-5 if form == "fp32" else 1e-4
        assert rel_l2(got[i][0], op) < tol and rel_l2(got[i][1], oq) < tol


@pytest.mark.parametrize("form", ["fp32", "fp16", "fp16x"])
def test_deep_shots_split_in_z_match_single_shot_runs(form):
    """Shots deeper than one 128-plane chunk: each tile column is several
    batch items, and the shot's fields still equal its single-shot run."""
    shots = [
        Problem("deep0", 40, 30, 150, absorb=4, dt=0.0006, steps=16, fcut=45.0, kind="layered", layers=4, seed=31,
                source=(20, 15, 60)),
        Problem("deep1", 33, 20, 262, absorb=3, dt=0.0006, steps=11, fcut=45.0, kind="layered", layers=5, seed=32,
                source=(18, 12, 140)),
    ]
    models = [p.model() for p in shots]
    batch = Batch(form=form)
    for p, m in zip(shots, models):
        batch.add(p, m)
    batch.run()
    got = [[batch.field(i, k) for k in range(4)] for i in range(len(shots))]
    batch.close()
    for i, (p, m) in enumerate(zip(shots, models)):
        ref = single(p, m, form)
        assert np.abs(ref[0]).max() > 0.0
        for k in range(4):
            assert np.array_equal(got[i][k], ref[k]), (form, i, k)


@pytest.mark.parametrize("chains", [1, 2, 3])
@pytest.mark.parametrize("use_graph", [True, False])
def test_chain_schedule_matches_single_shot_runs(chains, use_graph):
    """FLETCHER_BatchSetChains: each shot's steps as single-shot launches on
    one of `chains` concurrent streams.  Shots whose plans share out their
    last round (segment lists) and shots on round-robin chunks (tile items),
    three spacings included: every shot equals its own single-shot run."""
    shots = SHOTS + [
        Problem("c3", 70, 60, 150, absorb=5, dt=0.0006, steps=13, fcut=45.0, kind="layered", layers=4, seed=33,
                source=(35, 30, 70)),
        SHOTS[0].with_(name="c4", dx=10.0, dy=12.5, dz=15.0, dt=0.0005),
    ]
    models = [p.model() for p in shots]
    batch = Batch(chains=chains, dx=12.5, dy=12.5, dz=12.5)
    for p, m in zip(shots[:-1], models[:-1]):
        batch.add(p, m)
    batch.run(use_graph=use_graph)
    got = [[batch.field(i, k) for k in range(4)] for i in range(len(shots) - 1)]
    info = batch.info()
    batch.close()
    assert info["launches"] == sum(p.steps for p in shots[:-1])
    for i, (p, m) in enumerate(zip(shots[:-1], models[:-1])):
        ref = single(p, m)
        assert np.abs(ref[0]).max() > 0.0
        for k in range(4):
            assert np.array_equal(got[i][k], ref[k]), (chains, i, k)
    # A three-spacing batch on the chain schedule.
    p, m = shots[-1], models[-1]
    batch = Batch(chains=chains, dx=p.dx, dy=p.dy, dz=p.dz, dt=p.dt)
    batch.add(p, m)
    batch.run(use_graph=use_graph)
    got = [batch.field(0, k) for k in range(4)]
    batch.close()
    ref = single(p, m)
    for k in range(4):
        assert np.array_equal(got[k], ref[k]), (chains, "three spacings", k)



def test_default_schedule_follows_shot_size():
    """FLETCHER_BatchSetChains(-1), the default: small shots share the
    persistent launch; a batch whose work is mostly in shots of at least
    2.1 M updated cells (they fill the GPU on their own) runs one chain.
    Both give each shot its single-shot fields."""
    small = SHOTS[:2]
    big = Problem("big", 136, 120, 128, absorb=4, dt=0.0006, steps=6, fcut=45.0, kind="layered", layers=3, seed=41,
                  source=(70, 64, 60))
    assert (big.sx - 8) * (big.sy - 8) * (big.sz - 8) >= 2.1e6
    for shots, want in ((small, 0), ([big] + small, 1)):
        models = [p.model() for p in shots]
        batch = Batch()
        for p, m in zip(shots, models):
            batch.add(p, m)
        batch.run()
        got = [batch.field(i, 0) for i in range(len(shots))]
        chains = batch.info()["chains"]
        batch.close()
        assert chains == want
        for i, (p, m) in enumerate(zip(shots, models)):
            assert np.array_equal(got[i], single(p, m)[0]), (want, i)


@pytest.mark.parametrize("form", ["fp16", "fp16x"])
@pytest.mark.parametrize("chains", [1, 2])
def test_half_chain_schedule_matches_single_shot_runs(form, chains):
    """The chain schedule in the 16-bit forms: each step of a shot is the
    single-shot pair of launches (plane scales, step) on its chain's stream;
    every shot equals its single-shot run in that form, graph or not."""
    shots = SHOTS + [Problem("h3", 70, 60, 150, absorb=5, dt=0.0006, steps=13, fcut=45.0, kind="layered", layers=4,
                             seed=34, source=(35, 30, 70))]
    models = [p.model() for p in shots]
    for use_graph in (True, False):
        batch = Batch(form=form, chains=chains)
        for p, m in zip(shots, models):
            batch.add(p, m)
        batch.run(use_graph=use_graph)
        got = [[batch.field(i, k) for k in range(4)] for i in range(len(shots))]
        info = batch.info()
        batch.close()
        assert info["chains"] == chains
        for i, (p, m) in enumerate(zip(shots, models)):
            ref = single(p, m, form)
            assert np.abs(ref[0]).max() > 0.0
            for k in range(4):
                assert np.array_equal(got[i][k], ref[k]), (form, chains, use_graph, i, k)
