"""Asynchronous output path on the GPU, through the C ABI: snapshots and
slice appends taken while steps keep running must equal the synchronous
read-back (FLETCHER_GetField) of the same step, bit for bit, in the FP32
and FP16X forms, into page-locked and ordinary host buffers."""
import os

import numpy as np
import pytest

from conftest import gpu_available
from fletcher_petrobras_gb300 import Problem, Propagator
from fletcher_petrobras_gb300._lib import fptr

pytestmark = pytest.mark.gpu

PROB = Problem("snap", 40, 30, 24, absorb=5, dt=0.0006, steps=40, fcut=45.0, kind="layered", layers=3, seed=8)


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not gpu_available():
        pytest.fail("these tests need a CUDA GPU")


def start(form):
    prop = Propagator(form=form)
    p = PROB
    prop.initialize(p.sx, p.sy, p.sz, p.bord, p.dx, p.dy, p.dz, p.dt, p.model())
    return prop


@pytest.mark.parametrize("form", ["fp32", "fp16x"])
@pytest.mark.parametrize("pinned", [False, True])
def test_snapshot_equals_field_of_its_step(form, pinned):
    prop = start(form)
    lib = prop.lib
    src = PROB.sources()
    prop.run(20, PROB.i_source, src[:20])
    n = PROB.n
    outs = [np.full(n, np.nan, np.float32) for _ in range(4)]
    if pinned:
        for o in outs:
            assert lib.FLETCHER_PinHost(o.ctypes.data, o.nbytes) == 0
    for k in range(4):
        assert lib.FLETCHER_SnapshotBegin(k, fptr(outs[k])) == 0
    prop.run(20, PROB.i_source, src[20:])  # overlaps the copies
    assert lib.FLETCHER_SnapshotWait() == 0
    after = [prop.field(k) for k in range(4)]
    prop.finalize()
    # the same state, run to step 20 only
    prop = start(form)
    prop.run(20, PROB.i_source, src[:20])
    want = [prop.field(k) for k in range(4)]
    prop.finalize()
    Propagator(form="fp32")
    if pinned:
        for o in outs:
            lib.FLETCHER_UnpinHost(o.ctypes.data)
    for k in range(4):
        assert np.array_equal(outs[k], want[k]), k
        assert not np.array_equal(outs[k], after[k])


def test_slice_append_equals_host_slice_file(tmp_path, monkeypatch):
    prop = start("fp32")
    lib = prop.lib
    p = PROB
    monkeypatch.chdir(tmp_path)
    box = (4, p.sx - 5, p.sy // 2, p.sy // 2, 4, p.sz - 5)  # a y-slice
    a = lib.FLETCHER_OpenSliceFile(*box, p.dx, p.dz, p.dz, p.dt, b"async")
    h = lib.FLETCHER_OpenSliceFile(*box, p.dx, p.dz, p.dz, p.dt, b"host")
    src = p.sources()
    for it in range(0, 40, 10):
        prop.run(10, p.i_source, src[it:it + 10])
        assert lib.FLETCHER_SliceAppend(a, 0) == 0
        f = prop.field(0)
        assert lib.FLETCHER_DumpSliceFile(p.sx, p.sy, p.sz, fptr(f), h) == 0
    assert lib.FLETCHER_CloseSliceFile(a) == 0 and lib.FLETCHER_CloseSliceFile(h) == 0
    prop.finalize()
    for ext in (".rsf", ".rsf@"):
        x = open(os.path.join(tmp_path, "async" + ext), "rb").read()
        y = open(os.path.join(tmp_path, "host" + ext), "rb").read()
        assert x.replace(b"async", b"host") == y, ext
    assert os.path.getsize(os.path.join(tmp_path, "host.rsf@")) == 4 * 4 * (box[1] - box[0] + 1) * (box[5] - box[4] + 1)


def test_model_loop_snapshots_land_in_the_callers_arrays():
    """FLETCHER_Model with a snapshot cadence: the asynchronous snapshots
    leave the last one in a host p array and the final fields in pc / qc."""
    import ctypes as C

    p = PROB
    prop = Propagator()
    lib = prop.lib
    m = p.model()
    f = np.zeros((4, p.n), np.float32)
    stats = (C.c_double * 5)()
    rc = lib.FLETCHER_Model(p.steps, p.i_source, p.fcut, 0.003, p.sx, p.sy, p.sz, p.bord, p.dx, p.dy, p.dz, p.dt,
                            *[fptr(f[k]) for k in range(4)], *[fptr(m[k]) for k in range(6)], stats)
    assert rc == 0
    prop2 = Propagator()
    prop2.initialize(p.sx, p.sy, p.sz, p.bord, p.dx, p.dy, p.dz, p.dt, m)
    src = p.sources()
    prop2.run(p.steps, p.i_source, src)
    want_p, want_q = prop2.field(0), prop2.field(1)
    prop2.finalize()
    assert np.array_equal(f[1], want_p) and np.array_equal(f[3], want_q)
    assert stats[4] > 2 * 4 * p.n  # snapshots were taken


def test_consecutive_snapshots_each_hold_their_step(tmp_path, monkeypatch):
    """Snapshots one step apart use the two device buffers in turn (and a
    slice append in between uses the first): each copy still holds the field
    of its own step, while the steps after it run."""
    prop = start("fp32")
    lib = prop.lib
    p = PROB
    monkeypatch.chdir(tmp_path)
    src = p.sources()
    n = p.n
    at = [5, 6, 7, 9]
    outs = [np.full(n, np.nan, np.float32) for _ in at]
    box = (4, p.sx - 5, 4, p.sy - 5, p.sz // 2, p.sz // 2)  # a z-slice
    sl = lib.FLETCHER_OpenSliceFile(*box, p.dx, p.dy, p.dz, p.dt, b"mid")
    done = 0
    for i, step in enumerate(at):
        prop.run(step - done, p.i_source, src[done:step])
        done = step
        assert lib.FLETCHER_SnapshotBegin(0, fptr(outs[i])) == 0
        if i == 1:
            assert lib.FLETCHER_SliceAppend(sl, 0) == 0
    prop.run(10, p.i_source, src[done:done + 10])
    assert lib.FLETCHER_SnapshotWait() == 0
    assert lib.FLETCHER_CloseSliceFile(sl) == 0
    prop.finalize()
    prop = start("fp32")
    want = []
    done = 0
    for step in at:
        prop.run(step - done, p.i_source, src[done:step])
        done = step
        want.append(prop.field(0))
    prop.finalize()
    for o, w in zip(outs, want):
        assert np.array_equal(o, w)
    # The slice holds step 6: the host writer on that step's field gives the same file.
    h = lib.FLETCHER_OpenSliceFile(*box, p.dx, p.dy, p.dz, p.dt, b"ref")
    assert lib.FLETCHER_DumpSliceFile(p.sx, p.sy, p.sz, fptr(want[1]), h) == 0
    assert lib.FLETCHER_CloseSliceFile(h) == 0
    x = open(os.path.join(tmp_path, "mid.rsf@"), "rb").read()
    y = open(os.path.join(tmp_path, "ref.rsf@"), "rb").read()
    assert len(x) == 4 * (box[1] - box[0] + 1) * (box[3] - box[2] + 1) and x == y


def test_model_loop_with_page_locked_caller_arrays():
    """The caller's arrays already page-locked (cudaHostAlloc'd by torch):
    the library's own locking of them fails, is not an error, and leaves no
    CUDA error state behind; the run equals one on ordinary arrays."""
    import ctypes as C

    import torch

    p = PROB
    m = p.model()
    outs = []
    for pinned in (False, True):
        if pinned:
            tf = torch.zeros((4, p.n), dtype=torch.float32, pin_memory=True)
            tm = torch.empty((6, p.n), dtype=torch.float32, pin_memory=True)
            f, mm = tf.numpy(), tm.numpy()
            mm[...] = m
        else:
            f, mm = np.zeros((4, p.n), np.float32), m
        lib = Propagator().lib
        stats = (C.c_double * 5)()
        rc = lib.FLETCHER_Model(p.steps, p.i_source, p.fcut, 0.003, p.sx, p.sy, p.sz, p.bord, p.dx, p.dy, p.dz, p.dt,
                                *[fptr(f[k]) for k in range(4)], *[fptr(mm[k]) for k in range(6)], stats)
        assert rc == 0, lib.FLETCHER_GetLastErrorString()
        outs.append(f.copy())
    assert np.array_equal(outs[0], outs[1])
