"""FLETCHER_ReadFieldNoAlloc: the read-back for callers that cannot allocate
device memory (codes that reserve the whole GPU for their own volumes, or
whose time loop must not call cudaMalloc).  It must return exactly what the
regular read-back (FLETCHER_GetField) returns for the same field, call after
call, while allocating nothing itself.  The file name makes pytest collect it
last, so that if it fails, a run that stops at the first failure
(`pytest -x`) has already run every other test; it passes alone in a fresh
process as well as after the others."""
import ctypes as C

import numpy as np
import pytest

from conftest import gpu_available
from fletcher_petrobras_gb300 import Problem, Propagator
from fletcher_petrobras_gb300._lib import fptr, load

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not gpu_available():
        pytest.fail("these tests need a CUDA GPU")


def test_matches_regular_read_back_on_consecutive_calls():
    import torch

    lib = load()
    prob = Problem("noalloc", 20, 18, 16, absorb=4, dt=0.0006, steps=12, fcut=45.0, kind="layered", layers=3, seed=5)
    sx, sy, sz = prob.sx, prob.sy, prob.sz
    n = prob.n
    assert n <= 4 * 1024 * 1024  # FLETCHER_NOALLOC_MAX_CELLS
    prop = Propagator()
    prop.initialize(sx, sy, sz, prob.bord, prob.dx, prob.dy, prob.dz, prob.dt, prob.model())
    src = prob.sources()
    for it in range(1, prob.steps + 1):
        prop.insert_source(it - 1, prob.i_source, src[it - 1])
        prop.propagate(it)
    p, q = prop.field(0), prop.field(1)  # the regular entry point
    assert np.abs(p).max() > 0
    # The caller's own device volume of (p, q) pairs, with a pitch wider than sx.
    pitch = 64
    pairs = np.zeros((sz, sy, pitch, 2), np.float32)
    pairs[:, :, :sx, 0] = p.reshape(sz, sy, sx)
    pairs[:, :, :sx, 1] = q.reshape(sz, sy, sx)
    dev = torch.from_numpy(pairs).cuda()
    torch.cuda.synchronize()
    for comp, ref in [(0, p), (1, q), (0, p)]:  # consecutive calls share the staging array
        out = np.full(n, np.nan, np.float32)
        rc = lib.FLETCHER_ReadFieldNoAlloc(C.c_void_p(dev.data_ptr()), sx, sy, sz, pitch, comp, fptr(out))
        assert rc == 0, lib.FLETCHER_GetLastErrorString()
        assert np.array_equal(out, ref)  # data movement only: bit-identical
    prop.finalize()


def test_rejects_grids_beyond_the_staging_array():
    lib = load()
    lib.FLETCHER_ClearError()
    out = np.empty(1, np.float32)
    rc = lib.FLETCHER_ReadFieldNoAlloc(C.c_void_p(16), 256, 256, 65, 256, 0, fptr(out))  # 4,259,840 cells
    assert rc == 1
    assert b"exceeds" in lib.FLETCHER_GetLastErrorString()
    lib.FLETCHER_ClearError()


def test_orders_after_writes_on_the_callers_stream():
    """The volume is written on the caller's own stream, which is named with
    FLETCHER_SetStream; the read-back must see the finished writes without a
    device-wide synchronisation in between."""
    import torch

    lib = load()
    sx, sy, sz, pitch = 40, 24, 20, 48
    n = sx * sy * sz
    g = np.random.default_rng(11)
    vals = g.standard_normal((sz, sy, pitch, 2)).astype(np.float32)
    host = torch.from_numpy(vals).pin_memory()
    dev = torch.zeros((sz, sy, pitch, 2), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    side = torch.cuda.Stream()
    try:
        for comp in (0, 1):
            dev.zero_()
            torch.cuda.synchronize()
            with torch.cuda.stream(side):
                torch.cuda._sleep(20_000_000)  # keeps the stream busy ~10 ms before the write lands
                dev.copy_(host, non_blocking=True)
            assert lib.FLETCHER_SetStream(C.c_void_p(side.cuda_stream)) == 0
            out = np.full(n, np.nan, np.float32)
            rc = lib.FLETCHER_ReadFieldNoAlloc(C.c_void_p(dev.data_ptr()), sx, sy, sz, pitch, comp, fptr(out))
            assert rc == 0, lib.FLETCHER_GetLastErrorString()
            assert np.array_equal(out, vals[:, :, :sx, comp].ravel())
    finally:
        lib.FLETCHER_SetStream(None)
        torch.cuda.synchronize()
