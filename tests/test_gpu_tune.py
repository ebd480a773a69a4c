"""Online tile-shape tuning on the GPU (FLETCHER_Autotune): the tuning steps
are real steps -- a tuned run is bit-identical to an untuned one -- and the
chosen shape is stored and reused from the configuration file."""
import ctypes as C

import numpy as np
import pytest

from conftest import gpu_available
from fletcher_petrobras_gb300 import Problem, Propagator

pytestmark = pytest.mark.gpu

PROB = Problem("tune", 70, 40, 30, absorb=4, dt=0.0006, steps=30, fcut=45.0, kind="layered", layers=3, seed=5)


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not gpu_available():
        pytest.fail("these tests need a CUDA GPU")


def run(path=None, form="fp32"):
    p = PROB
    prop = Propagator(form=form)
    prop.initialize(p.sx, p.sy, p.sz, p.bord, p.dx, p.dy, p.dz, p.dt, p.model())
    found = None
    if path is not None:
        found = prop.lib.FLETCHER_Autotune(path, 2)
    prop.run(p.steps, p.i_source, p.sources())
    prop.synchronize()
    r, s = C.c_int(0), C.c_int(0)
    tuning = prop.lib.FLETCHER_GetTileConfig(C.byref(r), C.byref(s))
    out = [prop.field(k) for k in range(4)]
    prop.finalize()
    Propagator(form="fp32")
    return out, found, tuning, (r.value, s.value)


@pytest.mark.parametrize("form", ["fp32", "fp16x"])
def test_autotune_is_transparent_and_persists(tmp_path, form):
    path = str(tmp_path / "configurations.txt").encode()
    base, _, _, _ = run(form=form)
    tuned, found, tuning, shape = run(path, form)
    assert found == 0 and tuning == 0
    for a, b in zip(base, tuned):
        assert np.array_equal(a, b)
    lines = open(path).read().splitlines()
    assert len(lines) == 1 and lines[0].endswith(" | " + form)
    again, found2, tuning2, shape2 = run(path, form)
    assert found2 == 1 and tuning2 == 0 and shape2 == shape
    for a, b in zip(base, again):
        assert np.array_equal(a, b)
    assert len(open(path).read().splitlines()) == 1
