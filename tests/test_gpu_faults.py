"""Failure detection, exercised without faulting the GPU.

* A stalled pipeline: FLETCHER_InjectFault(FLETCHER_FAULT_STALL, n, wait_us)
  makes CTA 0 of the next propagate launch skip the loads of its n-th step.
  Its bounded waits for that stage run out after wait_us (the kernel's own
  limit is 2 s), it drains the loads it has in flight and returns; the host
  reads the error word and DRIVER_Propagate reports FLETCHER_ERR_TIMEOUT.
  Nothing waits forever and no address is touched out of bounds.  The
  process then re-initialises and runs a correct simulation.
* An allocation failure: FLETCHER_FAULT_ALLOC fails one device allocation of
  DRIVER_Initialize (host-side fake of cudaMalloc); the call reports
  FLETCHER_ERR_NOMEM, releases the rest, and the next set-up succeeds.
* Non-finite model values are rejected at set-up, naming array and cell.
"""
import numpy as np
import pytest

from conftest import gpu_available
from fletcher_petrobras_gb300 import FletcherError, Problem, Propagator

pytestmark = pytest.mark.gpu

FAULT_NONE, FAULT_ALLOC, FAULT_STALL = 0, 1, 2
ERR_TIMEOUT, ERR_NOMEM, ERR_ARGS = 3, 4, 1

PROB = Problem("faults", 36, 30, 28, absorb=5, dt=0.0006, steps=12, fcut=45.0, kind="layered", layers=3, seed=6)


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not gpu_available():
        pytest.fail("these tests need a CUDA GPU")


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def clean_run(orc, prob=PROB):
    """A full run after a failure, checked against the oracle."""
    m = prob.model()
    prop = Propagator()
    prop.initialize(prob.sx, prob.sy, prob.sz, prob.bord, prob.dx, prob.dy, prob.dz, prob.dt, m)
    prop.run(prob.steps, prob.i_source, prob.sources())
    prop.synchronize()
    p, q = prop.field(0), prop.field(1)
    prop.finalize()
    op, oq, _, _ = orc.run_f32(prob, m)
    assert rel_l2(p, op) < 1e-5 and rel_l2(q, oq) < 1e-5


@pytest.mark.parametrize("stall_step", [0, 5])
def test_stalled_pipeline_reports_timeout_then_recovers(stall_step, orc):
    prop = Propagator()
    lib = prop.lib
    m = PROB.model()
    prop.initialize(PROB.sx, PROB.sy, PROB.sz, PROB.bord, PROB.dx, PROB.dy, PROB.dz, PROB.dt, m)
    prop.propagate(1)  # a normal step first
    assert lib.FLETCHER_InjectFault(FAULT_STALL, stall_step, 20000) == 0
    with pytest.raises(FletcherError, match=r"gave up waiting.*\(code 3\)"):
        prop.propagate(2)
    # The injection applied to that one launch only.
    lib.FLETCHER_ClearError()
    prop.finalize()
    clean_run(orc)


def test_stall_argument_checks():
    lib = Propagator().lib
    lib.FLETCHER_ClearError()
    assert lib.FLETCHER_InjectFault(FAULT_STALL, 0, 10) == ERR_ARGS  # wait below 1 ms
    lib.FLETCHER_ClearError()
    assert lib.FLETCHER_InjectFault(FAULT_STALL, -1, 20000) == ERR_ARGS
    lib.FLETCHER_ClearError()
    assert lib.FLETCHER_InjectFault(7, 0, 0) == ERR_ARGS
    lib.FLETCHER_ClearError()
    assert lib.FLETCHER_InjectFault(FAULT_NONE, 0, 0) == 0


@pytest.mark.parametrize("which", [0, 2, 4])
def test_allocation_failure_reports_nomem_then_recovers(which, orc):
    prop = Propagator()
    lib = prop.lib
    assert lib.FLETCHER_InjectFault(FAULT_ALLOC, which, 0) == 0
    with pytest.raises(FletcherError, match=r"\(code 4\)"):
        prop.initialize(PROB.sx, PROB.sy, PROB.sz, PROB.bord, PROB.dx, PROB.dy, PROB.dz, PROB.dt, PROB.model())
    assert lib.FLETCHER_DeviceBytes() == 0  # nothing kept
    lib.FLETCHER_InjectFault(FAULT_NONE, 0, 0)
    clean_run(orc)


@pytest.mark.parametrize("array,value", [(2, np.nan), (0, np.inf), (5, -np.inf)])
def test_non_finite_model_values_rejected(array, value, orc):
    m = PROB.model()
    cell = PROB.n // 3 + 7
    m[array, cell] = value
    names = ["vpz", "vsv", "epsilon", "delta", "phi", "theta"]
    prop = Propagator()
    with pytest.raises(FletcherError, match=rf"{names[array]} holds a value that is not finite at cell {cell}"):
        prop.initialize(PROB.sx, PROB.sy, PROB.sz, PROB.bord, PROB.dx, PROB.dy, PROB.dz, PROB.dt, m)
    clean_run(orc)
