import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a); runs the CUDA path through the C ABI")
    config.addinivalue_line("markers", "slow: long-running")


def load_golden(name: str):
    """Returns (Problem, fixture dict) for tests/golden/golden_<name>.npz."""
    from fletcher_petrobras_gb300.models import Problem

    d = np.load(os.path.join(GOLDEN, f"golden_{name}.npz"))
    meta = json.loads(str(d["meta"]))
    fields = {f for f in Problem.__dataclass_fields__}
    kw = {k: (tuple(v) if isinstance(v, list) else v) for k, v in meta.items() if k in fields}
    return Problem(**kw), meta, {k: d[k] for k in ("p", "q", "psum", "qsum")}


def subsample(f, prob, stride):
    return np.ascontiguousarray(np.asarray(f).reshape(prob.sz, prob.sy, prob.sx)[::stride, ::stride, ::stride]).ravel()


def plane_sums(f, prob):
    v = np.asarray(f, np.float64).reshape(prob.sz, -1)
    return np.sum(v * v, axis=1)


@pytest.fixture(scope="session")
def lib():
    from fletcher_petrobras_gb300 import _lib

    return _lib.load()


@pytest.fixture(scope="session")
def orc():
    import oracle

    oracle.load()
    return oracle


def reference_dir():
    """The reference checkout's root (holding original/ and der1der1/):
    $FLETCHER_REF_DIR when set, else the copy staged by `make -C oracle stage`
    in oracle/_ref/src; None when neither holds original/main.c."""
    d = os.environ.get("FLETCHER_REF_DIR") or os.path.join(ROOT, "oracle", "_ref", "src")
    return d if os.path.isfile(os.path.join(d, "original", "main.c")) else None


def gpu_available() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False
