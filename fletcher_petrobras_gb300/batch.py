"""Batched shots: many independent Fletcher runs in one persistent launch per
time step (C ABI `FLETCHER_Batch*`), and the seeded batch used for the
multi-shot measurement.

`multishot_spec(nshots, seed)` draws, per shot: nx, ny, nz ~ U{96..320} in
multiples of 8, an 8-layer TTI model from the layered generator seeded with
the shot's own seed (absorb 32, bord 4, dx 12.5 m), a source cell in the top
quarter of the interior, and 500..1500 steps at dt = 0.6 ms, 15 Hz Ricker.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import fptr
from .driver import FORMS, FletcherError, _check
from .models import Problem


def multishot_spec(nshots: int = 48, seed: int = 0, nmin: int = 96, nmax: int = 320, steps=(500, 1500),
                   absorb: int = 32) -> list:
    """Seeded list of Problems for the batched configuration."""
    rng = np.random.default_rng(seed)
    out = []
    for s in range(nshots):
        nx, ny, nz = (int(v) for v in rng.integers(nmin // 8, nmax // 8 + 1, size=3) * 8)
        st = int(rng.integers(steps[0], steps[1] + 1))
        bord = 4
        b = bord + absorb
        src = (b + int(rng.integers(0, nx)), b + int(rng.integers(0, ny)), b + int(rng.integers(0, max(1, nz // 4))))
        out.append(Problem(f"shot{s}", nx, ny, nz, absorb=absorb, bord=bord, dt=0.0006, steps=st, fcut=45.0,
                           kind="layered", seed=1000 + s, source=src))
    return out


class Batch:
    """A batch of shots resident on the GPU (one per process)."""

    def __init__(self, bord=4, dx=12.5, dy=12.5, dz=12.5, dt=0.0006, form: str = "fp32", chains: int | None = None):
        """form: storage form of every shot's fields ("fp32", "fp16", "fp16x").
        chains: schedule of an FP32 batch (FLETCHER_BatchSetChains; None keeps
        the library's default)."""
        self.lib = _lib.load()
        self.lib.FLETCHER_ClearError()
        if form not in FORMS:
            raise ValueError(f"unknown form {form!r}; one of {sorted(FORMS)}")
        self.form = form
        if self.lib.FLETCHER_SetForm(FORMS[form]):
            _check(self.lib, "SetForm")
        if self.lib.FLETCHER_BatchCreate(bord, dx, dy, dz, dt):
            _check(self.lib, "FLETCHER_BatchCreate")
        if chains is not None and self.lib.FLETCHER_BatchSetChains(int(chains)):
            _check(self.lib, "FLETCHER_BatchSetChains")
        self.dt = dt
        self.probs = []

    def add(self, prob: Problem, model: np.ndarray | None = None) -> int:
        m = prob.model() if model is None else np.ascontiguousarray(model, np.float32)
        r = self.lib.FLETCHER_BatchAddShot(prob.sx, prob.sy, prob.sz, fptr(m), prob.i_source, prob.steps)
        if r < 0:
            _check(self.lib, "FLETCHER_BatchAddShot")
            raise FletcherError("FLETCHER_BatchAddShot failed")
        self.probs.append(prob)
        return r

    def set_tile(self, rows=0, stages=0):
        if self.lib.FLETCHER_BatchSetTileConfig(rows, stages):
            _check(self.lib, "FLETCHER_BatchSetTileConfig")

    def run(self, use_graph: bool = True, fcut: float | None = None, max_steps: int = 0) -> float:
        """Runs every shot for its own step count (or the first max_steps steps);
        returns the device time in ms."""
        steps = max(p.steps for p in self.probs)
        fc = self.probs[0].fcut if fcut is None else fcut
        src = np.array([self.lib.FLETCHER_Source(self.dt, it, fc) for it in range(steps)], np.float32)
        ms = C.c_float(0.0)
        if self.lib.FLETCHER_BatchRun(fptr(src), int(max_steps), 1 if use_graph else 0, C.byref(ms)):
            _check(self.lib, "FLETCHER_BatchRun")
        return float(ms.value)

    def reset(self):
        if self.lib.FLETCHER_BatchReset():
            _check(self.lib, "FLETCHER_BatchReset")

    def field(self, shot: int, which: int) -> np.ndarray:
        p = self.probs[shot]
        out = np.empty(p.n, np.float32)
        if self.lib.FLETCHER_BatchGetField(shot, which, fptr(out)):
            _check(self.lib, "FLETCHER_BatchGetField")
        return out

    def info(self) -> dict:
        ns, cs, la, db = C.c_long(0), C.c_double(0), C.c_long(0), C.c_size_t(0)
        self.lib.FLETCHER_BatchInfo(C.byref(ns), C.byref(cs), C.byref(la), C.byref(db))
        return {"shots": ns.value, "cell_steps": cs.value, "launches": la.value, "device_bytes": db.value,
                "chains": self.lib.FLETCHER_BatchLastChains()}

    def close(self):
        self.lib.FLETCHER_BatchDestroy()


def shape_class(probs) -> str:
    """Cache key part: shot count and the rounded median interior size."""
    ns = sorted(p.nx * p.ny * p.nz for p in probs)
    med = int(round(ns[len(ns) // 2] ** (1 / 3) / 32.0)) * 32
    return f"batch{len(probs)}-n{med}"
