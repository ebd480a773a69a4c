"""Python mirror of the reference's back-end interface (original/driver.h:8-22).

`Propagator` wraps the five DRIVER_* entry points of libfletcher_gb300.so with
the reference's argument meaning (host arrays of sx*sy*sz float32, x fastest)
and raises `FletcherError` where the C layer records an error.  The extension
entry points (multi-step runs, field read-back, tile shape) are methods too.
"""
from __future__ import annotations

import numpy as np

from . import _lib
from ._lib import fptr


class FletcherError(RuntimeError):
    pass


def _check(lib, what: str) -> None:
    code = lib.FLETCHER_GetLastError()
    if code:
        msg = lib.FLETCHER_GetLastErrorString().decode(errors="replace")
        lib.FLETCHER_ClearError()
        raise FletcherError(f"{what}: {msg} (code {code})")


def _f32(a) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a


# Storage forms of the wave fields (FLETCHER_FORM_*).
FORMS = {"fp32": 0, "fp16": 1, "fp16x": 2}
# Numerics of the FP32 step (FLETCHER_NUMERICS_*).
NUMERICS = {"fast": 0, "d1d1": 1}
# Device layouts of the FP32 form's coefficients (FLETCHER_COEF_*).
COEF_LAYOUTS = {"auto": 0, "planes": 1, "media": 2}


class Propagator:
    """One resident simulation on the current GPU (the library holds one).

    form: "fp32" (the reference's precision), "fp16" (FP16 fields with a
    power-of-two scale per z-plane) or "fp16x" (FP16 plus a residual byte per
    value); the arithmetic is FP32 in every form.
    numerics: "fast" (default) or "d1d1" (the der1der1/ tree's operation
    order, FP32 form only).
    coef_layout: "planes" (default; ten coefficient planes), "media" (the
    six angle coefficients in a table of at most 256 media; bit-identical
    results, 36% fewer bytes per step, a few % slower on GB300) or "auto"
    (media where the model and shape allow it)."""

    def __init__(self, tile_rows: int = 0, stages: int = 0, zchunks: int = 0, stream: int | None = None,
                 form: str = "fp32", numerics: str = "fast", coef_layout: str = "planes"):
        self.lib = _lib.load()
        self.lib.FLETCHER_ClearError()
        if stream is not None:
            self.lib.FLETCHER_SetStream(stream)
        if form not in FORMS:
            raise ValueError(f"unknown form {form!r}; one of {sorted(FORMS)}")
        self.form = form
        if self.lib.FLETCHER_SetForm(FORMS[form]):
            _check(self.lib, "SetForm")
        if numerics not in NUMERICS:
            raise ValueError(f"unknown numerics {numerics!r}; one of {sorted(NUMERICS)}")
        if self.lib.FLETCHER_SetNumerics(NUMERICS[numerics]):
            _check(self.lib, "SetNumerics")
        if coef_layout not in COEF_LAYOUTS:
            raise ValueError(f"unknown coefficient layout {coef_layout!r}; one of {sorted(COEF_LAYOUTS)}")
        if self.lib.FLETCHER_SetCoefLayout(COEF_LAYOUTS[coef_layout]):
            _check(self.lib, "SetCoefLayout")
        if self.lib.FLETCHER_SetTileConfig(tile_rows, stages, zchunks):
            _check(self.lib, "SetTileConfig")
        self.shape = None

    # ---- DRIVER_* ---------------------------------------------------------
    def initialize(self, sx, sy, sz, bord, dx, dy, dz, dt, model, pp=None, pc=None, qp=None, qc=None):
        """model: (6, n) float32 = vpz vsv epsilon delta phi theta."""
        n = sx * sy * sz
        model = _f32(model).reshape(6, n)
        fields = []
        for f in (pp, pc, qp, qc):
            fields.append(np.zeros(n, np.float32) if f is None else _f32(f).reshape(n))
        self._keep = (model, fields)
        self.lib.DRIVER_Initialize(sx, sy, sz, bord, dx, dy, dz, dt, *[fptr(model[k]) for k in range(6)],
                                   *[fptr(f) for f in fields])
        _check(self.lib, "DRIVER_Initialize")
        self.shape = (sx, sy, sz, bord, dx, dy, dz, dt)

    def insert_source(self, it: int, i_source: int, src: float) -> None:
        self.lib.DRIVER_InsertSource(self.shape[7], it, int(i_source), None, None, float(src))
        _check(self.lib, "DRIVER_InsertSource")

    def propagate(self, it: int = 0) -> None:
        sx, sy, sz, bord, dx, dy, dz, dt = self.shape
        self.lib.DRIVER_Propagate(sx, sy, sz, bord, dx, dy, dz, dt, it, None, None, None, None)
        _check(self.lib, "DRIVER_Propagate")

    def update_pointers(self, pc: np.ndarray) -> None:
        sx, sy, sz = self.shape[:3]
        assert pc.dtype == np.float32 and pc.flags.c_contiguous and pc.size == sx * sy * sz
        self.lib.DRIVER_Update_pointers(sx, sy, sz, fptr(pc))
        _check(self.lib, "DRIVER_Update_pointers")

    def finalize(self) -> None:
        self.lib.DRIVER_Finalize()
        _check(self.lib, "DRIVER_Finalize")
        self.shape = None

    # ---- extensions ---------------------------------------------------------
    def run(self, nsteps: int, i_source: int = -1, src=None) -> None:
        """nsteps x (insert source, propagate), asynchronous on the stream."""
        s = None if src is None else _f32(src)
        rc = self.lib.FLETCHER_Run(int(nsteps), int(i_source), fptr(s))
        if rc:
            _check(self.lib, "FLETCHER_Run")

    def coef_layout(self) -> str:
        """The coefficient layout of the initialised state: "planes" or "media"."""
        rc = self.lib.FLETCHER_CoefLayout()
        if rc < 0:
            _check(self.lib, "FLETCHER_CoefLayout")
        return {1: "planes", 2: "media"}[rc]

    def synchronize(self) -> None:
        if self.lib.FLETCHER_Synchronize():
            _check(self.lib, "FLETCHER_Synchronize")

    def field(self, which: int) -> np.ndarray:
        """0 current p, 1 current q, 2 previous p, 3 previous q."""
        sx, sy, sz = self.shape[:3]
        out = np.empty(sx * sy * sz, np.float32)
        if self.lib.FLETCHER_GetField(which, fptr(out)):
            _check(self.lib, "FLETCHER_GetField")
        return out

    def coefficients(self) -> np.ndarray:
        """(10, n): ch1dxx ch1dyy ch1dzz ch1dxy ch1dyz ch1dxz v2px v2pz v2sz v2pn."""
        sx, sy, sz = self.shape[:3]
        out = np.empty((10, sx * sy * sz), np.float32)
        if self.lib.FLETCHER_GetCoefficients(fptr(out)):
            _check(self.lib, "FLETCHER_GetCoefficients")
        return out

    def kernel_launches(self) -> int:
        return int(self.lib.FLETCHER_KernelLaunches())

    def device_bytes(self) -> int:
        return int(self.lib.FLETCHER_DeviceBytes())

    def bytes_per_cell(self) -> float:
        return float(self.lib.FLETCHER_BytesPerCell())
