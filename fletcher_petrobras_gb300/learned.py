"""Learned absorbing boundary (C ABI part 4, csrc/abc_learned.cu): training
data from plain-method runs on padded domains, training on the GPU with the
library's own forward/backward/Adam kernels, and the comparison with the
random-velocity boundary (original/boundary.c:7-98) by reflected energy.

Boundary forms compared on the same interior (n^3, the layered medium of the
C1 generator, 15 Hz Ricker 8 cells below the interior's top, at its centre):

* ``wide``: the medium extended over a padding wide enough that nothing
  comes back from the grid's edge within the run -- the reflection-free
  reference;
* ``random``: the reference's 32-cell random-velocity shell;
* ``learned``: an 8-cell layer of extended medium whose outer 4 cells get
  the one-way (box-scheme) update with the network's coefficients
  (``learned@N``: the network every N steps, the coefficients kept in
  between);
* ``oneway``: the same update with the medium's normal-incidence
  coefficients (the method without the network);
* ``sponge``: the same layer scaled by exp(-(a d)^2) after every step;
* ``plain8``: the same 8-cell layer with none of these (a zero edge).

Reflected energy of a form = sum over snapshot times of ||p - p_wide||^2
over the interior, divided by the same sum of ||p_wide||^2.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib
from ._lib import fptr, iptr
from .driver import FletcherError, Propagator, _check
from .models import Problem

LAYER = 8
RANDOM_ABSORB = 32
N_PARAMS = 2434
BOUNDARY_PLAIN, BOUNDARY_LEARNED, BOUNDARY_SPONGE, BOUNDARY_ONEWAY = 0, 1, 2, 3
DAMPING = 0.0


def _ok(lib, rc, what):
    if rc:
        _check(lib, what)
        raise FletcherError(what)


# ---- training data ---------------------------------------------------------------

def training_problem(index: int, n_virtual: int = 48, steps: int = 420) -> tuple:
    """Model `index` of the training set: the layered generator over a domain
    3x the virtual interior per axis (no absorbing shell), the source at a
    seeded position at least 8 cells inside the virtual interior.  Returns
    (Problem, interior_lo, interior_hi)."""
    N = 3 * n_virtual
    rng = np.random.default_rng(7919 * index + 17)
    lo = 4 + n_virtual
    src = tuple(int(lo + 8 + rng.integers(0, max(1, n_virtual - 16))) for _ in range(3))
    prob = Problem(f"abc-train-{index}", N, N, N, absorb=0, bord=4, dt=0.0006, steps=steps, fcut=45.0,
                   kind="layered", seed=1000 + index, source=src)
    return prob, (lo, lo, lo), (lo + n_virtual,) * 3


def collect(models: int = 64, n_virtual: int = 48, times=range(60, 421, 30), keep: float = 0.1,
            capacity: int = 8_000_000, seed: int = 1, stream: int | None = None) -> int:
    """Runs the plain method on `models` padded training domains and appends
    the layer-cell samples at each of `times` to the device training set.
    Returns the number of samples."""
    lib = _lib.load()
    _ok(lib, lib.FLETCHER_AbcReserve(capacity), "AbcReserve")
    times = list(times)
    for m in range(models):
        prob, lo, hi = training_problem(m, n_virtual, max(times))
        prop = Propagator(stream=stream)
        prop.initialize(prob.sx, prob.sy, prob.sz, prob.bord, prob.dx, prob.dy, prob.dz, prob.dt, prob.raw_model())
        src = prob.sources(max(times))
        lo_a, hi_a = np.array(lo, np.int32), np.array(hi, np.int32)
        t0 = 0
        for t in times:
            prop.run(t - t0, prob.i_source, src[t0:t])
            t0 = t
            prop.synchronize()
            pmax = float(np.abs(prop.field(0)).max())
            if pmax == 0.0:
                continue
            _ok(lib, lib.FLETCHER_AbcCollect(iptr(lo_a), iptr(hi_a), LAYER, keep, 31 * m + t + seed, 1e-6 * pmax),
                "AbcCollect")
        prop.finalize()
    return int(lib.FLETCHER_AbcSamples())


def samples(start: int = 0, n: int | None = None):
    """(features (n, 40), targets (n, 4): a_p a_q b_p b_q, cells (n, 4): x y z
    face+8d) from the device set."""
    lib = _lib.load()
    have = int(lib.FLETCHER_AbcSamples())
    n = have - start if n is None else n
    f = np.empty((n, 40), np.float32)
    t = np.empty((n, 4), np.float32)
    c = np.empty((n, 4), np.int32)
    _ok(lib, lib.FLETCHER_AbcGetSamples(start, n, fptr(f), fptr(t), iptr(c)), "AbcGetSamples")
    return f, t, c


# ---- network --------------------------------------------------------------------------

def init(seed: int = 0) -> None:
    lib = _lib.load()
    _ok(lib, lib.FLETCHER_AbcInit(seed), "AbcInit")


def train(iters: int = 3000, batch: int = 8192, lr: float = 3e-3, seed: int = 1, noise: float = 0.0) -> np.ndarray:
    """Adam on the device set with the library's kernels; returns the loss per step."""
    lib = _lib.load()
    loss = np.empty(iters, np.float32)
    _ok(lib, lib.FLETCHER_AbcTrain(iters, batch, lr, seed, noise, fptr(loss)), "AbcTrain")
    return loss


def get_weights() -> np.ndarray:
    lib = _lib.load()
    p = np.empty(N_PARAMS, np.float32)
    _ok(lib, lib.FLETCHER_AbcGetWeights(fptr(p)), "AbcGetWeights")
    return p


def set_weights(params) -> None:
    lib = _lib.load()
    p = np.ascontiguousarray(params, np.float32)
    _ok(lib, lib.FLETCHER_AbcSetWeights(fptr(p)), "AbcSetWeights")


def gradient(features, targets):
    lib = _lib.load()
    f = np.ascontiguousarray(features, np.float32)
    t = np.ascontiguousarray(targets, np.float32)
    g = np.empty(N_PARAMS, np.float32)
    loss = np.empty(1, np.float32)
    _ok(lib, lib.FLETCHER_AbcGradient(fptr(f), fptr(t), f.shape[0], fptr(g), fptr(loss)), "AbcGradient")
    return float(loss[0]), g


def forward(features):
    lib = _lib.load()
    f = np.ascontiguousarray(features, np.float32)
    out = np.empty((f.shape[0], 2), np.float32)
    _ok(lib, lib.FLETCHER_AbcForward(fptr(f), f.shape[0], fptr(out)), "AbcForward")
    return out


# ---- evaluation ---------------------------------------------------------------------

def wide_padding(steps: int, dt: float = 0.0006, dx: float = 12.5) -> int:
    """Padding from which nothing returns within `steps`: the fastest phase
    velocity of the generator's media (4000 m/s x sqrt(1 + 2 * 0.3)) over the
    way out and back, plus the source's 8 cells."""
    v = 4000.0 * math.sqrt(1.6)
    return int(math.ceil(0.5 * v * dt * steps / dx)) + 8


def boundary_problem(kind: str, n: int, steps: int, seed: int = 1) -> Problem:
    kind, _ = _split_kind(kind)
    pad = {"wide": wide_padding(steps), "random": RANDOM_ABSORB}.get(kind, LAYER)
    s = n + 2 * (4 + pad)
    return Problem(f"abc-{kind}-{n}", n, n, n, absorb=pad, bord=4, dt=0.0006, steps=steps, fcut=45.0,
                   kind="layered", seed=seed, source=(s // 2, s // 2, 4 + pad + 8))


def _split_kind(kind: str):
    """'learned@N' -> ('learned', N): the network every N steps."""
    base, _, n = kind.partition("@")
    return base, int(n) if n else 1


def _set_boundary(lib, kind: str, damping: float) -> None:
    kind, interval = _split_kind(kind)
    _ok(lib, lib.FLETCHER_AbcSetInterval(interval), "AbcSetInterval")
    if kind == "learned":
        _ok(lib, lib.FLETCHER_SetBoundary(BOUNDARY_LEARNED, LAYER, damping), "SetBoundary")
    elif kind == "oneway":
        _ok(lib, lib.FLETCHER_SetBoundary(BOUNDARY_ONEWAY, LAYER, damping), "SetBoundary")
    elif kind == "sponge":
        _ok(lib, lib.FLETCHER_SetBoundary(BOUNDARY_SPONGE, LAYER, damping if damping > 0 else 0.03), "SetBoundary")


def tuned_shape(kind: str, prob, model, damping: float = DAMPING, steps_per_shape: int = 4, stream=None):
    """(tile rows, stages) that the library's tuner (FLETCHER_Autotune) picks
    for this form's grid, boundary launches included, from a short untimed
    run."""
    import os
    import shutil
    import tempfile

    lib = _lib.load()
    prop = Propagator(stream=stream)
    prop.initialize(prob.sx, prob.sy, prob.sz, prob.bord, prob.dx, prob.dy, prob.dz, prob.dt, model)
    _set_boundary(lib, kind, damping)
    tmp = tempfile.mkdtemp(prefix="flt-tune-")
    rows, stages = C.c_int(0), C.c_int(0)
    try:
        rc = lib.FLETCHER_Autotune(os.path.join(tmp, "configurations.txt").encode(), steps_per_shape)
        _ok(lib, rc not in (0, 1), "Autotune")
        src = prob.sources(200)
        t = 0
        while lib.FLETCHER_GetTileConfig(C.byref(rows), C.byref(stages)) == 1 and t < 200:
            prop.run(5, prob.i_source, src[t:t + 5])
            t += 5
        prop.synchronize()
        lib.FLETCHER_GetTileConfig(C.byref(rows), C.byref(stages))
    finally:
        lib.FLETCHER_SetBoundary(BOUNDARY_PLAIN, 0, 0.0)
        lib.FLETCHER_AbcSetInterval(1)
        prop.finalize()
        shutil.rmtree(tmp, ignore_errors=True)
    return int(rows.value), int(stages.value)


def run_boundary(kind: str, n: int, steps: int, snaps, seed: int = 1, stream=None, damping: float = DAMPING,
                 tune: bool = True):
    """Runs one boundary form (with its tuned tile shape when `tune`);
    returns (interior p at each snapshot step, device ms per step (CUDA
    events), kernel launches per step, tile shape)."""
    import torch

    base, _ = _split_kind(kind)
    prob = boundary_problem(base, n, steps, seed)
    model = prob.model() if base == "random" else prob.raw_model()
    st = torch.cuda.Stream() if stream is None else stream
    shape = tuned_shape(kind, prob, model, damping, stream=st.cuda_stream) if tune else (0, 0)
    prop = Propagator(*shape, stream=st.cuda_stream)
    prop.initialize(prob.sx, prob.sy, prob.sz, prob.bord, prob.dx, prob.dy, prob.dz, prob.dt, model)
    lib = prop.lib
    _set_boundary(lib, kind, damping)
    src = prob.sources(steps)
    o = prob.bord + prob.absorb
    out = []
    ms = 0.0
    t0 = 0
    for t in sorted(snaps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        prop.run(t - t0, prob.i_source, src[t0:t])
        e1.record(st)
        prop.synchronize()
        ms += e0.elapsed_time(e1)
        t0 = t
        p = prop.field(0).reshape(prob.sz, prob.sy, prob.sx)
        out.append(np.ascontiguousarray(p[o:o + n, o:o + n, o:o + n]))
    rows, stages = C.c_int(0), C.c_int(0)
    lib.FLETCHER_GetTileConfig(C.byref(rows), C.byref(stages))
    lib.FLETCHER_SetBoundary(BOUNDARY_PLAIN, 0, 0.0)
    lib.FLETCHER_AbcSetInterval(1)
    prop.finalize()
    Propagator()  # back to the default tile shape
    extra = {"learned": 1, "oneway": 1, "sponge": 1}.get(base, 0)  # one boundary launch after the step
    extra += 1 if damping > 0 and base in ("learned", "oneway") else 0
    return out, ms / max(snaps), 1 + extra, (rows.value, stages.value)


def reflected_energy(fields, reference) -> float:
    num = sum(float(np.sum((a.astype(np.float64) - b) ** 2)) for a, b in zip(fields, reference))
    den = sum(float(np.sum(b.astype(np.float64) ** 2)) for b in reference)
    return num / den


def compare(n: int = 256, steps: int = 1500, nsnap: int = 5, kinds=("random", "learned", "oneway", "plain8"),
            seed: int = 1, damping: float = DAMPING, tune: bool = True):
    """Reflected energy (total and per snapshot) and interior MSamples/s of
    each boundary form, each run with the tile shape the tuner picks for it
    (`tune`)."""
    snaps = [int(round(steps * (k + 1) / nsnap)) for k in range(nsnap)]
    ref, ref_ms, _, ref_shape = run_boundary("wide", n, steps, snaps, seed, tune=tune)
    res = {"wide": {"ms_per_step": ref_ms, "interior_msamples": n ** 3 / ref_ms / 1e3, "reflected_energy": 0.0,
                    "padding": wide_padding(steps), "tile": list(ref_shape)}}
    for k in kinds:
        f, ms, launches, shape = run_boundary(k, n, steps, snaps, seed, damping=damping, tune=tune)
        res[k] = {"ms_per_step": ms, "interior_msamples": n ** 3 / ms / 1e3,
                  "reflected_energy": reflected_energy(f, ref),
                  "reflected_energy_by_snapshot": [reflected_energy([a], [b]) for a, b in zip(f, ref)],
                  "launches_per_step": launches, "tile": list(shape)}
    res["snapshots"] = snaps
    return res


def profile_case(kind: str = "learned", n: int = 256, steps: int = 24, seed: int = 0) -> float:
    """A short run of one boundary form with the network's initial weights
    (untrained: the kernels' work does not depend on the weights) and the
    default tile shape: the case the boundary kernels are profiled on.
    Returns (and prints) the device ms per step.

        python -c "from fletcher_petrobras_gb300 import learned; learned.profile_case('learned@8', 256, 24)"
    """
    import torch

    init(seed)
    base, _ = _split_kind(kind)
    prob = boundary_problem(base, n, steps, seed)
    model = prob.model() if base == "random" else prob.raw_model()
    st = torch.cuda.Stream()
    prop = Propagator(stream=st.cuda_stream)
    prop.initialize(prob.sx, prob.sy, prob.sz, prob.bord, prob.dx, prob.dy, prob.dz, prob.dt, model)
    _set_boundary(prop.lib, kind, 0.0)
    src = prob.sources(steps)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    prop.run(steps, prob.i_source, src)
    e1.record(st)
    prop.synchronize()
    ms = e0.elapsed_time(e1) / steps
    prop.lib.FLETCHER_SetBoundary(BOUNDARY_PLAIN, 0, 0.0)
    prop.lib.FLETCHER_AbcSetInterval(1)
    prop.finalize()
    print(f"{kind} {n}^3: {ms:.4f} ms per step")
    return ms
