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
* ``learned``: an 8-cell layer of extended medium whose outer face cells get
  the network's correction (every layer cell then scaled by exp(-(a d)^2)
  when a damping a > 0 is given);
* ``sponge``: the same layer and scaling without the network;
* ``plain8``: the same 8-cell layer without either (a zero edge).

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
BOUNDARY_PLAIN, BOUNDARY_LEARNED, BOUNDARY_SPONGE = 0, 1, 2
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
    """(features (n, 40), targets (n, 2), cells (n, 4): x y z d) from the device set."""
    lib = _lib.load()
    have = int(lib.FLETCHER_AbcSamples())
    n = have - start if n is None else n
    f = np.empty((n, 40), np.float32)
    t = np.empty((n, 2), np.float32)
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


def get_weights():
    lib = _lib.load()
    p = np.empty(N_PARAMS, np.float32)
    s = C.c_float(0)
    _ok(lib, lib.FLETCHER_AbcGetWeights(fptr(p), C.cast(C.pointer(s), _lib.FP)), "AbcGetWeights")
    return p, float(s.value)


def set_weights(params, out_scale: float) -> None:
    lib = _lib.load()
    p = np.ascontiguousarray(params, np.float32)
    _ok(lib, lib.FLETCHER_AbcSetWeights(fptr(p), float(out_scale)), "AbcSetWeights")


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
    pad = {"wide": wide_padding(steps), "random": RANDOM_ABSORB, "learned": LAYER, "sponge": LAYER,
           "plain8": LAYER}[kind]
    s = n + 2 * (4 + pad)
    return Problem(f"abc-{kind}-{n}", n, n, n, absorb=pad, bord=4, dt=0.0006, steps=steps, fcut=45.0,
                   kind="layered", seed=seed, source=(s // 2, s // 2, 4 + pad + 8))


def run_boundary(kind: str, n: int, steps: int, snaps, seed: int = 1, stream=None, damping: float = DAMPING):
    """Runs one boundary form; returns (interior p at each snapshot step,
    device ms per step (CUDA events), kernel launches per step)."""
    import torch

    prob = boundary_problem(kind, n, steps, seed)
    model = prob.model() if kind == "random" else prob.raw_model()
    st = torch.cuda.Stream() if stream is None else stream
    prop = Propagator(stream=st.cuda_stream)
    prop.initialize(prob.sx, prob.sy, prob.sz, prob.bord, prob.dx, prob.dy, prob.dz, prob.dt, model)
    lib = prop.lib
    if kind == "learned":
        _ok(lib, lib.FLETCHER_SetBoundary(BOUNDARY_LEARNED, LAYER, damping), "SetBoundary")
    elif kind == "sponge":
        _ok(lib, lib.FLETCHER_SetBoundary(BOUNDARY_SPONGE, LAYER, damping if damping > 0 else 0.03), "SetBoundary")
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
    if kind in ("learned", "sponge"):
        lib.FLETCHER_SetBoundary(BOUNDARY_PLAIN, 0, 0.0)
    prop.finalize()
    return out, ms / max(snaps), {"learned": 3, "sponge": 2}.get(kind, 1)


def reflected_energy(fields, reference) -> float:
    num = sum(float(np.sum((a.astype(np.float64) - b) ** 2)) for a, b in zip(fields, reference))
    den = sum(float(np.sum(b.astype(np.float64) ** 2)) for b in reference)
    return num / den


def compare(n: int = 256, steps: int = 1500, nsnap: int = 5, kinds=("random", "learned", "sponge", "plain8"),
            seed: int = 1, damping: float = DAMPING):
    """Reflected energy (total and per snapshot) and interior MSamples/s of
    each boundary form."""
    snaps = [int(round(steps * (k + 1) / nsnap)) for k in range(nsnap)]
    ref, ref_ms, _ = run_boundary("wide", n, steps, snaps, seed)
    res = {"wide": {"ms_per_step": ref_ms, "interior_msamples": n ** 3 / ref_ms / 1e3, "reflected_energy": 0.0,
                    "padding": wide_padding(steps)}}
    for k in kinds:
        f, ms, launches = run_boundary(k, n, steps, snaps, seed, damping=damping)
        res[k] = {"ms_per_step": ms, "interior_msamples": n ** 3 / ms / 1e3,
                  "reflected_energy": reflected_energy(f, ref),
                  "reflected_energy_by_snapshot": [reflected_energy([a], [b]) for a, b in zip(f, ref)],
                  "launches_per_step": launches}
    res["snapshots"] = snaps
    return res
