"""ORACLE -- test infrastructure only.

ctypes binding of oracle/_build/liborc.so, the CPU restatement of the
reference's FP32 OpenMP path (oracle/fletcher_oracle.c) plus its FP64
variant.  Only the tests, `__graft_entry__.smoke()` and the CPU-baseline leg
of `bench.py` import this package; the product never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liborc.so")
REF_LIB = os.path.join(HERE, "_ref", "libfletcher_ref.so")

FP = C.POINTER(C.c_float)
DP = C.POINTER(C.c_double)
_lib = None


def build() -> str:
    srcs = [os.path.join(HERE, f) for f in ("fletcher_oracle.c", "model_layered.c")]
    if not os.path.exists(LIB) or any(os.path.getmtime(LIB) < os.path.getmtime(s) for s in srcs):
        subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    return LIB


def load():
    global _lib
    if _lib is None:
        build()
        lib = C.CDLL(LIB)
        lib.orc_precompute.argtypes = [C.c_long] + [FP] * 7
        lib.orc_precompute_f64.argtypes = [C.c_long] + [FP] * 6 + [DP]
        lib.orc_random_velocity_boundary.argtypes = [C.c_int] * 8 + [FP, FP]
        lib.orc_srand.argtypes = [C.c_uint]
        lib.orc_source.restype = C.c_float
        lib.orc_source.argtypes = [C.c_float, C.c_int, C.c_double]
        lib.orc_propagate_f32.argtypes = [C.c_int] * 4 + [C.c_float] * 4 + [FP] * 5
        lib.orc_run_f32.argtypes = [C.c_int] * 4 + [C.c_float] * 4 + [C.c_int, C.c_long, C.c_double] + [FP] * 5
        lib.orc_run_f32.restype = C.c_int
        lib.orc_run_d1d1_f32.argtypes = lib.orc_run_f32.argtypes
        lib.orc_run_d1d1_f32.restype = C.c_int
        lib.orc_run_f64.argtypes = [C.c_int] * 4 + [C.c_double] * 4 + [C.c_int, C.c_long, C.c_double] + [DP] * 5
        lib.orc_run_f64.restype = C.c_int
        lib.orc_threads.restype = C.c_int
        lib.orc_recommended_dt.restype = C.c_float
        lib.orc_recommended_dt.argtypes = [C.c_long, FP, FP, C.c_float, C.c_float, C.c_float]
        lib.orc_model_layered.argtypes = [C.c_int] * 6 + [C.c_uint64, C.c_float, C.c_float, C.c_float, FP]
        _lib = lib
    return _lib


def _fp(a):
    return a.ctypes.data_as(FP)


def _dp(a):
    return a.ctypes.data_as(DP)


def model_layered(prob) -> np.ndarray:
    """(6, n) float32 layered medium of a layered `Problem` before the
    boundary (oracle/model_layered.c; equal to the product's generator)."""
    lib = load()
    m = np.empty((6, prob.n), np.float32)
    lib.orc_model_layered(prob.sx, prob.sy, prob.sz, prob.bord, prob.absorb, prob.layers, prob.seed,
                          float(prob.vrange[0]), float(prob.vrange[1]), float(prob.vs_ratio), _fp(m))
    return m


def model(prob) -> np.ndarray:
    """(6, n) float32 model of a layered `Problem` with the random-velocity
    boundary applied, built by the oracle alone (no product library)."""
    m = model_layered(prob)
    return boundary(prob.sx, prob.sy, prob.sz, prob.nx, prob.ny, prob.nz, prob.bord, prob.absorb, m, prob.seed)


def boundary(sx, sy, sz, nx, ny, nz, bord, absorb, model: np.ndarray, seed: int) -> np.ndarray:
    """Applies RandomVelocityBoundary after srand(seed) to a copy of model (6, n)."""
    lib = load()
    m = np.array(model, np.float32, copy=True)
    lib.orc_srand(seed)
    lib.orc_random_velocity_boundary(sx, sy, sz, nx, ny, nz, bord, absorb, _fp(m[0]), _fp(m[1]))
    return m


def precompute(model: np.ndarray) -> np.ndarray:
    """(10, n) float32: ch1dxx ch1dyy ch1dzz ch1dxy ch1dyz ch1dxz v2px v2pz v2sz v2pn."""
    lib = load()
    m = np.ascontiguousarray(model, np.float32)
    n = m.shape[1]
    out = np.empty((10, n), np.float32)
    lib.orc_precompute(n, *[_fp(m[k]) for k in range(6)], _fp(out))
    return out


def precompute_f64(model: np.ndarray) -> np.ndarray:
    lib = load()
    m = np.ascontiguousarray(model, np.float32)
    n = m.shape[1]
    out = np.empty((10, n), np.float64)
    lib.orc_precompute_f64(n, *[_fp(m[k]) for k in range(6)], _dp(out))
    return out


def source(dt: float, it: int, fcut: float) -> float:
    return load().orc_source(dt, it, fcut)


def run_f32(prob, model: np.ndarray, steps: int | None = None, coef: np.ndarray | None = None,
            fields=None):
    """FP32 oracle run of `steps` steps; returns (p, q, pp, qp) final current/previous fields."""
    lib = load()
    st = prob.steps if steps is None else steps
    coef = precompute(model) if coef is None else coef
    n = prob.n
    if fields is None:
        pp, pc, qp, qc = (np.zeros(n, np.float32) for _ in range(4))
    else:
        pp, pc, qp, qc = (np.array(f, np.float32, copy=True).reshape(n) for f in fields)
    odd = lib.orc_run_f32(prob.sx, prob.sy, prob.sz, prob.bord, prob.dx, prob.dy, prob.dz, prob.dt, st,
                          prob.i_source, prob.fcut, _fp(pp), _fp(pc), _fp(qp), _fp(qc), _fp(coef))
    return (pp, qp, pc, qc) if odd else (pc, qc, pp, qp)


def run_d1d1_f32(prob, model: np.ndarray, steps: int | None = None, coef: np.ndarray | None = None):
    """FP32 oracle run of the Der1-Der1 formulation (der1der1/ tree), with the
    given coefficients (default: the reference's precompute of `model`);
    returns (p, q, pp, qp) final current/previous fields."""
    lib = load()
    st = prob.steps if steps is None else steps
    coef = precompute(model) if coef is None else np.ascontiguousarray(coef, np.float32).reshape(10, -1)
    n = prob.n
    pp, pc, qp, qc = (np.zeros(n, np.float32) for _ in range(4))
    odd = lib.orc_run_d1d1_f32(prob.sx, prob.sy, prob.sz, prob.bord, prob.dx, prob.dy, prob.dz, prob.dt, st,
                               prob.i_source, prob.fcut, _fp(pp), _fp(pc), _fp(qp), _fp(qc), _fp(coef))
    return (pp, qp, pc, qc) if odd else (pc, qc, pp, qp)


def run_f64(prob, model: np.ndarray, steps: int | None = None):
    """FP64 oracle run; returns (p, q) final current fields as float64."""
    lib = load()
    st = prob.steps if steps is None else steps
    coef = precompute_f64(model)
    n = prob.n
    pp, pc, qp, qc = (np.zeros(n, np.float64) for _ in range(4))
    odd = lib.orc_run_f64(prob.sx, prob.sy, prob.sz, prob.bord, prob.dx, prob.dy, prob.dz, prob.dt, st,
                          prob.i_source, prob.fcut, _dp(pp), _dp(pc), _dp(qp), _dp(qc), _dp(coef))
    return (pp, qp) if odd else (pc, qc)


def rel_l2(a, b) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = np.sqrt(np.sum(b * b))
    return float(np.sqrt(np.sum((a - b) ** 2)) / den) if den > 0 else float(np.sqrt(np.sum(a * a)))


def threads() -> int:
    return int(load().orc_threads())


def time_slab(prob, model: np.ndarray, nplanes: int = 16, min_seconds: float = 10.0, max_steps: int = 10 ** 9,
              steps: int | None = None, seed: int = 0):
    """Times the FP32 oracle step on a bounded sample of `prob`'s grid: the
    full x-y extent of `nplanes` z-planes in the middle of the volume (the
    coefficients from `model`, the fields random with the magnitude of a
    propagated wavefield).  Runs `steps` steps, or until `min_seconds` have
    passed (at least 3).  Returns dict(msamples, steps, seconds, cells, threads)."""
    import time

    lib = load()
    r = 4
    z0 = max(prob.bord, prob.sz // 2 - nplanes // 2)
    z1 = min(prob.sz - prob.bord, z0 + nplanes)
    zs = slice(z0 - r, z1 + r)
    plane = prob.sx * prob.sy
    sub = np.ascontiguousarray(np.asarray(model, np.float32).reshape(6, prob.sz, plane)[:, zs, :]).reshape(6, -1)
    szs = z1 - z0 + 2 * r
    coef = precompute(sub)
    g = np.random.default_rng(seed)
    f = [(1e-3 * g.standard_normal(sub.shape[1])).astype(np.float32) for _ in range(4)]
    cells = (prob.sx - 2 * prob.bord) * (prob.sy - 2 * prob.bord) * (z1 - z0)
    args = (prob.sx, prob.sy, szs, r, prob.dx, prob.dy, prob.dz, prob.dt)
    n = 0
    t0 = time.perf_counter()
    while True:
        lib.orc_propagate_f32(*args, _fp(f[0]), _fp(f[1]), _fp(f[2]), _fp(f[3]), _fp(coef))
        f[0], f[1] = f[1], f[0]
        f[2], f[3] = f[3], f[2]
        n += 1
        el = time.perf_counter() - t0
        if steps is not None:
            if n >= steps:
                break
        elif (el >= min_seconds and n >= 3) or n >= max_steps:
            break
    el = time.perf_counter() - t0
    return {"msamples": 1e-6 * cells * n / el, "steps": n, "seconds": el, "cells": cells, "threads": threads(),
            "planes": z1 - z0}


REF_CLI = os.path.join(HERE, "_ref", "ref_cli")
REF_CLI_FTZ = os.path.join(HERE, "_ref", "ref_cli_ftz")


def reference_cli_available(ftz: bool = False) -> bool:
    return os.access(REF_CLI_FTZ if ftz else REF_CLI, os.X_OK)


def run_reference_cli(prob, steps: int, warmup: int = 0, ftz: bool = False, threads: int | None = None,
                      out: str = "-", stride: int = 1, timeout: float | None = None) -> dict:
    """Runs the reference's own FP32 OpenMP path (oracle/_ref/ref_cli, built
    from the unmodified original/ sources) on a layered `Problem`, in a
    separate process: the medium from oracle/model_layered.c, srand(seed) +
    RandomVelocityBoundary, precompute, then the Model() loop for `steps`
    steps.  Timing is the reference's own wtime() region (DRIVER_Propagate +
    SwapArrays, original/model.c:82-88) over the steps after `warmup`.
    Returns dict(msamples, timed_s, threads, setup_s, run_s, steps, warmup)."""
    exe = REF_CLI_FTZ if ftz else REF_CLI
    if not os.access(exe, os.X_OK):
        raise FileNotFoundError(exe)
    ix, iy, iz = prob.src_xyz
    spec = f"layered:{prob.layers}:{prob.vrange[0]}:{prob.vrange[1]}:{prob.vs_ratio}"
    args = [exe, spec, out, *map(str, [prob.sx, prob.sy, prob.sz, prob.nx, prob.ny, prob.nz, prob.bord, prob.absorb,
                                       prob.dx, prob.dy, prob.dz, prob.dt, steps, ix, iy, iz, prob.fcut, prob.seed,
                                       stride, warmup])]
    env = dict(os.environ)
    if threads:
        env["OMP_NUM_THREADS"] = str(threads)
    r = subprocess.run(args, capture_output=True, text=True, env=env, timeout=timeout)
    if r.returncode != 0:
        raise RuntimeError(f"ref_cli failed ({r.returncode}): {r.stderr.strip()[-400:]}")
    line = [ln for ln in r.stdout.splitlines() if ln.startswith("ref_cli:")][-1].split()
    kv = dict(zip(line[1::2], line[2::2]))
    return {"msamples": float(kv["msamples"]), "timed_s": float(kv["timed_s"]), "threads": int(kv["threads"]),
            "setup_s": float(kv["setup_s"]), "run_s": float(kv["run_s"]), "steps": int(kv["steps"]),
            "warmup": int(kv["warmup"])}
