"""Generates the golden fixtures in tests/golden/ from the reference itself.

Runs the reference's own FP32 OpenMP path, compiled from its unmodified
sources by `make -C oracle ref` into oracle/_ref/ (this needs the reference
checkout, so the fixtures are generated once and committed).  Inputs come
from the library's host model generators (layered / homogeneous media) with
the reference's RandomVelocityBoundary applied inside the reference build.

    python tests/golden/make_golden.py            # small cases (minutes)
    python tests/golden/make_golden.py --c1       # + the 504^3, 1000-step case (about an hour)
    python tests/golden/make_golden.py --c2-f64   # FP64 oracle, 128^3 interior, 2000 steps (minutes)
    python tests/golden/make_golden.py --d1d1     # the der1der1/ tree (Der1-Der1 formulation), small cases
    python tests/golden/make_golden.py --aniso    # only the small cases with dx != dy != dz (both trees)

Each fixture stores the problem definition, hashes of the boundary-modified
velocities and of the reference's coefficient fields, and the final current
p and q (full, or subsampled every `stride` cells) plus per-z-plane sums of
p^2 and q^2 at full resolution.
"""
from __future__ import annotations

import argparse
import ctypes as C
import dataclasses
import hashlib
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from fletcher_petrobras_gb300.models import C0, C1, Problem  # noqa: E402

FP = C.POINTER(C.c_float)


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def ref_lib(tree: str = "original"):
    """The harness over the reference's OpenMP back-end of `tree` ("original"
    or "der1der1", the Der1-Der1 formulation)."""
    target, name = ("ref", "libfletcher_ref.so") if tree == "original" else ("ref_d1d1", "libfletcher_ref_d1d1.so")
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), target], check=True)
    lib = C.CDLL(os.path.join(ROOT, "oracle", "_ref", name))
    lib.ref_boundary.argtypes = [C.c_int] * 8 + [FP, FP, C.c_uint]
    lib.ref_precompute.argtypes = [C.c_int] * 4 + [FP] * 7
    lib.ref_run.argtypes = [C.c_int] * 4 + [C.c_float] * 4 + [C.c_int, C.c_int, C.c_double] + [FP] * 10
    lib.ref_run.restype = C.c_int
    lib.ref_model.argtypes = [C.c_int] * 6 + [C.c_float] * 4 + [FP] * 10
    lib.ref_model.restype = C.c_int
    lib.ref_source.restype = C.c_float
    lib.ref_source.argtypes = [C.c_float, C.c_int]
    return lib


def fp(a):
    return a.ctypes.data_as(FP)


def plane_sums(f: np.ndarray, prob: Problem) -> np.ndarray:
    v = f.reshape(prob.sz, prob.sy * prob.sx).astype(np.float64)
    return np.sum(v * v, axis=1)


def subsample(f: np.ndarray, prob: Problem, stride: int) -> np.ndarray:
    return np.ascontiguousarray(f.reshape(prob.sz, prob.sy, prob.sx)[::stride, ::stride, ::stride]).ravel()


def save(name: str, prob: Problem, p, q, stride: int, extra: dict, use_model_fn: bool = False) -> None:
    meta = dataclasses.asdict(prob)
    meta.update(extra)
    meta["stride"] = stride
    meta["via_reference_model"] = use_model_fn
    out = os.path.join(HERE, f"golden_{name}.npz")
    np.savez_compressed(out, meta=np.array(json.dumps(meta)), p=subsample(p, prob, stride),
                        q=subsample(q, prob, stride), psum=plane_sums(p, prob), qsum=plane_sums(q, prob))
    print(f"wrote {out} ({os.path.getsize(out) / 1e3:.0f} kB)")


def run_small(lib, name: str, prob: Problem, stride: int = 1, raw: np.ndarray | None = None,
              use_model_fn: bool = False) -> None:
    t0 = time.time()
    m = prob.raw_model() if raw is None else raw.copy()
    lib.ref_boundary(prob.sx, prob.sy, prob.sz, prob.nx, prob.ny, prob.nz, prob.bord, prob.absorb, fp(m[0]),
                     fp(m[1]), prob.seed)
    coef = np.empty((10, prob.n), np.float32)
    lib.ref_precompute(prob.sx, prob.sy, prob.sz, prob.bord, *[fp(m[k]) for k in range(6)], fp(coef))
    f = [np.zeros(prob.n, np.float32) for _ in range(4)]
    if use_model_fn:
        assert prob.fcut == 40.0
        cwd = os.getcwd()
        with tempfile.TemporaryDirectory() as d:
            os.chdir(d)  # Model() writes Report.csv into the working directory
            odd = lib.ref_model(prob.steps, prob.i_source, prob.sx, prob.sy, prob.sz, prob.bord, prob.dx, prob.dy,
                                prob.dz, prob.dt, *[fp(m[k]) for k in range(6)], *[fp(x) for x in f])
            os.chdir(cwd)
    else:
        odd = lib.ref_run(prob.sx, prob.sy, prob.sz, prob.bord, prob.dx, prob.dy, prob.dz, prob.dt, prob.steps,
                          prob.i_source, prob.fcut, *[fp(m[k]) for k in range(6)], *[fp(x) for x in f])
    pp, pc, qp, qc = f
    p, q = (pp, qp) if odd else (pc, qc)
    extra = {"vpz_sha": sha(m[0]), "vsv_sha": sha(m[1]), "coef_sha": sha(coef)}
    if raw is not None:
        extra["raw_sha"] = sha(raw)
    save(name, prob, p, q, stride, extra, use_model_fn)
    print(f"  {name}: {prob.steps} steps on {prob.sx}x{prob.sy}x{prob.sz} in {time.time() - t0:.1f} s, "
          f"max|p| {np.abs(p).max():.4g}")


def main_tti_model(n: int, absorb: int, steps: int) -> tuple[Problem, np.ndarray]:
    """original/main.c:202-220's homogeneous TTI medium (phi = 1 rad, theta = atanf(1),
    vsv = vpz*sqrtf(|eps-delta|/SIGMA)), source at the grid centre, FCUT = 40."""
    prob = Problem("maintti", n, n, n, absorb=absorb, dt=0.001, steps=steps, fcut=40.0, seed=1)
    vsv = np.float32(3000.0) * np.sqrt(np.float32(abs(np.float32(0.24) - np.float32(0.1)) / 0.75)).astype(np.float32)
    raw = np.empty((6, prob.n), np.float32)
    for k, v in enumerate([3000.0, vsv, 0.24, 0.1, 1.0, np.arctan(np.float32(1.0))]):
        raw[k] = np.float32(v)
    return prob, raw


def run_c1(stride: int = 12) -> None:
    """The 504^3 layered case through the reference harness executable built
    with -mdaz-ftz (same operation order; no denormal stalls)."""
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref_ftz"], check=True)
    prob = C1
    raw = prob.raw_model()
    with tempfile.TemporaryDirectory(dir="/tmp") as d:
        fin, fout = os.path.join(d, "in.bin"), os.path.join(d, "out.bin")
        raw.tofile(fin)
        del raw
        ix, iy, iz = prob.src_xyz
        cmd = [os.path.join(ROOT, "oracle", "_ref", "ref_cli_ftz"), fin, fout, *map(str, [
            prob.sx, prob.sy, prob.sz, prob.nx, prob.ny, prob.nz, prob.bord, prob.absorb, prob.dx, prob.dy, prob.dz,
            prob.dt, prob.steps, ix, iy, iz, prob.fcut, prob.seed, stride])]
        t0 = time.time()
        r = subprocess.run(cmd, check=True, capture_output=True, text=True)
        print(r.stdout.strip(), f"({time.time() - t0:.0f} s)")
        ns = len(range(0, prob.sz, stride)) * len(range(0, prob.sy, stride)) * len(range(0, prob.sx, stride))
        data = np.fromfile(fout, np.float32, count=2 * ns)
        sums = np.fromfile(fout, np.float64, offset=8 * ns)
    meta = dataclasses.asdict(prob)
    meta.update({"stride": stride, "ftz": True, "via_reference_model": False})
    out = os.path.join(HERE, "golden_c1.npz")
    np.savez_compressed(out, meta=np.array(json.dumps(meta)), p=data[:ns], q=data[ns:],
                        psum=sums[:prob.sz], qsum=sums[prob.sz:])
    print(f"wrote {out}")


def run_c2_f64(stride: int = 4) -> None:
    """The 128^3-interior layered case, 2000 steps, through the FP64 oracle
    (the reference has no FP64 path; oracle/fletcher_oracle.c restates
    original/sample.h in double with exact rational weights).  The error of
    the 16-bit storage forms is measured against it."""
    import oracle as orc
    from fletcher_petrobras_gb300.models import C2

    prob = C2
    m = orc.boundary(prob.sx, prob.sy, prob.sz, prob.nx, prob.ny, prob.nz, prob.bord, prob.absorb,
                     prob.raw_model(), prob.seed)
    t0 = time.time()
    p, q = orc.run_f64(prob, m)
    print(f"  c2_f64: {prob.steps} steps on {prob.sx}x{prob.sy}x{prob.sz} in {time.time() - t0:.0f} s "
          f"({orc.threads()} threads), max|p| {np.abs(p).max():.4g}")
    meta = dataclasses.asdict(prob)
    meta.update({"stride": stride, "precision": "f64", "vpz_sha": sha(m[0])})
    out = os.path.join(HERE, "golden_c2_f64.npz")
    np.savez_compressed(out, meta=np.array(json.dumps(meta)), p=subsample(p, prob, stride).astype(np.float32),
                        q=subsample(q, prob, stride).astype(np.float32), psum=plane_sums(p, prob),
                        qsum=plane_sums(q, prob))
    print(f"wrote {out} ({os.path.getsize(out) / 1e3:.0f} kB)")


# Three different grid spacings (every derivative scaled on its own).
ANISO = Problem("tiny_aniso", 24, 20, 16, absorb=6, dx=10.0, dy=12.5, dz=15.0, dt=0.0005, steps=60, fcut=45.0,
                kind="layered", layers=4, seed=5)
ANISO = ANISO.with_(source=(ANISO.sx // 2 - 2, ANISO.sy // 2 + 1, ANISO.bord + ANISO.absorb + 5))


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--c1", action="store_true", help="also run the 504^3 x 1000-step case")
    ap.add_argument("--only-c1", action="store_true")
    ap.add_argument("--c2-f64", action="store_true", help="only the FP64 oracle's 128^3, 2000-step case")
    ap.add_argument("--d1d1", action="store_true", help="only the Der1-Der1 tree's small cases")
    ap.add_argument("--aniso", action="store_true", help="only the small case with three different spacings")
    a = ap.parse_args()
    if a.aniso:
        run_small(ref_lib(), "tiny_aniso", ANISO)
        run_small(ref_lib("der1der1"), "d1d1_tiny_aniso", ANISO.with_(name="d1d1_aniso"))
        return
    if a.c2_f64:
        run_c2_f64()
        return
    if a.d1d1:
        lib = ref_lib("der1der1")
        lay = Problem("d1d1_layered", 24, 20, 16, absorb=6, dt=0.0006, steps=60, fcut=45.0, kind="layered",
                      layers=4, seed=3)
        lay = lay.with_(source=(lay.sx // 2 + 3, lay.sy // 2 - 2, lay.bord + lay.absorb + 4))
        run_small(lib, "d1d1_tiny_layered", lay)
        run_small(lib, "d1d1_c0", C0, stride=3)
        return
    if not a.only_c1:
        lib = ref_lib()
        # Source values: the harness restates Source() for cut frequencies
        # other than 40; at 40 it must equal the reference's own Source().
        tiny = Problem("tiny_homog", 16, 16, 16, absorb=4, dt=0.001, steps=40, fcut=60.0, seed=7,
                       medium=C0.medium)
        run_small(lib, "tiny_homog", tiny)
        lay = Problem("tiny_layered", 24, 20, 16, absorb=6, dt=0.0006, steps=60, fcut=45.0, kind="layered",
                      layers=4, seed=3)
        lay = lay.with_(source=(lay.sx // 2 + 3, lay.sy // 2 - 2, lay.bord + lay.absorb + 4))
        run_small(lib, "tiny_layered", lay)
        prob, raw = main_tti_model(16, 4, 30)
        run_small(lib, "tiny_maintti", prob, raw=raw, use_model_fn=True)
        run_small(lib, "c0", C0, stride=3)
        src = np.array([lib.ref_source(np.float32(0.001), i) for i in range(400)], np.float32)
        np.save(os.path.join(HERE, "golden_source_fcut40.npy"), src)
    if a.c1 or a.only_c1:
        run_c1()


if __name__ == "__main__":
    main()
