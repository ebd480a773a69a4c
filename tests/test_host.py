"""Host side of the product (no GPU): model preparation against the reference's
own boundary and source, determinism of the layered generator, and the
C-ABI exports."""
import ctypes
import hashlib
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT, load_golden, reference_dir
from fletcher_petrobras_gb300 import C0, C1, C2, Problem
from fletcher_petrobras_gb300._lib import SIGNATURES, fptr


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("name", ["tiny_homog", "tiny_layered", "c0"])
def test_product_boundary_matches_reference(name, lib):
    prob, meta, _ = load_golden(name)
    m = prob.model()  # product generator + product RandomVelocityBoundary
    assert sha(m[0]) == meta["vpz_sha"]
    assert sha(m[1]) == meta["vsv_sha"]


def test_product_source_matches_reference(lib):
    ref = np.load(f"{GOLDEN}/golden_source_fcut40.npy")
    got = np.array([lib.FLETCHER_Source(np.float32(0.001), i, 40.0) for i in range(len(ref))], np.float32)
    assert np.array_equal(got, ref)


def test_source_peak_frequency(lib):
    """The Ricker's spectrum peaks at fcut/3 (20 Hz for fcut 60)."""
    dt = 1e-4
    s = np.array([lib.FLETCHER_Source(dt, i, 60.0) for i in range(20000)], np.float64)
    spec = np.abs(np.fft.rfft(s))
    f = np.fft.rfftfreq(len(s), dt)
    assert abs(f[np.argmax(spec)] - 20.0) < 0.5


def test_layered_generator_properties(lib):
    p = C2
    m = p.raw_model()
    assert sha(m) == sha(p.raw_model())  # deterministic
    tops = (ctypes.c_int * p.layers)()
    m2 = np.empty_like(m)
    lib.FLETCHER_ModelLayered(p.sx, p.sy, p.sz, p.bord, p.absorb, p.layers, p.seed, 1500.0, 4000.0, 0.5,
                              fptr(m2), tops)
    assert np.array_equal(m, m2)
    top = list(tops)
    assert top[0] == p.bord + p.absorb and all(b > a for a, b in zip(top, top[1:]))
    col = m[:, :].reshape(6, p.sz, -1)[:, :, 0]
    vp = col[0]
    assert np.all(np.diff(vp) >= 0) and vp.min() >= 1500 and vp.max() <= 4000  # increasing with depth
    assert np.allclose(col[1], 0.5 * vp)
    assert np.all((col[2] >= 0) & (col[2] <= 0.3)) and np.all((col[3] >= 0) & (col[3] <= col[2]))
    assert np.all((col[5] >= 0) & (col[5] <= np.radians(45) + 1e-6)) and np.all(col[4] <= np.radians(90) + 1e-6)
    assert len(np.unique(vp)) == p.layers
    # horizontally layered: every plane is constant
    assert np.all(np.ptp(m.reshape(6, p.sz, -1), axis=2) == 0)


def test_recommended_dt(lib, orc):
    m = C0.model()
    a = lib.FLETCHER_RecommendedDt(C0.n, fptr(m[0]), fptr(m[2]), 12.5, 12.5, 12.5)
    b = orc.load().orc_recommended_dt(C0.n, m[0].ctypes.data_as(orc.FP), m[2].ctypes.data_as(orc.FP), 12.5, 12.5,
                                      12.5)
    assert a == b
    assert abs(a - 0.2 * 12.5 / (3000 * np.sqrt(1.48))) < 1e-6


def test_problem_geometry():
    assert (C0.sx, C0.sy, C0.sz) == (96, 96, 96) and C0.updated_cells == 88 ** 3
    assert (C1.sx, C1.sz) == (576, 576) and C1.updated_cells == 568 ** 3
    assert C1.src_xyz == (288, 288, 44) and C1.fcut == 45.0 and C1.dt == pytest.approx(0.0006)
    assert C0.fcut == 60.0


def header_functions():
    txt = open(os.path.join(ROOT, "include", "fletcher_gb300.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    txt = "\n".join(line for line in txt.splitlines() if not line.lstrip().startswith("#"))
    return sorted(set(re.findall(r"\b((?:DRIVER|FLETCHER)_[A-Za-z_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol(lib):
    names = header_functions()
    assert len(names) >= 5 + 16
    out = subprocess.run(["nm", "-D", "--defined-only", lib._name], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (\S+)", out))
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    assert set(names) == set(SIGNATURES), set(names) ^ set(SIGNATURES)
    for n in ["DRIVER_Initialize", "DRIVER_Finalize", "DRIVER_Propagate", "DRIVER_Update_pointers",
              "DRIVER_InsertSource"]:
        assert n in exported


def test_argument_errors_are_reported_not_fatal(lib):
    """Invalid arguments are rejected before any CUDA call, with a status."""
    lib.FLETCHER_ClearError()
    n = 16 ** 3
    a = [np.zeros(n, np.float32) for _ in range(10)]
    lib.DRIVER_Initialize(16, 16, 16, 3, 12.5, 12.5, 12.5, 0.001, *[fptr(x) for x in a])  # bord < 4
    assert lib.FLETCHER_GetLastError() == 1
    assert b"bord" in lib.FLETCHER_GetLastErrorString()
    lib.FLETCHER_ClearError()
    lib.DRIVER_Propagate(16, 16, 16, 4, 12.5, 12.5, 12.5, 0.001, 1, None, None, None, None)
    assert lib.FLETCHER_GetLastError() == 1  # not initialised
    lib.FLETCHER_ClearError()
    assert lib.FLETCHER_SetTileConfig(7, 4, 0) == 1  # shape not built
    lib.FLETCHER_ClearError()
    assert lib.FLETCHER_SetTileConfig(0, 0, 0) == 0
    assert lib.FLETCHER_SetCoefLayout(3) == 1
    assert b"coefficient layout" in lib.FLETCHER_GetLastErrorString()
    lib.FLETCHER_ClearError()
    assert lib.FLETCHER_SetCoefLayout(1) == 0
    assert lib.FLETCHER_CoefLayout() < 0  # not initialised
    lib.FLETCHER_ClearError()
    assert lib.FLETCHER_BatchSetChains(9) == 1
    assert b"chains must be -1" in lib.FLETCHER_GetLastErrorString()
    lib.FLETCHER_ClearError()
    assert lib.FLETCHER_BatchSetChains(2) == 1  # no batch open
    lib.FLETCHER_ClearError()
    ph = (ctypes.c_double * 5)()
    assert lib.FLETCHER_InitPhases(ph) == 0
    assert lib.FLETCHER_DebugPoisonPadding(0.0) == 1  # not initialised
    lib.FLETCHER_ClearError()


@pytest.mark.skipif(reference_dir() is None, reason="reference sources absent (FLETCHER_REF_DIR or staged copy)")
def test_reference_front_end_links_against_library(tmp_path):
    """The reference's own front-end objects link against libfletcher_gb300.so
    in place of a back-end (the drop-in link line of original/Makefile:29-31).
    tests/test_gpu_dropin.py runs the result on a GPU."""
    ref = os.path.join(reference_dir(), "original")
    objs = []
    for src in ["main.c", "source.c", "utils.c", "boundary.c", "walltime.c", "model.c", "map.c"]:
        o = tmp_path / (src + ".o")
        subprocess.run(["gcc", "-O3", "-w", "-I" + ref, "-c", f"{ref}/{src}", "-o", str(o)], check=True)
        objs.append(str(o))
    from fletcher_petrobras_gb300.build import OUT

    exe = tmp_path / "ModelagemFletcher.exe"
    subprocess.run(["gcc", "-o", str(exe), *objs, "-L" + OUT, "-lfletcher_gb300", "-Wl,-rpath," + OUT, "-lm"],
                   check=True)
    assert exe.exists()


def test_multishot_spec_properties():
    from fletcher_petrobras_gb300.batch import multishot_spec

    spec = multishot_spec(48, seed=0)
    assert len(spec) == 48
    for p in spec:
        assert all(96 <= v <= 320 and v % 8 == 0 for v in (p.nx, p.ny, p.nz))
        assert 500 <= p.steps <= 1500 and p.dt == pytest.approx(0.0006)
        ix, iy, iz = p.src_xyz
        b = p.bord + p.absorb
        assert b <= iz < b + max(1, p.nz // 4) and b <= ix < b + p.nx and b <= iy < b + p.ny


def test_oracle_layered_model_matches_library():
    """The oracle's layered-medium generator (used by the benchmark's
    reference arm, which must not load this library) gives the library's
    floats, before and after the random-velocity boundary."""
    import oracle
    from fletcher_petrobras_gb300.models import C2, Problem

    for prob in (Problem("lay", 40, 36, 32, absorb=6, dt=0.0006, kind="layered", layers=4, seed=3),
                 Problem("lay1", 24, 20, 30, absorb=5, dt=0.0006, kind="layered", layers=1, seed=7),
                 Problem("lay9", 20, 20, 12, absorb=4, dt=0.0006, kind="layered", layers=9, seed=11), C2):
        assert np.array_equal(oracle.model_layered(prob), prob.raw_model()), prob.name
        assert np.array_equal(oracle.model(prob), prob.model()), prob.name


@pytest.mark.skipif(reference_dir() is None, reason="reference sources absent (FLETCHER_REF_DIR or staged copy)")
def test_reference_cli_matches_reference_library():
    """oracle/_ref/ref_cli (the reference's own OpenMP build driven by the
    reference arm of the benchmark) reproduces the reference fixture of a
    layered case bit for bit, and reports its wtime() region."""
    import tempfile

    import oracle

    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True, capture_output=True)
    prob, meta, g = load_golden("tiny_layered")
    with tempfile.TemporaryDirectory() as d:
        out = os.path.join(d, "o.bin")
        r = oracle.run_reference_cli(prob, prob.steps, 2, out=out, threads=2)
        n = prob.n
        f = np.fromfile(out, np.float32, count=2 * n)
    assert r["steps"] == prob.steps and r["warmup"] == 2 and r["timed_s"] > 0 and r["threads"] == 2
    assert np.array_equal(f[:n], g["p"]) and np.array_equal(f[n:], g["q"])
