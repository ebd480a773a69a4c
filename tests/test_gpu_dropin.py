"""The drop-in claim, run: the reference's own front-end (original/main.c,
model.c, boundary.c, source.c, utils.c, map.c, walltime.c, unmodified) linked
once with the reference's OpenMP back-end and once with libfletcher_gb300.so
in its place (the link line of original/Makefile:29-31), both run with the
same command line, and their final wavefields compared.

The reference's executable writes no wavefield at the end of a run, so both
executables carry the link-time probe oracle/final_fields.c, which dumps the
final current p and q just before Model() calls DRIVER_Finalize
(original/model.c:162).  The run follows Model()'s own call sequence
(original/model.c:63-107): precompute, DRIVER_Initialize, per step
InsertSource / Propagate / SwapArrays, DRIVER_Update_pointers every 0.01 s of
simulated time, DRIVER_Finalize.

Tolerance: relative L2 <= 1e-5 for p and q (the FP32 kernel evaluates the
cross derivatives as D1 of D1, which rounds differently from the reference's
64-point sums).
"""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, gpu_available, reference_dir

pytestmark = pytest.mark.gpu

ORACLE = os.path.join(ROOT, "oracle")
DROPIN = os.path.join(ORACLE, "_ref", "dropin")


@pytest.fixture(scope="module")
def executables(lib):
    if not gpu_available():
        pytest.fail("these tests need a CUDA GPU")
    if reference_dir() is None:
        pytest.skip("reference sources absent: neither FLETCHER_REF_DIR nor the staged copy oracle/_ref/src")
    subprocess.run(["make", "-s", "-C", ORACLE, "dropin"], check=True)
    return os.path.join(DROPIN, "ModelagemFletcher_omp.exe"), os.path.join(DROPIN, "ModelagemFletcher_gb300.exe")


def run_exe(exe, args, workdir, out):
    env = dict(os.environ, FLETCHER_FINAL_FIELDS=out, OMP_NUM_THREADS=str(os.cpu_count() or 1))
    r = subprocess.run([exe, *args], cwd=workdir, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


@pytest.mark.parametrize("args", [["TTI", "56", "56", "56", "16", "12.5", "12.5", "12.5", "0.001", "0.2"],
                                  ["VTI", "40", "36", "32", "8", "10.0", "12.5", "15.0", "0.0005", "0.04"]])
def test_reference_front_end_on_gpu_matches_openmp(executables, args, tmp_path):
    omp_exe, gpu_exe = executables
    nx, ny, nz, absorb = (int(a) for a in args[1:5])
    sx, sy, sz = (n + 2 * 4 + 2 * absorb for n in (nx, ny, nz))
    n = sx * sy * sz
    outs = []
    for tag, exe in (("omp", omp_exe), ("gb300", gpu_exe)):
        wd = tmp_path / tag
        wd.mkdir()
        out = str(wd / "final.bin")
        log = run_exe(exe, args, str(wd), out)
        assert "MSamples/s" in log, log
        f = np.fromfile(out, np.float32)
        assert f.size == 2 * n, (tag, f.size, 2 * n)
        outs.append((f[:n].astype(np.float64), f[n:].astype(np.float64)))
    (rp, rq), (gp, gq) = outs
    assert np.abs(rp).max() > 1e-6  # the wave has spread
    ep = np.linalg.norm(gp - rp) / np.linalg.norm(rp)
    eq = np.linalg.norm(gq - rq) / np.linalg.norm(rq)
    print(f"{args[0]} {nx}x{ny}x{nz}: drop-in vs reference OpenMP executable, rel L2 p {ep:.3g} q {eq:.3g}")
    assert ep < 1e-5 and eq < 1e-5
