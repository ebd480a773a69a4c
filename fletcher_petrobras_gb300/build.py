"""In-tree build of libfletcher_gb300.so and the fletcher_gb300 executable.

CUDA sources are compiled for sm_103a only; host C with -ffp-contract=off so
float expressions round as the reference's x86-64 build.  Translation units
compile in parallel and are skipped when up to date.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
ROOT = os.path.dirname(HERE)
INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(OUT, "libfletcher_gb300.so")
EXE = os.path.join(OUT, "fletcher_gb300")

NVCC = os.environ.get("NVCC", "nvcc")
GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = GENCODE + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                        "-Xptxas", "-v", "-I" + INCLUDE]
CC = os.environ.get("CC", "gcc")
C_FLAGS = ["-O3", "-fPIC", "-ffp-contract=off", "-std=gnu11", "-Wall", "-I" + INCLUDE]

CU_SOURCES = ["driver.cu", "propagate_fp32.cu", "propagate_half.cu", "abc_learned.cu", "snapshot.cu", "noalloc.cu"]
C_SOURCES = ["host/fletcher_host.c"]
HEADERS = ["device_util.cuh", "fletcher_internal.h", "stencil_common.cuh", "propagate_fp32_pipe.cuh"]


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _run(cmd: list[str], log: str | None = None) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if log:
        with open(log, "w") as f:
            f.write(r.stdout + r.stderr)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError("build step failed: " + " ".join(cmd))


def build(verbose: bool = False) -> str:
    """Builds the library (and CLI) if sources changed; returns the .so path."""
    os.makedirs(OUT, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "fletcher_gb300.h")]
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, os.path.basename(src) + ".o")
        objs.append(o)
        if _newer(o, [s] + hdrs):
            jobs.append(([NVCC] + NVCC_FLAGS + ["-c", s, "-o", o], o + ".log"))
    for src in C_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, os.path.basename(src) + ".o")
        objs.append(o)
        if _newer(o, [s] + hdrs):
            jobs.append(([CC] + C_FLAGS + ["-c", s, "-o", o], None))
    if jobs:
        with ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
            for f in [ex.submit(_run, c, l) for c, l in jobs]:
                f.result()
    if jobs or _newer(LIB, objs):
        _run([NVCC] + GENCODE + ["-shared", "-o", LIB] + objs + ["-lm"])
    main_c = os.path.join(CSRC, "host", "fletcher_main.c")
    if _newer(EXE, [main_c, LIB]):
        _run([CC] + C_FLAGS + ["-o", EXE, main_c, "-L" + OUT, "-lfletcher_gb300",
                               "-Wl,-rpath," + OUT, "-lm"])
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
