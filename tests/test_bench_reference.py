"""The benchmark's reference arm (`bench.py --impl reference`) on a tiny grid:
it prints one JSON line for the reference's own CPU build (or, without the
reference sources, the oracle restatement, saying so), and the process never
maps this project's library -- the reference arm must not run the product."""
import json
import os
import subprocess
import sys

from conftest import ROOT, reference_dir


def test_reference_arm_runs_without_the_product_library():
    if reference_dir() is not None:
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True, capture_output=True)
    env = dict(os.environ, OMP_NUM_THREADS="2")
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--interior", "16", "--steps", "2",
                        "--warmup", "1"], cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads([ln for ln in r.stdout.splitlines() if ln.startswith("{")][-1])
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["config"]["grid"] == [88, 88, 88]
    kind = line["cpu_baseline"]["kind"]
    assert kind == ("reference" if reference_dir() is not None else "port")
    if kind == "reference":
        assert line["steps"] == 2 and line["warmup"] == 1 and line["cpu_baseline"]["cores"] == 2
    libs = line["libraries_loaded"]
    assert libs is not None and not any("libfletcher_gb300" in p for p in libs), libs
