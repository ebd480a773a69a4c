"""Benchmark: Fletcher TTI FP32 propagation at 504^3 interior on one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Workload (one "step" = one propagation step of the whole grid): the layered
504^3-interior model (576^3 grid, bord 4, absorb 32, dt 0.6 ms, 15 Hz Ricker
at (288, 288, 44)), synthetic and seeded.  The line printed by rank 0:

  value     MSamples/s by the reference's definition (original/model.c:44,117:
            updated cells x steps / time), K steps timed with CUDA events on the
            library's stream, inputs resident in HBM (11+ GB, larger than L2,
            so no flush is needed between steps);
  e2e       the same metric through the C ABI with host buffers over the
            workload's own 1000 steps: the reference's Model() sequence
            (FLETCHER_Model: DRIVER_Initialize with the host-to-device copy of
            the model and fields, per step InsertSource + Propagate, a
            device-to-host snapshot of p every 0.01 s of simulated time, final
            read-back), wall-clock; `parity` compares its final fields with the
            reference build's own 1000-step result;
  roofline  the propagate kernel against the measured HBM copy bandwidth;
            algorithmic bytes = 64 B per updated cell (fields 16 B read + 8 B
            written, ten coefficients 40 B);
  forms     the 16-bit storage forms on the same workload;
  c3_batch, c4_learned  the batched-shot and learned-boundary workloads;
  cpu_baseline  the reference's own OpenMP build (oracle/_ref/ref_cli, the
            unmodified original/ sources compiled on this host) on all host
            cores, a few full-grid steps timed by its own wtime() region.

N > 1: replicas only -- every rank runs the whole workload on its own GPU,
no data exchange; timing is the max over ranks, value the sum of cells/time.
`--impl reference` runs the reference's own OpenMP build on the full grid
(K steps, at most 40) without loading this project's library.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "MSamples/s + HBM GB/s at 504^3: FP32 vs FP16-store/learned-ABC, equal L2 err"
UNIT = "MSamples/s"
FALLBACK_HBM_GBS = 6800.0


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Group:
    """Host-side coordination of replicas (gloo): barrier and max/sum of scalars."""

    def __init__(self, ws: int):
        self.ws = ws
        if ws > 1:
            import torch.distributed as dist

            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.ws > 1:
            self.dist.barrier()

    def reduce(self, x: float, op: str) -> float:
        if self.ws == 1:
            return x
        import torch

        t = torch.tensor([x], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX if op == "max" else self.dist.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.ws > 1:
            self.dist.destroy_process_group()


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def ncu_traffic_per_cell(layout):
    """DRAM bytes per updated cell of the propagate kernel in this
    coefficient layout from the committed ncu summary
    (profiles/propagate_fp32_traffic.json), or None."""
    path = os.path.join(ROOT, "profiles", "propagate_fp32_traffic.json")
    try:
        with open(path) as f:
            return float(json.load(f)[layout]["dram_bytes_per_cell"])
    except Exception:
        return None


class ClockSampler:
    """nvidia-smi samples (200 ms) during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.file,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.file.flush()
        rows = []
        with open(self.file.name) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.file.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}

        def num(s):
            try:
                return float(s)
            except ValueError:
                return None

        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        mx = [num(r[2]) for r in rows if num(r[2]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows),
                "power_w_max": max((num(r[3]) or 0.0) for r in rows)}


def workload(args):
    """The C1 problem, or the same generator at another interior size (profiling)."""
    from fletcher_petrobras_gb300 import C1

    if args.interior == C1.nx:
        return C1
    n = args.interior
    s = n + 2 * (C1.bord + C1.absorb)
    return C1.with_(name=f"C1-layered-{n}", nx=n, ny=n, nz=n, source=(s // 2, s // 2, C1.bord + C1.absorb + 8))


# Kernels one step launches in each storage form (the 16-bit forms set the
# new planes' scales in a small kernel before the propagate kernel).
LAUNCHES_PER_STEP = {"fp32": 1, "fp16": 2, "fp16x": 2}
KERNEL = {"fp32": "k_propagate_fp32", "fp16": "k_propagate_half<EXT=false>", "fp16x": "k_propagate_half<EXT=true>"}


def timed_run(prob, model, form, K, W, group, clocks=None, layout="planes"):
    """W untimed steps, then K steps timed with CUDA events on the library's
    stream.  Returns (ms, kernel launches, bytes per cell, device GB, clocks,
    coefficient layout)."""
    import torch

    from fletcher_petrobras_gb300 import Propagator

    src = prob.sources(W + K)
    stream = torch.cuda.Stream()
    prop = Propagator(stream=stream.cuda_stream, form=form, coef_layout=layout)
    prop.initialize(prob.sx, prob.sy, prob.sz, prob.bord, prob.dx, prob.dy, prob.dz, prob.dt, model)
    used_layout = prop.coef_layout()
    prop.run(W, prob.i_source, src[:W])
    prop.synchronize()
    launches0 = prop.kernel_launches()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if clocks:
        clocks.start()
    group.barrier()
    torch.cuda.synchronize()
    ev0.record(stream)
    prop.run(K, prob.i_source, src[W:W + K])
    ev1.record(stream)
    prop.synchronize()
    torch.cuda.synchronize()
    group.barrier()
    clk = clocks.stop() if clocks else None
    ms = ev0.elapsed_time(ev1)
    launches = (prop.kernel_launches() - launches0) * LAUNCHES_PER_STEP[form]
    bpc = prop.bytes_per_cell()
    dev_gb = prop.device_bytes() / 1e9
    prop.finalize()
    Propagator(form="fp32")
    return ms, launches, bpc, dev_gb, clk, used_layout


def reference_parity(prob, steps, form, p, q):
    """Relative L2 of an FP32 run's final p and q against the reference's own
    OpenMP build on the same problem and step count: the committed fixture
    tests/golden/golden_c1.npz (504^3 interior, 1000 steps, every 12th cell
    per axis).  None for any other run."""
    path = os.path.join(ROOT, "tests", "golden", "golden_c1.npz")
    if form != "fp32" or not os.path.exists(path):
        return None
    g = np.load(path)
    meta = json.loads(str(g["meta"]))
    if meta["name"] != prob.name or meta["steps"] != steps or meta["seed"] != prob.seed:
        return None
    st = meta["stride"]

    def sub(a):
        return np.asarray(a).reshape(prob.sz, prob.sy, prob.sx)[::st, ::st, ::st].ravel().astype(np.float64)

    def rel(a, b):
        b = b.astype(np.float64)
        return float(np.linalg.norm(a - b) / np.linalg.norm(b))

    return {"vs": f"reference OpenMP build, {steps} steps (tests/golden/golden_c1.npz, every {st}th cell)",
            "rel_l2_p": float(f"{rel(sub(p), g['p']):.3e}"), "rel_l2_q": float(f"{rel(sub(q), g['q']):.3e}"),
            "tolerance": 1e-4}


def cpu_baseline_leg(prob, model, args):
    """The reference's own OpenMP build on this host's cores, on a bounded
    sample of the workload (a few full-grid steps); the oracle port on a
    slab when that build is absent."""
    r = reference_cpu(prob, args.cpu_steps, 1)
    if r is not None:
        out = {"value": round(r["msamples"], 2), "unit": UNIT, "cores": r["threads"], "kind": "reference",
               "sample": f"{args.cpu_steps} timed steps (after 1 untimed) of the full {prob.sx}^3 grid, "
                         f"{r['timed_s']:.1f} s in the reference's wtime() region; the reference's Model() loop "
                         "over its OpenMP back-end (oracle/_ref/ref_cli)", "build": r["build"]}
        return out
    import oracle

    t = oracle.time_slab(prob, model, nplanes=16, min_seconds=args.cpu_seconds)
    return {"value": round(t["msamples"], 2), "unit": UNIT, "cores": t["threads"], "kind": "port",
            "sample": f"{t['steps']} FP32 steps of a {t['planes']}-plane slab of the {prob.sx}^3 grid "
                      f"({t['cells']} updated cells/step, {t['seconds']:.1f} s), oracle restatement of "
                      "original/OpenMP/openmp_propagate.c + original/sample.h (reference build absent)"}


def run_gb300(args, ws, rank, local, group):
    import torch

    from fletcher_petrobras_gb300 import C1, Propagator
    from fletcher_petrobras_gb300._lib import fptr, load

    torch.cuda.set_device(local)
    lib = load()
    prob = workload(args)
    K, W = args.steps, args.warmup
    model = prob.model()
    form = args.form
    ms, launches, bpc, dev_gb, clk, layout = timed_run(prob, model, form, K, W, group, ClockSampler(local),
                                                      layout=args.coef_layout)

    ms_max = group.reduce(ms, "max")
    cells = prob.updated_cells
    value = ws * cells * K / (ms_max / 1e3) / 1e6  # all ranks' cells over the slowest rank's time
    per_launch_s = ms / 1e3 / K
    achieved = bpc * cells / per_launch_s / 1e9
    peak, peak_kind = measured_peak()
    tpc = ncu_traffic_per_cell(layout) if form == "fp32" else None

    # End to end through the C ABI with host buffers (the reference's Model() sequence).
    import ctypes as C

    stats = (C.c_double * 5)()
    e2e = e2e_wall = parity = e2e_clk = None
    KE = args.e2e_steps or prob.steps  # the workload's own step count (1000 at C1)
    if not args.no_e2e:
        # The caller's host arrays -- the six model arrays and the four
        # fields, zeroed as the reference's main() does (original/main.c:
        # 257-258) -- live in page-locked memory it allocated beforehand, so
        # every copy in the call runs from pinned host memory at the link's
        # rate (the library copies page-locked arrays as they are and locks
        # pageable ones for their copies, whose speed then depends on how the
        # system backs their pages).
        pin_f = torch.zeros((4, prob.n), dtype=torch.float32, pin_memory=True)
        pin_m = torch.empty((6, prob.n), dtype=torch.float32, pin_memory=True)
        f = pin_f.numpy()
        model_e2e = pin_m.numpy()
        model_e2e[...] = model
        from fletcher_petrobras_gb300.driver import FORMS

        from fletcher_petrobras_gb300.driver import COEF_LAYOUTS

        lib.FLETCHER_SetForm(FORMS[form])
        lib.FLETCHER_SetCoefLayout(COEF_LAYOUTS[args.coef_layout])
        lib.FLETCHER_SetStream(None)  # the library's own stream, as a plain C caller has it
        # Untimed warm-up: a 2-step call on the same buffers (their first
        # transfers set up the mappings of freshly locked memory), then the
        # fields are zeroed again.
        rc = lib.FLETCHER_Model(2, prob.i_source, prob.fcut, 0.0, prob.sx, prob.sy, prob.sz, prob.bord, prob.dx,
                                prob.dy, prob.dz, prob.dt, *[fptr(f[k]) for k in range(4)],
                                *[fptr(model_e2e[k]) for k in range(6)], stats)
        if rc:
            raise RuntimeError("FLETCHER_Model failed: " + lib.FLETCHER_GetLastErrorString().decode())
        f[...] = 0.0
        group.barrier()
        e2e_clocks = ClockSampler(local)
        e2e_clocks.start()
        rc = lib.FLETCHER_Model(KE, prob.i_source, prob.fcut, 0.01, prob.sx, prob.sy, prob.sz, prob.bord, prob.dx,
                                prob.dy, prob.dz, prob.dt, *[fptr(f[k]) for k in range(4)],
                                *[fptr(model_e2e[k]) for k in range(6)], stats)
        e2e_clk = e2e_clocks.stop()
        if rc:
            raise RuntimeError("FLETCHER_Model failed: " + lib.FLETCHER_GetLastErrorString().decode())
        lib.FLETCHER_SetForm(FORMS["fp32"])
        lib.FLETCHER_SetCoefLayout(COEF_LAYOUTS["planes"])
        phases = (C.c_double * 4)()
        lib.FLETCHER_ModelPhases(phases)
        init_phases = (C.c_double * 5)()
        lib.FLETCHER_InitPhases(init_phases)
        e2e_wall = group.reduce(stats[2], "max")
        e2e = ws * cells * KE / e2e_wall / 1e6
        parity = reference_parity(prob, KE, form, f[1], f[3])  # FLETCHER_Model leaves the final p, q in pc, qc
        del f, model_e2e, pin_f, pin_m

    # The other storage forms on the same workload (fewer steps).
    forms = {}
    if not args.no_forms:
        # The FP32 form in the other coefficient layout, then the 16-bit forms.
        other = "planes" if layout == "media" else "media"
        for key, f, lay in ((f"fp32-{other}", "fp32", other), ("fp16x", "fp16x", "planes"), ("fp16", "fp16", "planes")):
            if f == form and (f != "fp32" or other == layout):
                continue
            fk = max(1, min(K, args.form_steps))
            try:
                fms, _, fbpc, _, _, flay = timed_run(prob, model, f, fk, W, group, layout=lay)
            except Exception as exc:  # e.g. a model the media table cannot hold
                forms[key] = {"error": f"{type(exc).__name__}: {exc}"[:200]}
                continue
            fms = group.reduce(fms, "max")
            forms[key] = {"value": round(ws * cells * fk / (fms / 1e3) / 1e6, 1), "ms_per_step": round(fms / fk, 4),
                          "steps": fk, "bytes_per_cell": fbpc, "coef_layout": flay,
                          "hbm_gbs": round(fbpc * cells / (fms / 1e3 / fk) / 1e9, 1)}
        for f in forms:
            if "ms_per_step" in forms[f]:
                forms[f]["speedup_vs_this_form"] = round((ms_max / K) / forms[f]["ms_per_step"], 3)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline_leg(prob, model, args)

    # C3 (batched shots) and C4 (learned layer) on their own workloads.
    extra = {}
    if not args.no_c3c4 and prob.nx == 504:
        for key, fn in (("c3_batch", lambda: run_batch_form(args, ws, rank, local, group)),
                        ("c4_learned", lambda: run_learned_form(args, ws, rank, local, group))):
            try:
                extra[key] = fn()
            except Exception as exc:  # reported, not fatal to the C1 line
                extra[key] = {"error": f"{type(exc).__name__}: {exc}"[:300]}
    group.barrier()
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": round(value, 1), "unit": UNIT, "n_gpus": ws, "steps": K, "warmup": W,
        "ms_per_step": round(ms_max / K, 4), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if form == "fp32" else "f32 arithmetic, " + form + " storage", "data": "synthetic (seeded 8-layer TTI model, random-velocity boundary)",
        "config": {"workload": f"C1: {form.upper()} single shot, {prob.nx}^3 interior ({prob.sx}^3 grid), bord 4, "
                               f"absorb 32, dx 12.5 m, dt 0.6 ms, 8-layer seeded TTI, 15 Hz Ricker at {prob.src_xyz}",
                   "grid": [prob.sx, prob.sy, prob.sz], "updated_cells_per_step": cells,
                   "form": form, "coef_layout": layout, "parallelism": "replicas" if ws > 1 else "single GPU",
                   "l2": f"inputs resident in HBM ({dev_gb:.1f} GB) are larger than L2 (129 MB); no flush",
                   "timed_steps_include": "fused source injection + one propagate launch per step"},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "peak_kind": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                     "algorithmic_bytes_per_cell": bpc,
                     "traffic": None if tpc is None else round(tpc * cells / 1e9, 3),
                     "traffic_unit": "GB per launch (ncu dram__bytes_read.sum + dram__bytes_write.sum)",
                     "kernel": KERNEL[form] + (" (media-table layout)" if layout == "media" else "")},
        "e2e": None if e2e is None else {
                "value": round(e2e, 1), "unit": UNIT, "h2d_bytes_per_step": int(stats[3] / KE),
                "d2h_bytes_per_step": int(stats[4] / KE), "wall_s": round(e2e_wall, 3), "steps": KE,
                "phases_s": {"setup": round(phases[0], 3), "steps": round(phases[1], 3),
                             "snapshot_drain": round(phases[2], 3), "readback_finalize": round(phases[3], 3)},
                "setup_phases_s": dict(zip(("alloc", "lock_and_issue_copies", "device_work", "plan_and_maps",
                                            "unlock"), (round(v, 4) for v in init_phases))),
                "clocks": e2e_clk,
                "what": f"FLETCHER_Model via the C ABI, the workload's {KE} steps: DRIVER_Initialize (H2D of 6 "
                        "model + 4 field arrays, FP64 coefficient precompute) + per step (InsertSource, Propagate) "
                        "+ D2H snapshot of p every 0.01 s simulated + final D2H of p,q; the caller's host arrays "
                        "in page-locked memory allocated before the call; one untimed 2-step call before"},
        "gpu_launches": launches,
        "clocks": clk,
    }
    if parity:
        line["parity"] = parity
    if forms:
        line["forms"] = forms
    if cpu:
        line["cpu_baseline"] = cpu
    for k, v in extra.items():
        if v is not None:
            line[k] = v
    print(json.dumps(line), flush=True)


def run_batch_form(args, ws, rank, local, group, shots=None):
    """C3: 48 independent shots of uneven size run as one batch, the whole
    time loop one CUDA graph, tile shape from the autotuner, schedule chosen
    by the library (FLETCHER_BatchSetChains default: one chain of
    single-shot launches when the shots fill the GPU on their own, else one
    persistent launch per step for all running shots); against the same
    shots run one after another through the single-shot path (one launch
    per step each, no graph).  The other schedule is timed too."""
    import torch

    from fletcher_petrobras_gb300 import Propagator
    from fletcher_petrobras_gb300.autotune import tune_batch
    from fletcher_petrobras_gb300.batch import Batch, multishot_spec

    torch.cuda.set_device(local)
    spec = multishot_spec(shots or args.shots, seed=args.seed + rank)
    form = args.batch_form
    t0 = time.time()
    batch = Batch(form=form)
    for p in spec:
        batch.add(p)
    setup_s = time.time() - t0
    tune = tune_batch(batch, steps=10)
    batch.reset()
    group.barrier()
    l0 = batch.info()["launches"]
    ms = batch.run(use_graph=True)
    info = batch.info()
    launches = info["launches"] - l0
    chains = info["chains"]
    # The other schedule on the same shots.
    batch.reset()
    other = 0 if chains > 0 else 1
    batch.lib.FLETCHER_BatchSetChains(other)
    other_ms = batch.run(use_graph=True)
    batch.lib.FLETCHER_BatchSetChains(-1)
    batch.close()
    ms_max = group.reduce(ms, "max")
    value = group.reduce(info["cell_steps"], "sum") / (ms_max / 1e3) / 1e6
    # The same shots one at a time (single-shot kernel, one launch per step).
    seq_ms = 0.0
    if not args.no_sequential:
        stream = torch.cuda.Stream()
        for p in spec:
            prop = Propagator(stream=stream.cuda_stream, form=form)
            prop.initialize(p.sx, p.sy, p.sz, p.bord, p.dx, p.dy, p.dz, p.dt, p.model())
            ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            ev0.record(stream)
            prop.run(p.steps, p.i_source, p.sources())
            ev1.record(stream)
            prop.synchronize()
            seq_ms += ev0.elapsed_time(ev1)
            prop.finalize()
    if rank != 0:
        return
    line = {
        "metric": "MSamples/s, batched shots (C3)", "value": round(value, 1), "unit": UNIT, "n_gpus": ws,
        "steps": max(p.steps for p in spec), "ms_total": round(ms_max, 1), "higher_is_better": True,
        "scaling": "weak", "dtype": "f32" if form == "fp32" else f"f32 arithmetic, {form} storage",
        "data": f"synthetic ({len(spec)} seeded layered TTI shots)",
        "config": {"workload": f"C3: {len(spec)} shots, n ~ U{{96..320}}/8*8 per axis, 500-1500 steps, dt 0.6 ms, "
                               "the whole time loop one CUDA graph",
                   "schedule": (f"{chains} chain(s) of single-shot launches" if chains > 0
                                else "one persistent launch per step for all running shots"),
                   "storage": form,
                   "cell_steps": info["cell_steps"], "device_gb": round(info["device_bytes"] / 1e9, 1),
                   "setup_s": round(setup_s, 1), "tile": tune["tile"], "autotune": tune["ms_per_step"]},
        "gpu_launches": launches,
    }
    line["other_schedule"] = {
        "schedule": "one persistent launch per step" if other == 0 else "1 chain of single-shot launches",
        "ms_total": round(other_ms, 1), "value": round(info["cell_steps"] / (other_ms / 1e3) / 1e6, 1)}
    if seq_ms:
        line["sequential_single_shot"] = {"ms_total": round(seq_ms, 1),
                                          "value": round(info["cell_steps"] / (seq_ms / 1e3) / 1e6, 1),
                                          "speedup_of_batch": round(seq_ms / ms, 3)}
        line["other_schedule"]["speedup_vs_sequential"] = round(seq_ms / other_ms, 3)
    return line


def run_learned_form(args, ws, rank, local, group):
    """C4: the learned 8-cell absorbing layer against the 32-cell random
    shell, by default on a 256^3 interior for 1500 steps.  The network is
    trained first (plain-method runs on 64 padded layered models, the
    library's own training kernels); each form's interior MSamples/s is
    timed with CUDA events and its reflected energy measured against a
    wide-domain run."""
    import math

    import torch

    from fletcher_petrobras_gb300 import learned

    torch.cuda.set_device(local)
    t0 = time.time()
    ns = learned.collect(models=64, n_virtual=48, keep=0.1)
    t1 = time.time()
    learned.init(0)
    loss = learned.train(iters=args.abc_iters, batch=8192, lr=3e-3, noise=args.abc_noise)
    t2 = time.time()
    n, steps = args.abc_interior, args.abc_steps
    res = learned.compare(n=n, steps=steps, nsnap=5,
                          kinds=("random", "learned", "learned@2", "learned@4", "learned@8", "oneway", "plain8"))
    group.barrier()
    if rank != 0:
        return

    def fin(v):
        return v if isinstance(v, float) and math.isfinite(v) else None

    forms = {}
    for k, v in res.items():
        if k == "snapshots":
            continue
        forms[k] = {"interior_msamples": round(v["interior_msamples"], 1), "ms_per_step": round(v["ms_per_step"], 4),
                    "reflected_energy": fin(v["reflected_energy"]),
                    "reflected_energy_by_snapshot": [fin(e) for e in v.get("reflected_energy_by_snapshot", [])],
                    "launches_per_step": v.get("launches_per_step", 1), "tile": v.get("tile")}
    # The headline form: the network every 8 steps (the every-step form and
    # the other intervals are in "forms").
    head = "learned@8"
    lv, rv = res[head], res["random"]
    line = {
        "metric": "interior MSamples/s, learned 8-cell layer (network every 8 steps) vs 32-cell random boundary (C4)",
        "value": round(lv["interior_msamples"], 1), "unit": UNIT, "n_gpus": ws, "steps": steps,
        "higher_is_better": True, "scaling": "weak", "dtype": "f32 (network: f16 weights, f32 accumulation)",
        "data": "synthetic (seeded layered TTI models)",
        "config": {"workload": f"C4: {n}^3 interior, {steps} steps, dt 0.6 ms, 15 Hz Ricker 8 cells below the "
                               "interior top; forms: learned 8-cell layer (one-way update of its outer 4 cells with "
                               "the network's coefficients), the same with the medium's coefficients (oneway), "
                               "32-cell random-velocity shell, bare 8-cell layer (plain8), wide reflection-free "
                               "reference",
                   "snapshots": res["snapshots"],
                   "training": {"models": 64, "samples": ns, "collect_s": round(t1 - t0, 1),
                                "train_s": round(t2 - t1, 1), "iters": args.abc_iters, "batch": 8192,
                                "input_noise": args.abc_noise,
                                "loss_first": float(loss[:20].mean()), "loss_last": float(loss[-50:].mean())}},
        "speedup_vs_random": round(rv["ms_per_step"] / lv["ms_per_step"], 3),
        "reflected_energy_learned": fin(lv["reflected_energy"]),
        "reflected_energy_random": fin(rv["reflected_energy"]),
        "reflected_energy_oneway": fin(res["oneway"]["reflected_energy"]) if "oneway" in res else None,
        "learned_stable": fin(lv["reflected_energy"]) is not None and lv["reflected_energy"] < 1.0,
        "learned_form": head,
        "reflected_energy_learned_every_step": fin(res["learned"]["reflected_energy"]),
        "forms": forms,
    }
    return line


# Full-grid reference steps per run: the reference's OpenMP path takes about a
# second per 576^3 step on the GPU host's cores, so a run is capped to end
# within a few minutes.
REF_MAX_STEPS = 40
REF_MAX_WARMUP = 5


def reference_cpu(prob, steps, warmup, ftz=False):
    """The reference's own FP32 OpenMP build (oracle/_ref/ref_cli, the
    unmodified original/ sources) on the full grid of `prob`, all host cores,
    timed by its own wtime() region; None if that build is absent."""
    import oracle

    if not oracle.reference_cli_available(ftz):
        return None
    r = oracle.run_reference_cli(prob, steps + warmup, warmup, ftz=ftz, timeout=900)
    r["build"] = "gcc -O3 -fopenmp" + (" , linked with -ffast-math (FTZ/DAZ start-up only)" if ftz else
                                       " (original/Makefile flags, IEEE denormals)")
    return r


def run_reference(args, ws, rank, group):
    """`--impl reference`: the reference's own CPU implementation of the path
    on this host's cores, on the same workload (the C1 grid), through its own
    code: oracle/_ref/ref_cli runs the unmodified original/ front-end pieces
    (RandomVelocityBoundary, precomp.h, Source) and OpenMP back-end in the
    Model() loop, timed by the reference's wtime() region.  Rank 0 only.  The
    product library is not loaded.  Falls back to the oracle restatement on
    a 16-plane slab when the reference build is absent."""
    if rank != 0:
        return
    import oracle

    prob = workload(args)  # C1, or the same generator at another interior size
    K, W = args.steps, args.warmup
    k_run, w_run = min(K, REF_MAX_STEPS), min(W, REF_MAX_WARMUP)
    r = reference_cpu(prob, k_run, w_run)
    if r is not None:
        v = round(r["msamples"], 2)
        sample = (f"{k_run} timed steps (after {w_run} untimed) of the full {prob.sx}^3 grid"
                  + (f", capped from the {K} requested" if k_run < K else "")
                  + f"; set-up {r['setup_s'] + r['run_s'] - r['timed_s']:.1f} s untimed")
        cpu = {"value": v, "unit": UNIT, "cores": r["threads"], "kind": "reference", "sample": sample,
               "build": r["build"]}
        ftz = reference_cpu(prob, min(k_run, 5), min(w_run, 1), ftz=True)
        if ftz is not None:
            cpu["ftz"] = {"value": round(ftz["msamples"], 2), "steps": ftz["steps"] - ftz["warmup"],
                          "build": ftz["build"]}
        ms = 1e3 * r["timed_s"] / k_run
        desc = (f"C1: plain FP32 single shot, {prob.nx}^3 interior ({prob.sx}^3 grid), bord 4, absorb 32, "
                    f"dt 0.6 ms, 8-layer seeded TTI, 15 Hz Ricker at {prob.src_xyz}; the reference's OpenMP "
                    "back-end in its Model() loop")
        steps_line = k_run
    else:
        model = oracle.model(prob)
        if W:
            oracle.time_slab(prob, model, nplanes=16, steps=W)
        t = oracle.time_slab(prob, model, nplanes=16, steps=K)
        v = round(t["msamples"], 2)
        cpu = {"value": v, "unit": UNIT, "cores": t["threads"], "kind": "port",
               "sample": f"{K} steps of a {t['planes']}-plane slab of the {prob.sx}^3 grid (reference build absent)"}
        ms = 1e3 * t["seconds"] / K
        desc = (f"C1: plain FP32 single shot, {prob.nx}^3 interior ({prob.sx}^3 grid); each step is one propagation of a "
                    f"{t['planes']}-plane slab ({t['cells']} cells)")
        steps_line = K
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": ws, "steps": steps_line,
        "warmup": w_run if r is not None else W, "ms_per_step": round(ms, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded 8-layer TTI model)",
        "config": {"workload": desc, "grid": [prob.sx, prob.sy, prob.sz],
                   "updated_cells_per_step": prob.updated_cells},
        "cpu_baseline": cpu,
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "libraries_loaded": repo_libraries_loaded(),
    }
    print(json.dumps(line), flush=True)


def repo_libraries_loaded():
    """Shared libraries of this repository mapped into this process (the
    reference arm must show none of the product's)."""
    try:
        with open("/proc/self/maps") as f:
            paths = {ln.split()[-1] for ln in f if ln.rstrip().endswith(".so") and ROOT in ln}
    except OSError:
        return None
    return sorted(os.path.relpath(p, ROOT) for p in paths)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=15.0, help="slab sample length when the reference build is absent")
    ap.add_argument("--cpu-steps", type=int, default=3, help="full-grid steps of the reference build's CPU baseline")
    ap.add_argument("--e2e-steps", type=int, default=0, help="steps of the end-to-end run (0: the workload's own)")
    ap.add_argument("--no-c3c4", action="store_true", help="skip the batched-shot and learned-layer sub-benchmarks")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--interior", type=int, default=504, help="interior size n (n^3); 504 is the workload")
    ap.add_argument("--form", default="fp32", choices=["fp32", "fp16", "fp16x", "batch", "learned"])
    ap.add_argument("--abc-interior", type=int, default=256)
    ap.add_argument("--abc-steps", type=int, default=1500)
    ap.add_argument("--abc-iters", type=int, default=3000, help="Adam steps of the learned layer's training")
    ap.add_argument("--abc-noise", type=float, default=0.0, help="input noise (std) in the learned layer's training")
    ap.add_argument("--no-forms", action="store_true", help="skip timing the other storage forms")
    ap.add_argument("--coef-layout", default="planes", choices=["auto", "planes", "media"],
                    help="coefficient layout of the FP32 form (the other one is timed under forms)")
    ap.add_argument("--form-steps", type=int, default=200, help="timed steps of each other storage form")
    ap.add_argument("--shots", type=int, default=48)
    ap.add_argument("--batch-form", default="fp32", choices=["fp32", "fp16", "fp16x"],
                    help="storage form of the batched shots (--form batch)")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--no-sequential", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "gb300":
        args.warmup = 3
    ws, rank, local = dist_env()
    group = Group(ws)
    try:
        if args.impl == "reference":
            run_reference(args, ws, rank, group)
        elif args.form in ("batch", "learned"):
            fn = run_batch_form if args.form == "batch" else run_learned_form
            line = fn(args, ws, rank, local, group)
            if line is not None:
                print(json.dumps(line), flush=True)
        else:
            run_gb300(args, ws, rank, local, group)
    finally:
        group.close()


if __name__ == "__main__":
    main()
