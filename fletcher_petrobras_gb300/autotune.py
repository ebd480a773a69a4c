"""Tile-shape autotuner.

Times each built (tile rows, pipeline stages) shape on the actual problem for
a few steps and keeps the fastest; results are cached in a JSON file keyed by
GPU name, form and problem shape class, so later runs skip the search (the
reference's block-size tuners cached their choice per GPU and size in
configurations.txt, original_singleGPU_PDP/model.c:51-113).
"""
from __future__ import annotations

import json
import os

CANDIDATES = [(16, 5), (16, 4), (12, 5), (12, 4), (12, 6), (8, 5)]
HALF_CANDIDATES = [(16, 5), (16, 4), (12, 5), (12, 4), (12, 6), (8, 6)]  # built 16-bit shapes
DEFAULT_CACHE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build", "autotune.json")


def gpu_name() -> str:
    try:
        import torch

        return torch.cuda.get_device_name(0)
    except Exception:
        return "unknown-gpu"


def _load(path):
    try:
        with open(path) as f:
            return json.load(f)
    except Exception:
        return {}


def _store(path, data):
    os.makedirs(os.path.dirname(path), exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def tune_batch(batch, steps: int = 20, cache: str | None = DEFAULT_CACHE, candidates=None) -> dict:
    """Chooses the batch's tile shape: cached, or timed over `steps` steps per
    candidate (the fields are zeroed afterwards).  Returns the record."""
    from .batch import shape_class

    form = getattr(batch, "form", "fp32")
    if candidates is None:
        candidates = CANDIDATES if form == "fp32" else HALF_CANDIDATES
    key = f"{gpu_name()}|{form}|{shape_class(batch.probs)}"
    data = _load(cache) if cache else {}
    if key in data:
        rec = data[key]
        batch.set_tile(*rec["tile"])
        return dict(rec, cached=True)
    timings = {}
    for rows, stages in candidates:
        batch.set_tile(rows, stages)
        batch.run(max_steps=2)  # warm-up (graph build, first touch)
        batch.reset()
        ms = batch.run(max_steps=steps)
        batch.reset()
        timings[f"{rows}x{stages}"] = ms / steps
    best = min(timings, key=timings.get)
    rec = {"tile": [int(v) for v in best.split("x")], "ms_per_step": timings, "steps": steps}
    batch.set_tile(*rec["tile"])
    if cache:
        data[key] = rec
        _store(cache, data)
    return dict(rec, cached=False)
