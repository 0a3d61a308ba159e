"""Autotuner of the launch shapes.

Chooses, on the device at hand, the strip rows of the resize and blur / FAST
pre-test kernels, the warps per block of the FAST cell kernel, the keypoints
per staging round and the rounds in flight of the descriptor kernel (each
timed on the pipeline stage it shapes, from the stage events of a batch
extraction) and the problem size from which the kNN uses the tensor cores
instead of the popcount kernel.  Launches too small to fill the device
(one frame, a few frames) follow the POLICIES below instead where they
apply.  Results never depend on these choices; only the time does.

The table is JSON keyed by workload: ``"<W>x<H>/<nFeatures>"`` for a single
frame configuration, ``"batch:"`` + the sorted distinct configurations for a
mix, and ``"knn"`` for the crossover.

    from orb_slam2_detailed_comments_gb300 import autotune
    entry = autotune.tune_batch(batch, images, nfeatures)
    autotune.save_table({autotune.workload_key(sizes, nfeatures): entry}, "tuning.json")
    autotune.apply(autotune.load_table("tuning.json")[key])
"""
from __future__ import annotations

import ctypes as C
import json
import os
import statistics
import time

from ._lib import check, lib

# parameter -> (candidate values, pipeline stage it shapes)
PARAMS = {
    "resize_rows": ((8, 22, 36, 64), "resize_blur"),
    "fast_cells_per_block": ((1, 2, 4), "fast"),
    "describe_group": ((1, 2, 4), "describe"),
    "describe_depth": ((2, 4), "describe"),
}
KNN_PARAM = "knn_tc_min_pairs"
# Launch policies for launches too small to fill the device (not tuned):
# keypoints per descriptor task and cells per FAST chunk (0: chosen from the
# launch's size) and the strip rows of short resize / blur launches (8; 0:
# resize_rows always), with their defaults; FULL_SIZE is what a launch that
# fills the device uses, which the tuner times the shapes under.
POLICIES = {"describe_task": 0, "fast_chunk": 0, "strip_rows_small": 8}
FULL_SIZE = {"describe_task": 32, "fast_chunk": 4, "strip_rows_small": 0}


def set_param(name: str, value: int) -> None:
    check(lib().orbgpu_tune_set(name.encode(), C.c_longlong(int(value))), f"orbgpu_tune_set({name})")


def get_param(name: str) -> int:
    v = C.c_longlong(0)
    check(lib().orbgpu_tune_get(name.encode(), C.byref(v)), f"orbgpu_tune_get({name})")
    return int(v.value)


def current() -> dict:
    return {name: get_param(name) for name in list(PARAMS) + list(POLICIES) + [KNN_PARAM]}


def workload_key(sizes, nfeatures) -> str:
    """sizes: [(w, h), ...] and nfeatures per frame (or one int for all)."""
    if isinstance(nfeatures, int):
        nfeatures = [nfeatures] * len(sizes)
    configs = sorted({f"{w}x{h}/{nf}" for (w, h), nf in zip(sizes, nfeatures)})
    return configs[0] if len(configs) == 1 else "batch:" + ",".join(configs)


def tune_batch(batch, images, nfeatures, reps: int = 5) -> dict:
    """Times every candidate of each parameter on the stage it shapes (median
    of 'reps' extractions, the other parameters at their current values and
    the small-launch policies at their full-size values), leaves the fastest
    applied and returns {name: {"value", "ms": {v: ms}}}."""
    out = {}
    policies = {name: get_param(name) for name in POLICIES}
    apply(FULL_SIZE)
    try:
        for name, (values, stage) in PARAMS.items():
            times = {}
            for v in values:
                set_param(name, v)
                batch.extract(images, nfeatures)  # re-plan, capture, warm
                samples = []
                for _ in range(reps):
                    batch.extract(images, nfeatures)
                    samples.append(batch.stage_times()[stage])
                times[v] = statistics.median(samples)
            best = min(times, key=times.get)
            set_param(name, best)
            out[name] = {"value": best, "ms": {str(k): round(t, 5) for k, t in times.items()}}
    finally:
        apply(policies)
    return out


def tune_knn(matcher, sizes=((2000, 8000), (8000, 32000), (20000, 80000), (50000, 200000)), seed: int = 1) -> dict:
    """Times the popcount and tensor-core kNN at growing sizes and sets the
    crossover to the first size where the tensor cores win (uniform random
    descriptors; the work per pair does not depend on the bits)."""
    import torch
    from . import synthetic as syn
    rows = []
    crossover = None
    for nq, nt in sizes:
        q = torch.from_numpy(syn.random_descriptors(nq, seed)).cuda()
        t = torch.from_numpy(syn.random_descriptors(nt, seed + 1)).cuda()
        ms = {}
        for algo in (0, 1):
            matcher.knn2(q, t, algo=algo)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for _ in range(3):
                matcher.knn2(q, t, algo=algo)
            torch.cuda.synchronize()
            ms[algo] = (time.perf_counter() - t0) / 3 * 1e3
        rows.append({"nq": nq, "nt": nt, "popc_ms": round(ms[0], 4), "tc_ms": round(ms[1], 4)})
        if crossover is None and ms[1] < ms[0]:
            crossover = nq * nt
    if crossover is None:
        crossover = 1 << 62
    set_param(KNN_PARAM, crossover)
    return {"value": crossover, "sizes": rows}


def apply(entry: dict) -> None:
    """Applies a table entry ({name: {"value": v}} or {name: v})."""
    for name, v in entry.items():
        set_param(name, v["value"] if isinstance(v, dict) else v)


def save_table(table: dict, path: str) -> None:
    old = load_table(path) if os.path.exists(path) else {}
    old.update(table)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(old, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def load_table(path: str) -> dict:
    with open(path) as f:
        return json.load(f)
