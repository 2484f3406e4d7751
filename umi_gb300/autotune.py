"""Autotuning of the batched image operators, cached per (GPU, op, size class).

The tile-shape sweep itself is native (umi_autotune_batch times every
variant with CUDA events on the caller's stream); this module only keeps the
winners in a JSON file so that later runs on the same size class skip the
sweep.  Cache path: $UMI_AUTOTUNE_CACHE, else ~/.cache/umi_gb300/autotune.json.
"""
from __future__ import annotations

import json
import math
import os

import umi_gb300 as U

OP_NAMES = {U.OP_BILATERAL: "bilateral", U.OP_WFILTER_PP: "wfilter_pp", U.OP_COST_VOLUME: "cost_volume"}


def cache_path() -> str:
    return os.environ.get("UMI_AUTOTUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "umi_gb300", "autotune.json"))


def size_class(images) -> str:
    """Batch size class: image count and log2 of the mean pixel count."""
    if not images:
        return "empty"
    px = [max(1, t.shape[-2] * t.shape[-1]) for t, _, _ in images]
    mean = sum(px) / len(px)
    return f"n{len(images)}_px2^{round(math.log2(mean))}"


def _load() -> dict:
    try:
        return json.load(open(cache_path()))
    except (OSError, ValueError):
        return {}


def _store(d: dict) -> None:
    path = cache_path()
    os.makedirs(os.path.dirname(path), exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(d, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def tuned_variant(op: int, images, params=None, reps: int = 3, refresh: bool = False):
    """Best variant for this op and batch size class: from the cache, or measured now.

    Returns (variant, ms, from_cache)."""
    import torch
    key = f"{torch.cuda.get_device_name()}|{OP_NAMES[op]}|{size_class(images)}"
    cache = _load()
    # a cached winner stands while the operator offers the same variants
    if not refresh and key in cache and cache[key].get("variants") == U.batch_variants(op):
        return cache[key]["variant"], cache[key]["ms"], True
    v, ms = U.autotune_batch(op, images, params, reps=reps)
    cache[key] = {"variant": v, "ms": ms, "variants": U.batch_variants(op)}
    _store(cache)
    return v, ms, False


# ---- the fused launch: one variant per operator and image size class

SIZE_CLASSES = ((18, "px<2^18"), (20, "2^18<=px<2^20"), (99, "px>=2^20"))


def image_class(h: int, w: int) -> str:
    """Size class of one image by its pixel count (log2 buckets)."""
    lg = math.log2(max(1, h * w))
    for bound, name in SIZE_CLASSES:
        if lg < bound:
            return name
    return SIZE_CLASSES[-1][1]


def _time_fused(jobs, reps: int) -> float:
    import torch
    U.batch_run_fused(jobs)  # warm-up
    st = torch.cuda.current_stream()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(st)
    for _ in range(reps):
        U.batch_run_fused(jobs)
    b.record(st)
    b.synchronize()
    return a.elapsed_time(b) / reps


def tuned_fused_variants(jobs, reps: int = 3, refresh: bool = False):
    """Per-image variants for batch_run_fused, chosen per operator and size class.

    jobs: batch_run_fused's list [(op, images, params, variants_or_None), ...].
    For each filter operator (bilateral, per-pixel wfilter) and each size
    class present in its images, every fused variant of the operator (tile
    width x height = the P block, pixels per thread = Expand) is timed on that
    class's images alone (one fused launch per candidate, CUDA events) and the
    fastest wins; winners are cached per (GPU, operator, radius, class).  The
    cost volume has one fused form (tensor-core tiles of 128 pixels x 64
    disparities).  Returns (jobs with their variants filled in, report) with
    report[op_name][class] = {"variant", "ms", "images", "candidates_ms"}.
    """
    import torch
    cache = _load()
    gpu = torch.cuda.get_device_name()
    out_jobs, report = [], {}
    for op, images, params, _ in jobs:
        nvar = U.batch_fused_variants(op)
        if op == U.OP_COST_VOLUME or nvar <= 1:
            out_jobs.append((op, images, params, None))
            continue
        classes = {}
        for i, (inp, _, _) in enumerate(images):
            classes.setdefault(image_class(inp.shape[-2], inp.shape[-1]), []).append(i)
        variants = [0] * len(images)
        rep = {}
        radius = params.radius if params is not None else 0
        for cls, idx in sorted(classes.items()):
            key = f"{gpu}|fused|{OP_NAMES[op]}|r{radius}|{cls}"
            hit = cache.get(key)
            if not refresh and hit and hit.get("variants") == nvar:
                best, ms, cand = hit["variant"], hit["ms"], hit.get("candidates_ms")
            else:
                sub = [images[i] for i in idx]
                cand = {v: _time_fused([(op, sub, params, [v] * len(sub))], reps) for v in range(nvar)}
                best = min(cand, key=cand.get)
                ms = cand[best]
                cache[key] = {"variant": best, "ms": ms, "variants": nvar,
                              "candidates_ms": {str(k): v for k, v in cand.items()}}
            for i in idx:
                variants[i] = best
            rep[cls] = {"variant": best, "ms": ms, "images": len(idx), "candidates_ms": cand}
        report[OP_NAMES[op]] = rep
        out_jobs.append((op, images, params, variants))
    _store(cache)
    return out_jobs, report
