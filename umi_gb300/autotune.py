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
