"""Autotuning of the traversal launch, cached on disk.

The native tuner (cbq_autotune) times every form (one thread per ray,
persistent with lane refill, octant-sorted persistent) x block size x refill
threshold x stack placement (shared or local memory) on the caller's rays and
keeps the fastest.  Results are cached in a JSON file keyed by GPU, DAG size
class (rounded log2 of its bytes) and ray mix (coherent or incoherent, from
how often consecutive rays share an octant), so a known configuration is
applied without re-timing.
"""
from __future__ import annotations

import json
import math
import os
from pathlib import Path

import numpy as np

import cubiquity_gb300 as cbq

CACHE_PATH = Path(os.environ.get("CBQ_AUTOTUNE_CACHE",
                                 str(Path.home() / ".cache" / "cubiquity_gb300" / "autotune.json")))


def ray_mix(direction) -> str:
    """'coherent' when >= 90% of consecutive rays (in a 65536-ray sample) share an octant."""
    d = direction[: 1 << 16]
    if not isinstance(d, np.ndarray):
        d = d.detach().cpu().numpy()
    sb = (d[:, 0] < 0).astype(np.int32) | ((d[:, 1] < 0).astype(np.int32) << 1) | ((d[:, 2] < 0).astype(np.int32) << 2)
    if sb.size < 2:
        return "coherent"
    return "coherent" if float((sb[1:] == sb[:-1]).mean()) >= 0.9 else "incoherent"


def cache_key(dag: cbq.Dag, direction) -> str:
    import torch
    gpu = torch.cuda.get_device_name() if torch.cuda.is_available() else "cpu"
    size_class = int(round(math.log2(max(1, dag.bytes))))
    layout = "|compact" if getattr(dag, "layout", 0) == cbq.LAYOUT_COMPACT else ""
    return f"{gpu}|dag2^{size_class}{layout}|{ray_mix(direction)}"


def _load() -> dict:
    try:
        return json.loads(CACHE_PATH.read_text())
    except (OSError, ValueError):
        return {}


def _store(cache: dict) -> None:
    try:
        CACHE_PATH.parent.mkdir(parents=True, exist_ok=True)
        tmp = CACHE_PATH.with_suffix(".tmp")
        tmp.write_text(json.dumps(cache, indent=1, sort_keys=True))
        os.replace(tmp, CACHE_PATH)
    except OSError:
        pass  # the cache is an optimisation only


def tune(dag: cbq.Dag, origin_tmax, direction, scratch, out: dict, compute_surface_properties=True,
         max_footprint=cbq.MAX_FOOTPRINT_DISABLED, use_tmax=False, repetitions: int = 3, use_cache: bool = True,
         stream=None, image_width: int = 0) -> dict:
    """Applies (and returns) the best launch config for this DAG and ray mix
    (rays taken in image tiles when image_width is given: tuned, and cached,
    apart from rays taken in order)."""
    key = cache_key(dag, direction) + ("|image" if image_width else "")
    cache = _load() if use_cache else {}
    if key in cache:
        cfg = dict(cache[key]["config"])
        cfg.setdefault("steps", 1)
        cfg.setdefault("registers", 0)
        dag.set_launch_config(cfg["kernel"], cfg["block"], cfg["chunk"], cfg["refill_min"], cfg["stack"], cfg["form"],
                              cfg["steps"], cfg["registers"])
        return dict(cfg, cached=True, key=key)
    cfg, ms = cbq.autotune_launch(dag, origin_tmax, direction, scratch, out, compute_surface_properties,
                                  max_footprint, use_tmax, repetitions, stream, image_width)
    if use_cache:
        cache = _load()
        cache[key] = {"config": cfg, "ms": ms, "rays": int(origin_tmax.shape[0])}
        _store(cache)
    return dict(cfg, cached=False, key=key, ms=ms)
