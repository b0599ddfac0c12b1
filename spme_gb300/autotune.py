"""Autotuner for the mesh-tile shape of the spread / interpolation kernels.

The tile (tx, ty, tz) sets how many particles each spread CTA stages (tile
plus a p-1 halo), the register footprint of its accumulators (tz planes), the
shared-memory halo box of the interpolation and the sort granularity.  The
best shape depends on density, mesh size, order and the number of
right-hand sides, so it is measured: each candidate runs a few position
builds + applies on the device (CUDA events on the engine's stream) and the
fastest is kept.  Results are cached in a JSON file keyed by the device name
and the configuration (N rounded to a power of two, K, p, R, precision,
terms).
"""
from __future__ import annotations

import json
import math
import os

CANDIDATES = [(8, 8, 8), (8, 8, 4), (8, 4, 4), (16, 4, 4), (16, 8, 8), (16, 8, 4),
              (16, 16, 4), (8, 16, 8), (4, 4, 4), (12, 12, 8)]


def cache_path() -> str:
    return os.environ.get("SPME_AUTOTUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "spme_gb300",
                                       "autotune.json"))


def config_key(device: str, np_: int, K: int, p: int, nrhs: int, precision: str,
               terms: int) -> str:
    nb = 1 << max(0, int(math.ceil(math.log2(max(np_, 1)))))
    return f"{device}|N{nb}|K{K}|p{p}|R{nrhs}|{precision}|t{terms}"


def _load_cache(path):
    try:
        with open(path) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return {}


def _save_cache(path, data):
    os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as fh:
        json.dump(data, fh, indent=1, sort_keys=True)
    os.replace(tmp, path)


def autotune(engine, pos, f, reps: int = 3, candidates=None, use_cache: bool = True,
             cache_file: str | None = None) -> tuple[tuple[int, int, int], dict]:
    """Pick the fastest tile for `engine` on positions `pos` (CUDA float64 tensor
    (N,3)) and right-hand sides `f` (CUDA tensor (nrhs, 3N) of the engine's
    precision).  Leaves the engine on the chosen tile with positions set.
    Returns (tile, {tile: ms per build+apply})."""
    import torch

    p = engine.params
    precision = "fp32" if engine.dtype.__name__ == "float32" else "fp64"
    key = config_key(torch.cuda.get_device_name(), p.np, p.dim, p.porder, f.shape[0],
                     precision, p.terms)
    path = cache_file or cache_path()
    cache = _load_cache(path) if use_cache else {}
    if key in cache:
        tile = tuple(cache[key]["tile"])
        engine.set_tile(*tile)
        engine.set_positions(pos)
        return tile, {tuple(map(int, k.split("x"))): v for k, v in cache[key]["ms"].items()}

    stream = torch.cuda.Stream()
    engine.set_stream(stream.cuda_stream)
    u = torch.zeros_like(f)
    timings = {}
    with torch.cuda.stream(stream):
        for tile in candidates or CANDIDATES:
            try:
                engine.set_tile(*tile)
                engine.set_positions(pos)
                engine.apply(f, u)  # warm-up (plans, descriptors)
            except Exception:
                continue  # shape not supported for this order / precision
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(reps):
                engine.set_positions(pos)
                engine.apply(f, u)
            e1.record(stream)
            stream.synchronize()
            timings[tile] = e0.elapsed_time(e1) / reps
    engine.set_stream(None)
    if not timings:
        raise RuntimeError("no tile candidate ran")
    best = min(timings, key=timings.get)
    engine.set_tile(*best)
    engine.set_positions(pos)
    if use_cache:
        cache[key] = {"tile": list(best), "ms": {"x".join(map(str, k)): v for k, v in timings.items()}}
        _save_cache(path, cache)
    return best, timings


BATCH_TILES = [(16, 8, 4), (8, 8, 8), (8, 8, 4), (16, 8, 8), (16, 16, 4)]
BATCH_OVERLAP = [0, 1, 2, 3]


def autotune_batch(batch, pos, f, u, reps: int = 3, tiles=None, overlaps=None) -> tuple:
    """Pick the interpolation tile (every system on the same tile) and the
    in-step concurrency (real-space sum on a second stream, cuFFT groups on
    four streams) of a native batch: each candidate times a few batched steps
    (CUDA events on torch's current stream).  Leaves the batch on the chosen
    settings.  Returns ((tile, overlap), {(tile, overlap): ms per step})."""
    import torch

    stream = torch.cuda.current_stream()

    def time_steps():
        batch.step(pos, f, u)  # capture (graphs on) and warm-up
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            batch.step(pos, f, u)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    timings = {}
    for tile in tiles or BATCH_TILES:
        try:
            batch.set_tile(*tile)
            batch.set_overlap(0)
            timings[(tile, 0)] = time_steps()
        except Exception:
            continue
    if not timings:
        raise RuntimeError("no tile candidate ran")
    best_tile = min(timings, key=timings.get)[0]
    batch.set_tile(*best_tile)
    for ov in overlaps or BATCH_OVERLAP:
        if (best_tile, ov) in timings:
            continue
        batch.set_overlap(ov)
        timings[(best_tile, ov)] = time_steps()
    best = min(timings, key=timings.get)
    batch.set_tile(*best[0])
    batch.set_overlap(best[1])
    batch.step(pos, f, u)
    torch.cuda.synchronize()
    return best, timings
