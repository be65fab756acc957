"""Launch-shape autotuner for the batched geocode.

For a batch it times a small set of persistent-kernel shapes — the tile
shape (32 x 8, 32 x 16 or 32 x 32 output pixels, i.e. 1, 2 or 4 geogrid
lines per thread; on UTM grids the tile is also the unit of the fitted
projection inverse), tiles taken per counter pop, persistent blocks per SM —
and the per-request form (each request's own fused kernel on concurrent
streams, which suits few large requests), with CUDA events on the real
requests, keeps the fastest, and caches the
choice in JSON keyed by GPU name and a hash of the batch's shape (request
count, tile count bucket, geogrid projection, geo2rdr precision), so later
batches of the same kind skip the search.
"""
from __future__ import annotations

import hashlib
import json
import threading
from pathlib import Path

import torch

from .batch import BatchTuning, GeocodeBatch

CACHE = Path(__file__).resolve().parent / "_build" / "autotune.json"
_lock = threading.Lock()


def _key(requests, precision: str, n_tiles: int) -> str:
    name = torch.cuda.get_device_name()
    epsg = requests[0].geogrid.epsg if requests else 0
    kind = "lonlat" if epsg == 4326 else "utm"
    bucket = max(n_tiles, 1).bit_length()
    raw = f"{name}|{precision}|{len(requests)}|{bucket}|{kind}"
    return hashlib.sha1(raw.encode()).hexdigest()[:16]


def _load() -> dict:
    try:
        return json.loads(CACHE.read_text())
    except (OSError, ValueError):
        return {}


def _store(d: dict) -> None:
    CACHE.parent.mkdir(exist_ok=True)
    tmp = CACHE.with_suffix(".tmp")
    tmp.write_text(json.dumps(d, indent=1, sort_keys=True))
    tmp.replace(CACHE)


def time_batch(batch: GeocodeBatch, reps: int = 2) -> float:
    """Mean ms per launch (CUDA events on the current stream), after one warm-up."""
    s = torch.cuda.current_stream()
    batch.run(s)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(reps):
        batch.launch(s)
    e1.record(s)
    batch.wait(s)
    return e0.elapsed_time(e1) / reps


def tune(requests, precision: str = "fp64", candidates=None, use_cache: bool = True, reps: int = 2):
    """Return (best BatchTuning, {tuning: ms}) for these requests."""
    probe = GeocodeBatch(requests, precision, BatchTuning())
    info = probe.info()
    key = _key(requests, precision, info["tiles"])
    with _lock:
        cache = _load() if use_cache else {}
    if key in cache:
        c = cache[key]
        probe.close()
        return (BatchTuning(c["tiles_per_pop"], c["blocks_per_sm"], True, c.get("rows_per_thread", 4),
                            bool(c.get("per_request", False))),
                {"cached": c["ms"]})
    occ = max(1, info["blocks"] // torch.cuda.get_device_properties(0).multi_processor_count)
    if candidates is None:
        if info["tiles"] > 50_000:      # large batches: a short search, one timed launch each
            candidates = [BatchTuning(p, occ, True, r) for r in (1, 2, 4) for p in (1, 2)]
            reps = 1
        else:
            candidates = [BatchTuning(p, b, True, r) for r in (1, 2, 4) for p in (1, 2, 4)
                          for b in sorted({occ, max(1, occ - 1)})]
        candidates.append(BatchTuning(per_request=True))
    results = {}
    best, best_ms = None, float("inf")
    probe.close()
    for t in candidates:
        b = GeocodeBatch(requests, precision, t)
        ms = time_batch(b, reps)
        b.close()
        results["per-request" if t.per_request else (t.rows_per_thread, t.tiles_per_pop, t.blocks_per_sm)] = ms
        if ms < best_ms:
            best, best_ms = t, ms
    if use_cache:
        with _lock:
            cache = _load()
            cache[key] = {"tiles_per_pop": best.tiles_per_pop, "blocks_per_sm": best.blocks_per_sm,
                          "rows_per_thread": best.rows_per_thread, "per_request": best.per_request, "ms": best_ms,
                          "gpu": torch.cuda.get_device_name(), "precision": precision, "requests": len(requests)}
            _store(cache)
    return best, results
