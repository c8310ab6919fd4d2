"""Autotuner of the grid-chunked path's chunk size, cached on disk.

The chunk size of ``engine.ChunkedResident`` trades device memory (one
chunk's AO tables and workspace) against the per-chunk fixed costs (table
packing launches, split-K tails, the last wave of each contraction).  For a
problem bucket (AO count rounded up to the tile of 128, arithmetic form,
network shape, GPU name) the tuner times the real call at each candidate
size that fits the memory budget, keeps the smallest size within ``tol`` of
the fastest, and records it in a JSON cache (``$GDFT_AUTOTUNE_CACHE``, by
default ``~/.cache/graddft_gb300/autotune.json``), so later processes reuse
the choice without timing.
"""
from __future__ import annotations

import json
import os
from typing import Callable, Iterable, Optional

import torch

CANDIDATES = (1 << 14, 1 << 15, 1 << 16, 1 << 17, 1 << 18)


def cache_path() -> str:
    return os.environ.get("GDFT_AUTOTUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "graddft_gb300", "autotune.json"))


def _load() -> dict:
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(table: dict) -> None:
    path = cache_path()
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        tmp = path + f".{os.getpid()}.tmp"
        with open(tmp, "w") as f:
            json.dump(table, f, indent=1, sort_keys=True)
        os.replace(tmp, path)
    except OSError:
        pass  # a read-only home: the choice is still used by this process


def bucket_key(n_ao: int, precision: str, net_key, device) -> str:
    name = torch.cuda.get_device_name(device)
    return f"chunk|{name}|{precision}|ao{-(-int(n_ao) // 128) * 128}|net{net_key}"


def time_call(fn: Callable[[], None], device, reps: int = 2) -> float:
    """Milliseconds per call of fn on the current stream (one untimed warm-up)."""
    fn()
    stream = torch.cuda.current_stream(device)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize(device)
    a.record(stream)
    for _ in range(reps):
        fn()
    b.record(stream)
    torch.cuda.synchronize(device)
    return a.elapsed_time(b) / reps


def choose(key: str, run: Callable[[int], None], ws_bytes: Callable[[int], int], n_grid: int, device,
           budget_bytes: Optional[int] = None, candidates: Iterable[int] = CANDIDATES, tol: float = 0.03) -> int:
    """The chunk size for a bucket: cached, or timed now with run(chunk) and cached.

    Sizes above the grid (rounded to 256) are not tried; nor are sizes whose
    workspace exceeds the budget (default: half of the device memory free now).
    """
    table = _load()
    if key in table:
        return int(table[key]["chunk"])
    if budget_bytes is None:
        free, _ = torch.cuda.mem_get_info(device)
        budget_bytes = free // 2
    top = max(256, -(-int(n_grid) // 256) * 256)
    sizes = sorted({min(int(c), top) for c in candidates})
    sizes = [c for c in sizes if ws_bytes(c) <= budget_bytes] or [sizes[0]]
    times = {}
    for c in sizes:
        times[c] = time_call(lambda c=c: run(c), device)
    best = min(times.values())
    chunk = min(c for c, t in times.items() if t <= (1.0 + tol) * best)
    table[key] = {"chunk": chunk, "ms": {str(c): round(t, 3) for c, t in times.items()}}
    _store(table)
    return chunk
