"""Tile-shape autotuner: times each candidate launch configuration once with
CUDA events and caches the winner per (kernel, problem shape, device) in a
JSON file next to the built library."""
import json
import os
import threading

import torch

from . import build as _build

_PATH = os.path.join(_build.OUT_DIR, "autotune.json")
_lock = threading.Lock()
_cache = None


def _load():
    global _cache
    if _cache is None:
        try:
            with open(_PATH) as f:
                _cache = json.load(f)
        except (OSError, ValueError):
            _cache = {}
    return _cache


def _save():
    try:
        os.makedirs(os.path.dirname(_PATH), exist_ok=True)
        tmp = _PATH + ".tmp"
        with open(tmp, "w") as f:
            json.dump(_cache, f, indent=1, sort_keys=True)
        os.replace(tmp, _PATH)
    except OSError:
        pass


def time_fn(fn, reps=3):
    """Median CUDA-event time (ms) of fn() after one warm-up call."""
    fn()
    torch.cuda.synchronize()
    times = []
    for _ in range(reps):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        fn()
        b.record()
        b.synchronize()
        times.append(a.elapsed_time(b))
    times.sort()
    return times[len(times) // 2]


def choose(kernel, shape_key, candidates, run_candidate):
    """Returns the fastest candidate (cached).  ``run_candidate(c)`` launches
    the kernel once with candidate ``c`` on scratch buffers."""
    dev = torch.cuda.get_device_name()
    key = f"{kernel}|{shape_key}|{dev}"
    with _lock:
        cache = _load()
        if key in cache and cache[key]["best"] in candidates:
            return cache[key]["best"]
    results = {}
    for c in candidates:
        try:
            results[c] = time_fn(lambda: run_candidate(c))
        except (RuntimeError, NotImplementedError, ValueError):
            continue
    if not results:
        return candidates[0]
    best = min(results, key=results.get)
    with _lock:
        cache = _load()
        cache[key] = {"best": best, "ms": {str(k): v for k, v in results.items()}}
        _save()
    return best
