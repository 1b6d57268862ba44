"""Tile-shape autotuner.

Times every candidate tile of a kernel on the caller's real shapes (device
CUDA events, a few repetitions after one untimed call) and keeps the fastest
in a JSON cache keyed by (tuning key, shape class, device name), so later
processes skip the sweep. The chosen value is installed in the library with
``totri_tune_set``; candidates the library refuses for a shape (tile too large
for the bin count) are skipped.

Cache file: $TOTRI_TUNE_CACHE, else ~/.cache/totri_gb300/tune.json.
"""
import json
import os
import threading

import torch

from . import _lib

CANDIDATES = {
    # 1 per-lane BVH walk, 2 warp-packet walk, 3 per-lane with postponed leaf tests
    # (point-major warps), 4 postponed leaf tests with face-major warps over
    # Morton-ordered wall-point patches (the built-in choice), 5 the same warps
    # walking as one packet, 6 the same warps over the 4-wide tree
    "mesh.visibility.mode": (3, 4, 6),
    "mesh.confocal.splat.ts": (1, 2, 4, 8, 16),
    "mesh.exhaustive.splat.lt": (1, 4, 8, 16, 32),
}

_lock = threading.Lock()


def cache_path():
    p = os.environ.get("TOTRI_TUNE_CACHE")
    if p:
        return p
    return os.path.join(os.path.expanduser("~"), ".cache", "totri_gb300", "tune.json")


def _load():
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _save(cache):
    path = cache_path()
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        tmp = path + ".tmp%d" % os.getpid()
        with open(tmp, "w") as f:
            json.dump(cache, f, indent=1, sort_keys=True)
        os.replace(tmp, path)
    except OSError:
        pass  # a read-only home still gets the in-process choice


def shape_class(**dims):
    """Buckets each dimension to the next power of two: 'F=32768,S=4096,T=1024'."""
    parts = []
    for k in sorted(dims):
        v = max(int(dims[k]), 1)
        parts.append("%s=%d" % (k, 1 << (v - 1).bit_length()))
    return ",".join(parts)


def set_tile(key, value):
    _lib.check(_lib.load().totri_tune_set(key.encode(), int(value)))


def get_tile(key):
    return int(_lib.load().totri_tune_get(key.encode()))


def _time(run, reps):
    stream = torch.cuda.current_stream()
    run()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        run()
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1) / reps


def tune(key, run, shape, reps=3, force=False):
    """Picks the fastest tile for `key` on `run()` (a closure launching the op
    with the real arguments) and installs it; returns (value, {value: ms})."""
    device = torch.cuda.get_device_name()
    ckey = "%s|%s|%s" % (key, shape, device)
    with _lock:
        cache = _load()
        if not force and ckey in cache:
            set_tile(key, cache[ckey]["best"])
            return cache[ckey]["best"], cache[ckey]["ms"]
        times = {}
        for cand in CANDIDATES[key]:
            set_tile(key, cand)
            try:
                times[cand] = _time(run, reps)
            except (ValueError, NotImplementedError):
                continue
        if not times:
            set_tile(key, 0)
            return 0, {}
        best = min(times, key=times.get)
        set_tile(key, best)
        cache[ckey] = {"best": best, "ms": {str(k): v for k, v in times.items()}}
        _save(cache)
        return best, times
