"""Autotuner of the sky-loop launch shape.

A launch shape (pgw_tile_shape) fixes the sky directions per CTA
(threads / lanes_per_sky), the cluster pixels each lane walks
(1 / lanes_per_sky of them), the shared-memory pipeline (chunk size and
stages) and the compiled occupancy target.  The best one depends on the
detector count, the delay window, the sky size and the cluster-size mix, so
it is measured: every candidate runs the batched sky loop on a sample of
the workload (whole sky, a size-stratified subset of clusters) and is timed
with CUDA events; the fastest is kept in a JSON cache keyed by GPU and
problem class.
"""

from __future__ import annotations

import itertools
import json
import os
import threading

import numpy as np
import torch

from . import _lib

CACHE_PATH = os.environ.get(
    "PYCWB_GB300_TUNE_CACHE",
    os.path.join(os.environ.get("XDG_CACHE_HOME", os.path.join(os.path.expanduser("~"), ".cache")),
                 "pycwb_gb300", "tile_shapes.json"))
_lock = threading.Lock()


def candidates(n_ifo: int, fast_math: bool):
    """Launch shapes to try; fast_math selects the scan's arithmetic (True:
    refined division and approximate square root, False: IEEE rounding)."""
    out = []
    minbs = (3, 4) if n_ifo <= 4 else (2,)
    for threads, lanes, stages, chunk, minb in itertools.product((128, 256), (1, 2), (2, 3),
                                                                  (0, 16), minbs):
        out.append(_lib.TileShape(threads, lanes, chunk, stages, minb, 1 if fast_math else -1))
    return out


def problem_key(n_ifo, n_delay, n_sky, sizes, fast_math) -> str:
    name = torch.cuda.get_device_name() if torch.cuda.is_available() else "none"
    sizes = np.asarray(sizes)
    mean_bucket = int(2 ** round(np.log2(max(float(sizes.mean()), 1.0))))
    n_bucket = int(2 ** round(np.log2(max(len(sizes), 1))))
    return f"{name}|ifo{n_ifo}|d{n_delay}|s{n_sky}|meanP{mean_bucket}|n{n_bucket}|fast{int(fast_math)}"


def _load_cache():
    try:
        with open(CACHE_PATH) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(key, shape, timings):
    """Add one entry to the cache file: written to a file of this process
    and renamed over the cache, so that concurrent tuners never leave a torn
    file; without a writable cache the shape is simply measured again next
    time."""
    with _lock:
        cache = _load_cache()
        cache[key] = {"shape": list(shape.key()), "timings_ms": timings}
        tmp = f"{CACHE_PATH}.{os.getpid()}.tmp"
        try:
            os.makedirs(os.path.dirname(CACHE_PATH), exist_ok=True)
            with open(tmp, "w") as f:
                json.dump(cache, f, indent=1)
            os.replace(tmp, CACHE_PATH)
        except OSError:
            try:
                os.remove(tmp)
            except OSError:
                pass


def cached_shape(key):
    """The cached shape of a problem class, or None (also for an entry the
    cache holds in another form)."""
    ent = _load_cache().get(key)
    try:
        return None if ent is None else _lib.TileShape(*[int(v) for v in ent["shape"]])
    except (KeyError, TypeError, ValueError):
        return None


def time_shape(loop, shape, reps=2):
    """Median of `reps` timed launches (after one warm-up launch), in ms."""
    loop.shape = shape
    loop.launch()
    ts = []
    for _ in range(reps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(loop.stream)
        loop.launch()
        e1.record(loop.stream)
        e1.synchronize()
        ts.append(e0.elapsed_time(e1))
    return float(np.median(ts))


def sample_indices(sizes, n_sample=48, seed=0):
    """A size-stratified subset: every k-th cluster in size order."""
    order = np.argsort(np.asarray(sizes), kind="stable")
    if len(order) <= n_sample:
        return np.sort(order)
    pick = np.linspace(0, len(order) - 1, n_sample).round().astype(int)
    return np.sort(order[pick])


def autotune(tables, batch, fast_math=True, n_sample=48, reps=2, use_cache=True, verbose=False):
    """Best TileShape for this tables/batch problem class (measured)."""
    from .likelihoodWP.batched import BatchedSkyLoop, ClusterBatch

    key = problem_key(batch.n_ifo, batch.n_delay, tables.n_sky, batch.sizes, fast_math)
    if use_cache:
        hit = cached_shape(key)
        if hit is not None:
            return hit
    idx = sample_indices(batch.sizes, n_sample)
    sample = ClusterBatch(batch.n_ifo, batch.n_delay, batch.sizes[idx])
    for j, c in enumerate(idx):
        sample.set_cluster(j, *batch.cluster_views(int(c)))
    loop = BatchedSkyLoop(tables, sample)
    loop.upload()
    timings = {}
    best, best_t = None, float("inf")
    for shp in candidates(batch.n_ifo, fast_math):
        try:
            t = time_shape(loop, shp, reps)
        except ValueError:  # a shape this device or build cannot run
            continue
        timings[",".join(map(str, shp.key()))] = t
        if verbose:
            print(f"  shape {shp.key()}: {t:.3f} ms")
        if t < best_t:
            best, best_t = shp, t
    if best is None:
        raise RuntimeError("no candidate launch shape ran")
    _store(key, best, timings)
    return best
