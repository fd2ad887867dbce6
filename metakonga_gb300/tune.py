"""Autotuner for the mixed form: skin width, list capacities, contact block.

The reference fixes its grid (128^3 cells of twice the largest radius,
dem_simulation.cpp:259-261) and its launch shapes.  The mixed form has five
choices that trade against each other differently per scene:

* the skin width (cells are 2 r_max + skin wide).  A wider skin re-bins less
  often (a particle may move half the skin before it must) but every list
  holds more neighbours, and the contact pass tests them all each step;
* the Verlet-list and triangle-list capacities: a particle whose list
  overflows has its contact pass search the cells instead (correct, slower);
* the contact pass's block size (32, 64 or 128 threads);
* its pair pass: a thread per listed particle (best when few particles touch
  anything) or warp-cooperative (the warp's contacts spread one per lane:
  best in packed beds).

``tune`` times candidate settings on a short window of the scene's own steps
(CUDA events, the same step graphs a run replays) and keeps the fastest; the
list capacities are raised where the defaults' lists overflowed.  Results
are cached in a JSON file keyed by the scene's shape -- particle count
(octave), radius spread, walls and triangles, packing -- so that similar
scenes reuse them (``tuned``).  Every setting gives the same contacts: the
choices change only how the contact pass finds them (and the two pair
passes give the same bits).
"""
from __future__ import annotations

import json
import math
import os
import time

import numpy as np

from . import engine

SKINS = (0.05, 0.1, 0.2, 0.35)
THREADS = (32, 64, 128)
MODES = (0, 1)


def cache_path() -> str:
    p = os.environ.get("XDEM_TUNE_CACHE")
    if p:
        return p
    return os.path.join(os.path.expanduser("~"), ".cache", "metakonga_gb300", "tuning.json")


def shape_key(sc) -> str:
    """The scene's shape: particle-count octave, radius spread (max / min, to
    0.5), plane and triangle counts, and packing (spheres per cubic largest
    diameter of the particles' bounding box, to a power of two)."""
    r = sc.pos[:, 3]
    n = sc.np_
    ext = np.maximum(sc.pos[:, :3].max(axis=0) - sc.pos[:, :3].min(axis=0), 2.0 * r.max())
    dens = n * (2.0 * r.max()) ** 3 / float(np.prod(ext))
    return (f"n2^{int(round(math.log2(max(n, 1))))}/spread{round(2 * r.max() / r.min()) / 2:g}/"
            f"planes{sc.planes.shape[0]}/tri{sc.ntri}/dens2^{int(round(math.log2(max(dens, 1e-6))))}")


def _load() -> dict:
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(cache: dict) -> None:
    p = cache_path()
    try:
        os.makedirs(os.path.dirname(p), exist_ok=True)
        tmp = p + ".tmp"
        with open(tmp, "w") as f:
            json.dump(cache, f, indent=1, sort_keys=True)
        os.replace(tmp, p)
    except OSError:
        pass


def tuned(sc) -> dict:
    """The cached tuning of the scene's shape, else the defaults."""
    return dict(_load().get(shape_key(sc), {}).get("tuning", engine.DEFAULT_TUNING))


def _time(sc, tuning, warm, steps):
    """ms per step of the scene with this tuning (CUDA events on the stream
    the steps run on) and its diagnostics."""
    import torch
    q = torch.cuda.Stream()
    d = engine.DeviceScene(sc, mode=engine.MODE_MIXED, tuning=tuning)
    try:
        d.step(warm, check=True, stream=q.cuda_stream)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(q)
        d.step(steps, check=False, stream=q.cuda_stream)
        e1.record(q)
        e1.synchronize()
        return e0.elapsed_time(e1) / steps, d.stats(q.cuda_stream)
    finally:
        d.close()


def tune(sc, steps: int = 200, warm: int = 20, store: bool = True, min_gain: float = 0.05) -> dict:
    """Times the candidates on `steps` steps of the scene (after `warm`
    steps) and returns {"tuning", "ms_per_step", "default_ms_per_step",
    "candidates", "key", "seconds"}; stores the choice in the cache.  A
    candidate replaces the choice so far only when it is faster by more than
    `min_gain` (timing noise and re-binnings falling in or out of the window
    move a short window by a few per cent)."""
    t0 = time.perf_counter()
    base = dict(engine.DEFAULT_TUNING)
    ms0, st0 = _time(sc, base, warm, steps)
    results = [(ms0, base)]
    # lists that overflowed at the default capacities search the cells: give
    # them room
    vcap, tcap = base["verlet_cap"], base["triangle_cap"]
    if st0["verlet_overflows"]:
        vcap = 96
    if st0["triangle_overflows"]:
        tcap = 48
    best = dict(base, verlet_cap=vcap, triangle_cap=tcap)
    best_ms = ms0 if (vcap, tcap) == (base["verlet_cap"], base["triangle_cap"]) else float("inf")
    for skin in SKINS:
        cand = dict(best, skin_factor=skin)
        if cand == base:
            continue
        ms, _ = _time(sc, cand, warm, steps)
        results.append((ms, cand))
        if ms < best_ms * (1.0 - min_gain):
            best, best_ms = cand, ms
    for th in THREADS:
        cand = dict(best, contact_threads=th)
        if any(c == cand for _, c in results):
            continue
        ms, _ = _time(sc, cand, warm, steps)
        results.append((ms, cand))
        if ms < best_ms * (1.0 - min_gain):
            best, best_ms = cand, ms
    for mode in MODES:
        cand = dict(best, contact_mode=mode)
        if any(c == cand for _, c in results):
            continue
        ms, _ = _time(sc, cand, warm, steps)
        results.append((ms, cand))
        if ms < best_ms * (1.0 - min_gain):
            best, best_ms = cand, ms
    out = {"key": shape_key(sc), "tuning": best, "ms_per_step": best_ms, "default_ms_per_step": ms0,
           "candidates": [{"tuning": c, "ms_per_step": m} for m, c in results],
           "window_steps": steps, "seconds": time.perf_counter() - t0}
    if store:
        cache = _load()
        cache[out["key"]] = {"tuning": best, "ms_per_step": best_ms, "default_ms_per_step": ms0}
        _store(cache)
    return out
