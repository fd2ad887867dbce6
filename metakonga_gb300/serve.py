"""Serving many DEM scenes on one GPU: admission by device memory, continuous
batching of their steps.

A ``Server`` takes requests (a scene and a step count) that arrive over time.
It admits a request as soon as the device memory the scene will hold fits in
the budget next to the scenes already resident, then advances every resident
scene by up to ``chunk`` steps per tick: as one ``engine.Batch`` (every step of
every resident scene in one CUDA graph) when asked to and they all take the
same number of steps and can be batched, else in one ``engine.step_many`` call (the scenes'
kernels side by side on the library's stream pool).  Requests that arrive
while others run join the next tick instead of waiting for the GPU to drain.  Ticks are queued ``depth`` deep: the host counts steps, marks
each tick with an event and only waits for the oldest mark, so the GPU is fed
while the host admits, downloads and retires.  A scene whose steps are done is
downloaded (on a side stream that waits for its last tick only) and freed when
the device is idle or memory is needed, which makes room for the next
request.  Each result is the one the scene gives when stepped alone (the step
sequence of a scene does not depend on how its steps are split into calls or
on what runs beside it).

The reference runs one model per process (xDynamicsSolver); this loop has no
counterpart there.
"""
from __future__ import annotations

import collections
import dataclasses
import math
import time

import numpy as np

from . import engine

_MIXED_PER_PARTICLE = 1100     # bytes: two state copies, view, lists, sort, transfer buffer
_FP64_PER_PARTICLE = 320       # bytes: reference layouts, grid arrays, sort scratch
_PER_TRIANGLE = 512            # bytes: records, circumspheres, vertex lists, cell ranges


def _mixed_cells(sc) -> tuple:
    """Cells of the mixed form's grid and its cell size (the rule of
    mixed_setup: bounding box of particles, planes and triangles, 4 r_max
    padding, cell = 2.002 r_max + skin + extent 2^-19, two margin cells)."""
    pts = [sc.pos[:, :3]]
    if sc.planes.shape[0]:
        for f in ("xw", "w2", "w3", "w4"):
            pts.append(np.asarray(sc.planes[f]).reshape(-1, 3))
    if sc.ntri:
        pts.append(sc.vlist.reshape(-1, 3))
    p = np.concatenate(pts)
    lo, hi = p.min(axis=0), p.max(axis=0)
    rmax = float(sc.pos[:, 3].max()) if sc.np_ else 0.5
    extent = float((hi - lo + 8.0 * rmax).max())
    cs = 2.0 * rmax * 1.001 + 0.1 * rmax + extent * 2.0 ** -19
    g = np.ceil((hi - lo + 4.0 * cs) / cs) + 3
    return float(np.prod(g)), cs, rmax


def estimate_device_bytes(sc, mode: int = engine.MODE_MIXED) -> int:
    """Upper estimate of the device memory a DeviceScene of `sc` holds once
    uploaded (what the server books against its budget)."""
    n, t = sc.np_, sc.ntri
    nb = 0 if not t else int(sc.pmi.shape[0])
    if mode == engine.MODE_MIXED:
        ncell, cs, rmax = _mixed_cells(sc)
        total = n * _MIXED_PER_PARTICLE + 8.0 * ncell
        if t:
            tri = sc.vlist.reshape(-1, 3, 3)
            edge = float(np.linalg.norm(tri - np.roll(tri, 1, axis=1), axis=2).max())
            reach = 2.0 * (1.1 * rmax + 1e-4)
            span = math.ceil((edge + 2.0 * reach) / cs) + 1.0
            # cell-triangle table (keys, triangles, sort buffers), per-particle
            # triangle lists and per-body reaction slots
            total += t * _PER_TRIANGLE + t * span ** 3 * 20.0 + n * (4 + 64 + 48 * nb)
    else:
        ncell = float(sc.params["ncell"])
        total = n * _FP64_PER_PARTICLE + t * (_PER_TRIANGLE + 16) + 8.0 * ncell
    return int(1.1 * total) + (4 << 20)


@dataclasses.dataclass
class Request:
    rid: object
    scene: object
    steps: int
    arrival: float                       # seconds after the server's start
    bytes: int = 0
    admitted: float = math.nan
    done: float = math.nan
    remaining: int = 0
    handle: object = None
    result: dict = None
    error: str = None                    # why the request failed (it is then not stepped further)
    fetch: object = None                 # cohorts: gives the result once its download has run
    held: bool = False                   # cohorts: finished, but its scene is still in a cohort's batch


class _Cohort:
    """Requests admitted together and stepped as one batch.  A member that
    finishes has its state downloaded in stream order and stays in the batch
    (stepped on, its result already taken) until enough of the cohort has
    finished to make a new batch worth its capture."""

    def __init__(self, reqs):
        self.reqs = list(reqs)
        self.batch = None                # engine.Batch, None (not made yet) or False (not batchable)


class _CudaMarks:
    """Tick marks: CUDA events on the server's stream, and a side stream for
    downloads that waits for one mark only."""

    def __init__(self, stream: int):
        import torch
        self.torch = torch
        self.main = torch.cuda.ExternalStream(stream) if stream else torch.cuda.current_stream()
        self.side = torch.cuda.Stream()

    def mark(self):
        ev = self.torch.cuda.Event()
        ev.record(self.main)
        return ev

    def wait(self, mark) -> None:
        mark.synchronize()

    def side_after(self, mark) -> int:
        self.side.wait_event(mark)
        return self.side.cuda_stream


class Server:
    """Continuous-batching DEM server on the current CUDA device.

    budget_bytes: device memory the resident scenes may hold together (a
    request larger than the budget is admitted alone when nothing else is
    resident).  chunk: steps per scene per tick; smaller chunks admit new
    requests sooner, larger ones cost fewer host calls.  depth: ticks queued
    on the device before the host waits for the oldest (0: wait for each).
    batch: step the resident scenes as an engine.Batch when they can be.  The
    batch is made again whenever the resident set changes, which waits for
    the device and captures its graphs; with a few resident scenes whose set
    changes every few ticks that costs more than it saves (measured on the
    served stream of the bench: p50 latency 1.43 s batched against 1.02 s),
    so it is off by default.
    cohorts: the requests admitted in one tick form a cohort stepped as one
    engine.Batch for as long as it lives: each tick advances a cohort by the
    chunk or up to its next member's last step, a finished member's state is
    downloaded in stream order and the member rides along until more than
    `dead_fraction` of the cohort's particles have finished (then the cohort
    is made again from its live members); more than `max_cohorts` cohorts
    are merged into one.  Batches are then made per admission wave and per
    re-forming, not per change of the resident set."""

    def __init__(self, budget_bytes: int, chunk: int = 20, mode: int = engine.MODE_MIXED,
                 stream: int = 0, keep_results: bool = True, clock=time.perf_counter, depth: int = 2,
                 marks=None, batch: bool = False, cohorts: bool = False, max_cohorts: int = 4,
                 dead_fraction: float = 0.5):
        if chunk < 1:
            raise ValueError("chunk must be >= 1")
        if depth < 0:
            raise ValueError("depth must be >= 0")
        self.budget = int(budget_bytes)
        self.chunk = int(chunk)
        self.depth = int(depth)
        self.marks = marks
        self.mode = mode
        self.stream = stream
        self.keep_results = keep_results
        self.clock = clock
        self.pending: list = []
        self.finished: list = []
        self.failed: list = []
        self.used = 0
        self.peak_used = 0
        self.ticks = 0
        self.peak_active = 0
        self.wall = 0.0
        self._to_close: list = []
        self.use_batch = batch
        self._batch = None
        self._batch_key = None
        self.batched_ticks = 0
        self.use_cohorts = cohorts
        self.max_cohorts = int(max_cohorts)
        self.dead_fraction = float(dead_fraction)
        self._cohorts: list = []
        self.batches_made = 0

    def _drop_batch(self) -> None:
        if self._batch is not None:
            self._batch.close()   # waits for the steps queued from it
        self._batch = None
        self._batch_key = None

    def _step(self, active: list, counts: list) -> None:
        handles = [r.handle for r in active]
        if self.use_batch and len(active) > 1 and len(set(counts)) == 1:
            key = tuple(id(h) for h in handles)
            if key != self._batch_key:
                self._drop_batch()
                self._batch_key = key
                try:
                    self._batch = engine.Batch(handles)
                except Exception:
                    self._batch = None   # not batchable (history, kinematics, FP64 form)
            if self._batch is not None:
                self._batch.step(counts[0], check=False, stream=self.stream)
                self.batched_ticks += 1
                return
        engine.step_many(handles, counts, check=False, stream=self.stream)

    # ---- cohorts ---------------------------------------------------------

    def _tick_cohorts(self) -> list:
        """One tick of every cohort; returns the requests that finished."""
        fin = []
        for c in self._cohorts:
            live = [r for r in c.reqs if r.remaining > 0]
            if not live:
                continue
            k = min(self.chunk, min(r.remaining for r in live))
            if c.batch is None and len(c.reqs) > 1:
                try:
                    c.batch = engine.Batch([r.handle for r in c.reqs])
                    self.batches_made += 1
                except Exception:
                    c.batch = False   # not batchable (history, kinematics, FP64 form)
            if c.batch:
                c.batch.step(k, check=False, stream=self.stream)
                self.batched_ticks += 1
            else:
                engine.step_many([r.handle for r in live], [k] * len(live), check=False, stream=self.stream)
            for r in live:
                r.remaining -= k
                if r.remaining == 0:
                    fin.append(r)
                    if self.keep_results:
                        r.fetch = r.handle.download_async(self.stream)
                    r.held = bool(c.batch)
        return fin

    def _reform_cohorts(self, force: bool = False) -> None:
        """Cohorts whose finished members hold more than dead_fraction of
        their particles (all of them with force) are made again from their
        live members; more than max_cohorts are merged into one.  Closing a
        batch waits for its queued steps; the finished members' scenes are
        then free to close."""
        keep = []
        for c in self._cohorts:
            dead = [r for r in c.reqs if r.remaining == 0]
            live = [r for r in c.reqs if r.remaining > 0]
            if dead:
                n_dead = sum(r.scene.np_ for r in dead)
                n_all = sum(r.scene.np_ for r in c.reqs)
                if force or not live or not c.batch or n_dead > self.dead_fraction * n_all:
                    if c.batch:
                        c.batch.close()
                    c.batch = None
                    for r in dead:
                        r.held = False
                    c.reqs = live
            if c.reqs:
                keep.append(c)
        if len(keep) > self.max_cohorts:
            for c in keep:
                if c.batch:
                    c.batch.close()
                for r in c.reqs:
                    if r.remaining == 0:
                        r.held = False
            keep = [_Cohort([r for c in keep for r in c.reqs if r.remaining > 0])]
        self._cohorts = keep

    def _close_cohorts(self) -> None:
        for c in self._cohorts:
            if c.batch:
                c.batch.close()
            for r in c.reqs:
                r.held = False
        self._cohorts = []

    def submit(self, rid, scene, steps: int, arrival: float = 0.0) -> None:
        if steps < 1:
            raise ValueError("a request needs at least one step")
        self.pending.append(Request(rid=rid, scene=scene, steps=int(steps), arrival=float(arrival),
                                    bytes=estimate_device_bytes(scene, self.mode),
                                    remaining=int(steps)))

    def _fits(self, r: Request, active: list) -> bool:
        # alone only when nothing else holds device memory
        return (not active and not self._to_close) or self.used + r.bytes <= self.budget

    def _admit(self, now: float, active: list, t0: float) -> None:
        # first come, first served: a request that does not fit holds back the
        # ones behind it, so that a large request is not starved
        while self.pending and self.pending[0].arrival <= now:
            r = self.pending[0]
            if not self._fits(r, active):
                break
            self.pending.pop(0)
            try:
                r.handle = engine.DeviceScene(r.scene, mode=self.mode)
            except Exception as e:   # a scene the library refuses fails alone
                r.error = f"admission: {e}"
                r.admitted = r.done = self.clock() - t0
                self.failed.append(r)
                continue
            r.admitted = self.clock() - t0
            self.used += r.bytes
            self.peak_used = max(self.peak_used, self.used)
            active.append(r)

    def run(self) -> list:
        """Serve every submitted request; returns them in completion order."""
        marks = self.marks if self.marks is not None else _CudaMarks(self.stream)
        self.pending.sort(key=lambda r: r.arrival)
        active: list = []
        inflight = collections.deque()   # (mark, requests whose last tick it ends)
        to_close = self._to_close = []    # retired, device memory not yet freed
        t0 = self.clock()

        def retire_one():
            mark, fin = inflight.popleft()
            marks.wait(mark)
            for r in fin:
                if self.keep_results:
                    r.result = r.fetch() if r.fetch is not None else r.handle.download(marks.side_after(mark))
                    r.fetch = None
                    # a state that blew up (non-finite positions or velocities)
                    # is reported as failed, the other requests unaffected
                    if not all(np.isfinite(r.result[k]).all() for k in ("pos", "vel") if k in r.result):
                        r.error = "non-finite state"
                r.done = self.clock() - t0
                self.finished.append(r)
                to_close.append(r)

        def close_finished():
            # freeing device memory synchronises the device: done when it is idle
            while inflight:
                retire_one()
            self._drop_batch()   # before any of its scenes
            held = [r for r in to_close if r.held]   # still inside a cohort's batch
            for r in to_close:
                if r.held:
                    continue
                r.handle.close()
                r.handle = None
                self.used -= r.bytes
            to_close[:] = held

        while self.pending or active or inflight:
            now = self.clock() - t0
            n_before = len(active)
            self._admit(now, active, t0)
            if self.use_cohorts and len(active) > n_before:
                self._cohorts.append(_Cohort(active[n_before:]))
            blocked = bool(self.pending and self.pending[0].arrival <= now
                           and not self._fits(self.pending[0], active))
            if blocked and to_close:
                if any(r.held for r in to_close):
                    self._reform_cohorts(force=True)   # their memory is needed now
                close_finished()
                continue
            if active:
                self.peak_active = max(self.peak_active, len(active))
                if self.use_cohorts:
                    fin = self._tick_cohorts()
                    active = [r for r in active if r.remaining > 0]
                    self._reform_cohorts()
                else:
                    counts = [min(self.chunk, r.remaining) for r in active]
                    self._step(active, counts)
                    fin, still = [], []
                    for r, c in zip(active, counts):
                        r.remaining -= c
                        (still if r.remaining else fin).append(r)
                    active = still
                self.ticks += 1
                inflight.append((marks.mark(), fin))
            while inflight and (len(inflight) > self.depth or not active):
                retire_one()
            if not active and not inflight:
                self._close_cohorts()
                if to_close:
                    close_finished()
                if self.pending:
                    time.sleep(max(0.0, self.pending[0].arrival - (self.clock() - t0)))
        self._close_cohorts()
        close_finished()
        self._drop_batch()
        self.wall = self.clock() - t0
        return self.finished

    def report(self) -> dict:
        """Completion latency (arrival to result) percentiles in ms, waiting
        time before admission, and the aggregate particle-steps/s."""
        if not self.finished:
            return {"requests": 0, "failed_admission": len(self.failed)}
        lat = np.array([r.done - r.arrival for r in self.finished]) * 1e3
        wait = np.array([r.admitted - r.arrival for r in self.finished]) * 1e3
        work = float(sum(r.scene.np_ * r.steps for r in self.finished))
        span = max(r.arrival for r in self.finished)
        return {"requests": len(self.finished),
                "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                "p50_wait_ms": float(np.percentile(wait, 50)),
                "p99_wait_ms": float(np.percentile(wait, 99)),
                "particle_steps": work, "wall_s": self.wall,
                "particle_steps_per_s": work / self.wall if self.wall > 0 else 0.0,
                "offered_particle_steps_per_s": work / span if span > 0 else None,
                "failed_admission": len(self.failed),
                "non_finite": sum(1 for r in self.finished if r.error),
                "ticks": self.ticks, "batched_ticks": self.batched_ticks, "batches_made": self.batches_made,
                "peak_active": self.peak_active,
                "peak_booked_bytes": self.peak_used}


def poisson_arrivals(count: int, rate: float, seed: int = 0) -> np.ndarray:
    """Arrival times (s) of a Poisson stream of `rate` requests per second."""
    rng = np.random.Generator(np.random.MT19937(seed))
    return np.cumsum(rng.exponential(1.0 / rate, size=count))
