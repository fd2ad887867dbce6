"""Device-resident scenes (libxdem's xd_scene_* API).

``DeviceScene`` uploads a metakonga_gb300.scenes.Scene once and advances whole
steps on the GPU in the reference's order (dem_simulation::oneStepAnalysis,
dem_simulation.cpp:447-469), without per-step host work.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

# xd_scene_step_many overlaps scenes on 32 library streams; the device gives
# streams their own hardware queues only up to this count (default 8).  It
# takes effect when set before the process creates its CUDA context.
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

from . import _lib
from ._lib import call
from .layouts import PLANE

MODE_FP64 = 0
MODE_MIXED = 1


class _Desc(C.Structure):
    _fields_ = [
        ("params", C.c_byte * 112), ("np", C.c_uint), ("mode", C.c_int),
        ("cp_pp", C.c_byte * 88), ("nplanes", C.c_uint),
        ("planes", C.c_void_p), ("cp_planes", C.c_void_p),
        ("ntri", C.c_uint), ("nbodies", C.c_uint),
        ("poly", C.c_void_p), ("sphere", C.c_void_p), ("vlist", C.c_void_p),
        ("pmi", C.c_void_p), ("cp_poly", C.c_void_p),
    ]


assert C.sizeof(_Desc) == 280 and _Desc.planes.offset == 216 and _Desc.poly.offset == 240


def _addr(a):
    return None if a is None or a.size == 0 else a.ctypes.data


class Tuning(C.Structure):
    """xd_tuning: skin width over r_max, Verlet/triangle list capacities, the
    contact pass's block size and its pair pass (0 a thread per listed
    particle, 1 warp-cooperative; mixed form; set before the first upload)."""
    _fields_ = [("skin_factor", C.c_float), ("verlet_cap", C.c_uint), ("triangle_cap", C.c_uint),
                ("contact_threads", C.c_uint), ("contact_mode", C.c_uint)]

    def as_dict(self) -> dict:
        return {k: (round(float(getattr(self, k)), 6) if k == "skin_factor" else int(getattr(self, k)))
                for k, _ in self._fields_}


DEFAULT_TUNING = {"skin_factor": 0.1, "verlet_cap": 48, "triangle_cap": 16, "contact_threads": 64,
                  "contact_mode": 1}


class DeviceScene:
    def __init__(self, scene, mode: int = MODE_FP64, tuning: dict = None):
        if _lib.lib().xd_sizeof(b"xd_scene_desc") != C.sizeof(_Desc):
            raise RuntimeError("xd_scene_desc layout mismatch between binding and library")
        self.scene = scene
        self.np = scene.np_
        self.ntri = scene.ntri
        d = _Desc()
        p = scene.params.copy()
        p["np"] = scene.np_
        C.memmove(d.params, p.ctypes.data, 112)
        d.np = scene.np_
        d.mode = mode
        C.memmove(d.cp_pp, scene.cp_pp.ctypes.data, 88)
        self._keep = []
        planes = np.ascontiguousarray(scene.planes)
        cpl = np.ascontiguousarray(scene.cp_planes)
        self._keep += [planes, cpl]
        d.nplanes = planes.shape[0]
        d.planes, d.cp_planes = _addr(planes), _addr(cpl)
        if scene.ntri:
            arrs = [np.ascontiguousarray(a) for a in (scene.poly, scene.sphere, scene.vlist,
                                                      scene.pmi, scene.cp_poly)]
            self._keep += arrs
            d.ntri = scene.ntri
            d.nbodies = scene.pmi.shape[0]
            d.poly, d.sphere, d.vlist, d.pmi, d.cp_poly = (a.ctypes.data for a in arrs)
        h = C.c_void_p()
        call("xd_scene_create", C.addressof(d), C.addressof(h))
        self.handle = h
        if tuning is not None:
            t = Tuning(**dict(DEFAULT_TUNING, **tuning))
            call("xd_scene_set_tuning", self.handle, C.addressof(t))
        self.upload(scene)

    def tuning(self) -> dict:
        """The scene's tuning (mixed form)."""
        t = Tuning()
        call("xd_scene_get_tuning", self.handle, C.addressof(t))
        return t.as_dict()

    def upload(self, sc, stream: int = 0):
        arrs = [np.ascontiguousarray(getattr(sc, f)) for f in
                ("pos", "vel", "acc", "omega", "alpha", "force", "moment", "mass", "inertia")]
        call("xd_scene_upload", self.handle, *[a.ctypes.data for a in arrs], stream)

    def download(self, stream: int = 0) -> dict:
        n = self.np
        out = {"pos": np.empty((n, 4)), "vel": np.empty((n, 3)), "acc": np.empty((n, 3)),
               "omega": np.empty((n, 3)), "alpha": np.empty((n, 3)), "force": np.empty((n, 3)),
               "moment": np.empty((n, 3))}
        call("xd_scene_download", self.handle, *[out[k].ctypes.data for k in
                                                 ("pos", "vel", "acc", "omega", "alpha", "force",
                                                  "moment")], stream)
        return out

    def download_async(self, stream: int = 0):
        """Queue the state's download on `stream` into pinned host memory, in
        stream order (a later step on the stream cannot change what it
        copies); returns a function that, once the stream has passed the
        copy, gives the state as download() does."""
        import torch
        n = self.np
        shapes = (("pos", 4), ("vel", 3), ("acc", 3), ("omega", 3), ("alpha", 3))
        block = torch.empty(16 * n, dtype=torch.float64).pin_memory()
        views, off = {}, 0
        for k, w in shapes:
            views[k] = block[off:off + w * n]
            off += w * n
        call("xd_scene_download_async", self.handle, *[views[k].data_ptr() for k, _ in shapes], None, None,
             stream)

        def result():
            return {k: views[k].numpy().reshape(n, w).copy() for k, w in shapes}
        return result

    def device_state(self) -> dict:
        ptrs = [C.c_void_p() for _ in range(9)]
        call("xd_scene_device_state", self.handle, *[C.addressof(p) for p in ptrs])
        names = ("pos", "vel", "acc", "omega", "alpha", "force", "moment", "mass", "inertia")
        return {k: p.value for k, p in zip(names, ptrs)}

    def device_grid(self) -> dict:
        ptrs = [C.c_void_p() for _ in range(5)]
        call("xd_scene_device_grid", self.handle, *[C.addressof(p) for p in ptrs])
        return {k: p.value for k, p in zip(("hash", "index", "sorted", "cstart", "cend"), ptrs)}

    def download_grid(self, stream: int = 0) -> dict:
        ng = self.np + self.ntri
        nc = int(self.scene.params["ncell"])
        out = {"hash": np.empty(ng, np.uint32), "index": np.empty(ng, np.uint32),
               "sorted": np.empty(ng, np.uint32), "cstart": np.empty(nc, np.uint32),
               "cend": np.empty(nc, np.uint32)}
        call("xd_scene_download_grid", self.handle, *[out[k].ctypes.data for k in
                                                      ("hash", "index", "sorted", "cstart", "cend")],
             stream)
        return out

    def set_bodies(self, pmi: np.ndarray, stream: int = 0):
        a = np.ascontiguousarray(pmi)
        call("xd_scene_set_bodies", self.handle, a.ctypes.data, stream)

    def get_bodies(self, stream: int = 0) -> np.ndarray:
        out = np.zeros_like(self.scene.pmi)
        call("xd_scene_get_bodies", self.handle, out.ctypes.data, stream)
        return out

    def step(self, nsteps: int = 1, check: bool = False, stream: int = 0):
        call("xd_scene_step", self.handle, nsteps, 1 if check else 0, stream)

    PHASES = ("vv", "hash", "sort_cells", "p2p", "planes", "triangles", "reorder")

    def set_timing(self, enable: bool = True):
        call("xd_scene_set_timing", self.handle, 1 if enable else 0)

    def phase_times(self) -> dict:
        ms = np.zeros(len(self.PHASES))
        n = np.zeros(len(self.PHASES), np.uint64)
        call("xd_scene_phase_times", self.handle, ms.ctypes.data, n.ctypes.data)
        return {k: (float(ms[i]), int(n[i])) for i, k in enumerate(self.PHASES)}

    def eval_contacts(self, stream: int = 0):
        """Contact force/moment (no gravity) of the current state, original order."""
        f = np.empty((self.np, 3))
        m = np.empty((self.np, 3))
        call("xd_scene_eval_contacts", self.handle, f.ctypes.data, m.ctypes.data, stream)
        return f, m

    def pair_list(self, cap: int = 32, stream: int = 0):
        """(i, k) contact pairs of the current state (mixed mode), original ids."""
        counts = np.zeros(self.np, np.uint32)
        partners = np.zeros((self.np, cap), np.uint32)
        call("xd_scene_pair_list", self.handle, cap, counts.ctypes.data, partners.ctypes.data, stream)
        assert counts.max(initial=0) <= cap, "pair capacity exceeded"
        i = np.repeat(np.arange(self.np, dtype=np.uint32), counts)
        k = np.concatenate([partners[a, :c] for a, c in enumerate(counts)]) if counts.sum() else \
            np.zeros(0, np.uint32)
        return np.stack([i, k], axis=1)

    def counters(self, stream: int = 0):
        out = np.zeros(4, np.uint64)
        call("xd_scene_counters", self.handle, out.ctypes.data, stream)
        return {"contact_list": int(out[0]), "fp64_decisions": int(out[1]),
                "fp64_normal_forces": int(out[2]), "fp64_slips": int(out[3])}

    STATS = ("contact_list", "fp64_decisions", "fp64_normal_forces", "fp64_slips", "fp64_wall_regions",
             "rebinnings", "listed_with_triangles", "verlet_overflows", "triangle_overflows",
             "verlet_entries", "triangle_entries")

    def stats(self, stream: int = 0) -> dict:
        """Mixed-form diagnostics (xd_scene_stats): the counters above, FP64
        wall region tests, re-binnings, and list overflows at the last build."""
        out = np.zeros(len(self.STATS), np.uint64)
        call("xd_scene_stats", self.handle, out.ctypes.data, len(self.STATS), stream)
        return {k: int(v) for k, v in zip(self.STATS, out)}

    def rebuilds(self, stream: int = 0):
        """(re-binnings so far, kernel launches per re-binning) of a mixed scene."""
        cnt = np.zeros(1, np.uint64)
        each = np.zeros(1, np.uint64)
        call("xd_scene_rebuilds", self.handle, cnt.ctypes.data, each.ctypes.data, stream)
        return int(cnt[0]), int(each[0])

    def launches(self, nsteps: int) -> int:
        return int(_lib.lib().xd_scene_launches(self.handle, nsteps))

    def set_kinematic_bodies(self, enable: bool = True):
        """Move the polygon bodies by their own vel and omega every step, on the
        device (xd_scene_set_kinematic_bodies)."""
        call("xd_scene_set_kinematic_bodies", self.handle, 1 if enable else 0)

    def set_planes(self, planes, stream: int = 0):
        """Move the walls: a PLANE array of the scene's plane count, in its
        order (xd_scene_set_planes)."""
        arr = np.ascontiguousarray(planes, dtype=PLANE)
        if arr.shape != (self.scene.planes.shape[0],):
            raise ValueError("set_planes: the scene's plane count and order")
        call("xd_scene_set_planes", self.handle, arr.ctypes.data, stream)

    def set_emitter(self, period: int, groups=None, active: int = 0, stream: int = 0):
        """Emit the staged particles: only the first ``active`` take part; every
        ``period`` steps (from the next one) the next group of ``groups`` joins,
        one particle at a time when groups is None (xd_scene_set_emitter)."""
        if groups is None:
            g, ng = None, 0
        else:
            g = np.ascontiguousarray(groups, dtype=np.uint32)
            ng = int(g.shape[0])
            if ng == 0:
                period = 0
        call("xd_scene_set_emitter", self.handle, int(active), int(period),
             g.ctypes.data if ng else None, ng, stream)

    def active(self) -> int:
        """Particles taking part in the next step (xd_scene_active)."""
        out = np.zeros(1, np.uint32)
        call("xd_scene_active", self.handle, out.ctypes.data)
        return int(out[0])

    def set_particle_grid(self, grid=None, cell_size: float = None, origin=None):
        """FP64 form: the particles on a grid of their own (xd_scene_set_particle_grid),
        the triangles on the scene's.  With no arguments the grid is the one that
        holds the current particles unwrapped: cells of the largest diameter (or
        cell_size), the origin one cell below the lowest particle, power-of-two
        dimensions.  Returns (grid, cell size, origin)."""
        if grid is None:
            pos = self.download()["pos"]
            cell = float(2.0 * pos[:, 3].max()) if cell_size is None else float(cell_size)
            lo = pos[:, :3].min(axis=0) - cell
            hi = pos[:, :3].max(axis=0) + cell
            grid = [1 << int(np.ceil(np.log2(max(2.0, (h - l) / cell)))) for l, h in zip(lo, hi)]
            origin, cell_size = lo, cell
        g = np.ascontiguousarray(grid, np.uint32)
        o = np.ascontiguousarray(origin, np.float64)
        call("xd_scene_set_particle_grid", self.handle, g.ctypes.data, float(cell_size), o.ctypes.data)
        return [int(x) for x in g], float(cell_size), [float(x) for x in o]

    def set_tangential_history(self, slots: int = 12):
        """Tangential springs kept per contact (xd_scene_set_tangential_history);
        0 restores the reference's DHS model."""
        self.hist_slots = int(slots)
        call("xd_scene_set_tangential_history", self.handle, self.hist_slots)

    def download_history(self, stream: int = 0):
        """(keys [slots, np], delta [slots, np, 3], overflow) in original order."""
        k = np.zeros((self.hist_slots, self.np), np.uint32)
        d = np.zeros((self.hist_slots, self.np, 3))
        ov = np.zeros(1, np.uint64)
        call("xd_scene_download_history", self.handle, k.ctypes.data, d.ctypes.data, ov.ctypes.data, stream)
        return k, d, int(ov[0])

    def device_bytes(self) -> int:
        """Device memory the scene holds, in bytes."""
        out = np.zeros(1, np.uint64)
        call("xd_scene_device_bytes", self.handle, out.ctypes.data)
        return int(out[0])

    def close(self):
        if getattr(self, "handle", None) is not None and self.handle.value:
            call("xd_scene_destroy", self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def step_many(scenes, nsteps, check: bool = False, stream: int = 0) -> None:
    """Advance several DeviceScenes side by side (xd_scene_step_many): scene
    k by nsteps[k] steps (an int applies to all).  Each result equals the one
    the scene's own step gives alone."""
    scenes = list(scenes)
    k = len(scenes)
    if k == 0:
        return
    if isinstance(nsteps, (int, np.integer)):
        nsteps = [int(nsteps)] * k
    if len(nsteps) != k:
        raise ValueError("step_many: one step count per scene")
    if len({id(s) for s in scenes}) != k:
        raise ValueError("step_many: a scene appears twice")
    handles = (C.c_void_p * k)(*[s.handle.value for s in scenes])
    counts = np.ascontiguousarray(nsteps, dtype=np.uint32)
    call("xd_scene_step_many", C.cast(handles, C.c_void_p), counts.ctypes.data, k, 1 if check else 0, stream)


class Batch:
    """Mixed-form DeviceScenes advanced together (xd_batch_*): every step of
    every scene in one CUDA graph, each scene's result the same bits as when
    it is stepped alone.  Close it before its scenes."""

    def __init__(self, scenes):
        self.scenes = list(scenes)
        k = len(self.scenes)
        if len({id(s) for s in self.scenes}) != k:
            raise ValueError("Batch: a scene appears twice")
        handles = (C.c_void_p * k)(*[s.handle.value for s in self.scenes])
        out = C.c_void_p()
        call("xd_batch_create", C.cast(handles, C.c_void_p), k, C.byref(out))
        self.handle = out

    def step(self, nsteps: int, check: bool = False, stream: int = 0) -> None:
        call("xd_batch_step", self.handle, int(nsteps), 1 if check else 0, stream)

    def set_timing(self, enable: bool = True) -> None:
        """Direct launches with CUDA events around the advance and contact
        launches (xd_batch_set_timing)."""
        call("xd_batch_set_timing", self.handle, 1 if enable else 0)

    def kernel_times(self) -> dict:
        """{"advance": (ms, launches), "contact": (ms, launches), "walls": (ms, launches)} since
        timing was enabled: the advance, the pair pass (the whole contact pass in contact_mode
        0) and the wall pass that follows a cooperative pair pass."""
        ms = np.zeros(3)
        n = np.zeros(3, np.uint64)
        call("xd_batch_kernel_times", self.handle, ms.ctypes.data, n.ctypes.data)
        return {"advance": (float(ms[0]), int(n[0])), "contact": (float(ms[1]), int(n[1])),
                "walls": (float(ms[2]), int(n[2]))}

    def close(self) -> None:
        if self.handle:
            call("xd_batch_destroy", self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
