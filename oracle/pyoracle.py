"""ctypes access to the CPU oracle (TEST INFRASTRUCTURE ONLY).

``Oracle``      the C restatement, oracle/libxd_oracle.so (built by
                ``make -C oracle``; __graft_entry__.build() does this).
``RefKernels``  the reference's own kernels compiled as host code,
                oracle/_ref/libxdref.so (``make -C oracle ref``); only
                available where the reference tree is present.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
module; the product (metakonga_gb300) never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_ORACLE = os.path.join(HERE, "libxd_oracle.so")
LIB_REF = os.path.join(HERE, "_ref", "libxdref.so")
LIB_REF_LEGACY = os.path.join(HERE, "_ref", "libxdref_legacy.so")

_vp = C.c_void_p
_u = C.c_uint


def _p(a):
    if a is None:
        return None
    assert isinstance(a, np.ndarray) and a.flags["C_CONTIGUOUS"], "need a C-contiguous array"
    return a.ctypes.data_as(_vp)


def build_oracle(quiet: bool = True) -> str:
    subprocess.run(["make", "-C", HERE, "libxd_oracle.so"], check=True,
                   stdout=subprocess.DEVNULL if quiet else None)
    return LIB_ORACLE


class _Scene(C.Structure):
    _fields_ = [
        ("prm", C.c_byte * 112), ("np", _u),
        ("pos", _vp), ("vel", _vp), ("acc", _vp), ("omega", _vp), ("alpha", _vp),
        ("force", _vp), ("moment", _vp), ("mass", _vp), ("inertia", _vp),
        ("hash", _vp), ("index", _vp), ("sorted", _vp), ("cstart", _vp), ("cend", _vp),
        ("cp_pp", _vp), ("nplanes", _u), ("planes", _vp), ("cp_planes", _vp),
        ("ntri", _u), ("poly", _vp), ("sphere", _vp), ("pmi", _vp), ("cp_poly", _vp),
        ("hist", _vp), ("kinematic", C.c_int), ("nbodies", _u), ("vlist", _vp), ("emit", _vp),
    ]


class _Emitter(C.Structure):
    _fields_ = [("period", _u), ("groups", _vp), ("ngroups", _u), ("next", _u), ("active", _u),
                ("step", C.c_ulonglong)]


class _History(C.Structure):
    _fields_ = [("slots", _u), ("np", _u), ("key", _vp), ("delta", _vp), ("overflow", C.c_ulonglong)]


HIST_EMPTY = 0xFFFFFFFF
HIST_PLANE = 0x80000000
HIST_TRI = 0xC0000000


class History:
    """Tangential-spring history of a scene (xdo_history): up to `slots`
    contacts per particle, key[s, i] and delta[s, i, 3]."""

    def __init__(self, np_: int, slots: int = 12):
        assert 1 <= slots <= 32
        self.key = np.full((slots, np_), HIST_EMPTY, np.uint32)
        self.delta = np.zeros((slots, np_, 3))
        self.c = _History(slots, np_, self.key.ctypes.data, self.delta.ctypes.data, 0)

    @property
    def overflow(self) -> int:
        return int(self.c.overflow)

    def contacts(self, i: int) -> dict:
        """{key: delta} of particle i."""
        return {int(k): self.delta[s, i].copy() for s, k in enumerate(self.key[:, i]) if k != HIST_EMPTY}


class Emitter:
    """Particle emitter of a scene (xdo_emitter): the first `active` particles
    take part; before step k (1-based, counted from construction) with
    (k - 1) % period == 0 the next group joins (one particle when groups is
    None).  Keeps its state across ``Oracle.run`` calls."""

    def __init__(self, period: int, groups=None, active: int = 0):
        self.groups = None if groups is None else np.ascontiguousarray(groups, dtype=np.uint32)
        ng = 0 if self.groups is None else self.groups.shape[0]
        self.c = _Emitter(period, self.groups.ctypes.data if ng else None, ng, 0, active, 0)
        if self.groups is not None and ng == 0:
            self.c.period = 0

    @property
    def active(self) -> int:
        return int(self.c.active)

    @property
    def step(self) -> int:
        return int(self.c.step)


class Oracle:
    """The C restatement of the reference's FP64 GPU path (xdo_*) and CPU path (xdo_cpu_*)."""

    def __init__(self, path: str = LIB_ORACLE):
        if not os.path.exists(path):
            build_oracle()
        self.lib = C.CDLL(path)
        L = self.lib
        for name in ("xdo_calculate_hash_and_index", "xdo_calculate_hash_and_index_polysphere",
                     "xdo_reorder_and_find_cell_start", "xdo_vv_update_position",
                     "xdo_vv_update_velocity", "xdo_calculate_p2p", "xdo_plane_contact_force",
                     "xdo_cube_contact_force", "xdo_particle_polygon_collision", "xdo_cylinder_contact_force",
                     "xdo_update_polygon_object_data", "xdo_step", "xdo_run_steps",
                     "xdo_cpu_step", "xdo_cpu_run_steps", "xdo_contact_magnitudes"):
            getattr(L, name).restype = None
        L.xdo_pair_list.restype = C.c_ulonglong
        L.xdo_pair_list.argtypes = [_vp, _vp, _vp, _vp, _vp, _u, _vp, C.c_ulonglong]
        L.xdo_grid_hash.restype = _u
        for s in ("params", "plane", "polygon", "polygon_mass", "contact_property"):
            getattr(L, "xdo_sizeof_" + s).restype = _u

    def sizes(self):
        L = self.lib
        return {s: getattr(L, "xdo_sizeof_" + s)() for s in
                ("params", "plane", "polygon", "polygon_mass", "contact_property")}

    # ---- grid ----
    def hash_and_index(self, prm, pos, hash_, index):
        self.lib.xdo_calculate_hash_and_index(_p(prm), _p(hash_), _p(index), _p(pos), _u(pos.shape[0]))

    def hash_and_index_polysphere(self, prm, hash_, index, sid, sphere):
        self.lib.xdo_calculate_hash_and_index_polysphere(_p(prm), _p(hash_), _p(index), _u(sid),
                                                         _u(sphere.shape[0]), _p(sphere))

    def reorder(self, hash_, index, cstart, cend, sorted_, n, ncell):
        self.lib.xdo_reorder_and_find_cell_start(_p(hash_), _p(index), _p(cstart), _p(cend),
                                                 _p(sorted_), _u(n), _u(ncell))

    def detection(self, prm, pos, sphere=None):
        """Hash + sort + cell ranges (neighborhood_cell::detection GPU branch)."""
        npt = pos.shape[0]
        nt = 0 if sphere is None else sphere.shape[0]
        n = npt + nt
        ncell = int(prm["ncell"])
        h = np.zeros(n, np.uint32)
        ix = np.zeros(n, np.uint32)
        self.hash_and_index(prm, pos, h, ix)
        if nt:
            self.hash_and_index_polysphere(prm, h, ix, npt, sphere)
        cs = np.zeros(ncell, np.uint32)
        ce = np.zeros(ncell, np.uint32)
        so = np.zeros(n, np.uint32)
        self.reorder(h, ix, cs, ce, so, n, ncell)
        return h, ix, cs, ce, so

    # ---- integrator ----
    def vv_position(self, prm, pos, vel, acc):
        self.lib.xdo_vv_update_position(_p(prm), _p(pos), _p(vel), _p(acc), _u(pos.shape[0]))

    def vv_velocity(self, prm, vel, acc, omega, alpha, force, moment, mass, inertia):
        self.lib.xdo_vv_update_velocity(_p(prm), _p(vel), _p(acc), _p(omega), _p(alpha), _p(force),
                                        _p(moment), _p(mass), _p(inertia), _u(mass.shape[0]))

    # ---- contacts ----
    def p2p(self, prm, pos, vel, omega, force, moment, mass, sorted_, cstart, cend, cp):
        self.lib.xdo_calculate_p2p(_p(prm), _p(pos), _p(vel), _p(omega), _p(force), _p(moment),
                                   _p(mass), _p(sorted_), _p(cstart), _p(cend), _p(cp),
                                   _u(pos.shape[0]))

    def plane(self, prm, plane, pos, vel, omega, force, moment, mass, cp):
        self.lib.xdo_plane_contact_force(_p(prm), _p(plane), _p(pos), _p(vel), _p(omega), _p(force),
                                         _p(moment), _p(mass), _u(pos.shape[0]), _p(cp))

    def cylinder(self, prm, cyl, pos, vel, omega, force, moment, mass, cp, mpos, mf, mm):
        self.lib.xdo_cylinder_contact_force(_p(prm), _p(cyl), _p(pos), _p(vel), _p(omega), _p(force),
                                            _p(moment), _p(mass), _u(pos.shape[0]), _p(cp), _p(mpos),
                                            _p(mf), _p(mm))

    def cube(self, prm, planes6, pos, vel, omega, force, moment, mass, cp):
        self.lib.xdo_cube_contact_force(_p(prm), _p(planes6), _p(pos), _p(vel), _p(omega),
                                        _p(force), _p(moment), _p(mass), _u(pos.shape[0]), _p(cp))

    def polygon(self, prm, poly, sphere, pmi, pos, vel, omega, force, moment, mass, sorted_,
                cstart, cend, cp):
        self.lib.xdo_particle_polygon_collision(_p(prm), _p(poly), _p(sphere), _p(pmi), _p(pos),
                                                _p(vel), _p(omega), _p(force), _p(moment),
                                                _p(mass), _p(sorted_), _p(cstart), _p(cend),
                                                _p(cp), _u(pos.shape[0]))

    def advance_bodies(self, pmi, dt):
        self.lib.xdo_advance_bodies(_p(pmi), _u(pmi.shape[0]), C.c_double(dt))

    def update_polygon(self, pmi, vlist, sphere, poly):
        self.lib.xdo_update_polygon_object_data(_p(pmi), _p(vlist), _p(sphere), _p(poly),
                                                _u(poly.shape[0]))

    def contact_magnitudes(self, prm, pos, vel, omega, mass, sorted_, cstart, cend, cp, planes,
                           cp_planes):
        mag = np.zeros(pos.shape[0])
        npl = planes.shape[0]
        self.lib.xdo_contact_magnitudes(_p(prm), _p(pos), _p(vel), _p(omega), _p(mass), _p(sorted_),
                                        _p(cstart), _p(cend), _p(cp), _u(pos.shape[0]),
                                        _p(planes) if npl else None,
                                        _p(cp_planes) if npl else None, _u(npl), _p(mag))
        return mag

    def hist_p2p(self, prm, pos, vel, omega, force, moment, mass, sorted_, cstart, cend, cp,
                 history):
        self.lib.xdo_hist_p2p(_p(prm), _p(pos), _p(vel), _p(omega), _p(force), _p(moment),
                              _p(mass), _p(sorted_), _p(cstart), _p(cend), _p(cp),
                              _u(pos.shape[0]), C.byref(history.c))

    def hist_planes(self, prm, planes, cps, pos, vel, omega, force, moment, mass, history):
        self.lib.xdo_hist_planes(_p(prm), _p(planes), _p(cps), _u(planes.shape[0]), _p(pos),
                                 _p(vel), _p(omega), _p(force), _p(moment), _p(mass),
                                 _u(pos.shape[0]), C.byref(history.c))

    def pair_list(self, prm, pos, sorted_, cstart, cend, cap=None):
        npt = pos.shape[0]
        if cap is None:
            cap = 64 * npt + 16
        out = np.zeros((cap, 2), np.uint32)
        n = self.lib.xdo_pair_list(_p(prm), _p(pos), _p(sorted_), _p(cstart), _p(cend), _u(npt),
                                   _p(out), C.c_ulonglong(cap))
        assert n <= cap, "pair list overflow"
        return out[:n]

    # ---- whole steps ----
    def _scene_struct(self, sc, work):
        s = _Scene()
        C.memmove(s.prm, sc.params.ctypes.data, 112)
        s.np = sc.np_
        for f in ("pos", "vel", "acc", "omega", "alpha", "force", "moment", "mass", "inertia"):
            setattr(s, f, getattr(sc, f).ctypes.data)
        for f in ("hash", "index", "sorted", "cstart", "cend"):
            setattr(s, f, work[f].ctypes.data)
        s.cp_pp = sc.cp_pp.ctypes.data
        s.nplanes = sc.planes.shape[0]
        s.planes = sc.planes.ctypes.data if sc.planes.shape[0] else None
        s.cp_planes = sc.cp_planes.ctypes.data if sc.planes.shape[0] else None
        s.ntri = sc.ntri
        if sc.ntri:
            s.poly, s.sphere = sc.poly.ctypes.data, sc.sphere.ctypes.data
            s.pmi, s.cp_poly = sc.pmi.ctypes.data, sc.cp_poly.ctypes.data
            s.nbodies = sc.pmi.shape[0]
            s.vlist = sc.vlist.ctypes.data
        return s

    @staticmethod
    def _work(sc):
        n = sc.np_ + sc.ntri
        return {"hash": np.zeros(n, np.uint32), "index": np.zeros(n, np.uint32),
                "sorted": np.zeros(n, np.uint32), "cstart": np.zeros(sc.ncell, np.uint32),
                "cend": np.zeros(sc.ncell, np.uint32)}

    def work_arrays(self, sc):
        """Grid work arrays for ``run`` (allocate once, reuse across calls)."""
        return self._work(sc)

    def run(self, sc, nsteps: int, cpu_path: bool = False, history: "History" = None,
            kinematic: bool = False, emitter: "Emitter" = None, work=None):
        """Advance ``sc`` (in place) by nsteps whole steps; returns the grid work
        arrays (``work`` if given, else new ones).  With ``history`` the
        contacts keep tangential springs; with ``kinematic`` the polygon bodies
        move by their own vel and omega each step (xdo_advance_bodies); with
        ``emitter`` only its active particles take part (xdo_emitter)."""
        for a in ("pos", "vel", "acc", "omega", "alpha", "force", "moment", "mass", "inertia"):
            assert getattr(sc, a).flags["C_CONTIGUOUS"]
        if work is None:
            work = self._work(sc)
        s = self._scene_struct(sc, work)
        if history is not None:
            assert not cpu_path
            s.hist = C.addressof(history.c)
        if kinematic:
            assert not cpu_path and sc.ntri
            assert sc.vlist.flags["C_CONTIGUOUS"]
            s.kinematic = 1
        if emitter is not None:
            assert not cpu_path
            s.emit = C.addressof(emitter.c)
        fn = self.lib.xdo_cpu_run_steps if cpu_path else self.lib.xdo_run_steps
        fn(C.byref(s), _u(nsteps))
        return work


class RefKernels:
    """The reference's own kernels, compiled as host code (oracle/_ref)."""

    def __init__(self, path: str = LIB_REF):
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.lib = C.CDLL(path)
        for s in ("params", "plane", "polygon", "polygon_mass", "contact_property"):
            getattr(self.lib, "xdref_sizeof_" + s).restype = _u

    @staticmethod
    def available(path: str = LIB_REF) -> bool:
        return os.path.exists(path)

    def sizes(self):
        return {s: getattr(self.lib, "xdref_sizeof_" + s)() for s in
                ("params", "plane", "polygon", "polygon_mass", "contact_property")}

    def set_params(self, prm):
        self.lib.xdref_set_params(_p(prm))

    def hash_and_index(self, prm, pos, hash_, index):
        self.set_params(prm)
        self.lib.xdref_calculate_hash_and_index(_p(hash_), _p(index), _p(pos), _u(pos.shape[0]))

    def hash_and_index_polysphere(self, prm, hash_, index, sid, sphere):
        self.set_params(prm)
        self.lib.xdref_calculate_hash_and_index_polysphere(_p(hash_), _p(index), _u(sid),
                                                           _u(sphere.shape[0]), _p(sphere))

    def reorder(self, hash_, index, cstart, cend, sorted_, n, ncell):
        self.lib.xdref_reorder_and_find_cell_start(_p(hash_), _p(index), _p(cstart), _p(cend),
                                                   _p(sorted_), _u(n), _u(ncell))

    def detection(self, prm, pos, sphere=None):
        npt = pos.shape[0]
        nt = 0 if sphere is None else sphere.shape[0]
        n = npt + nt
        ncell = int(prm["ncell"])
        h = np.zeros(n, np.uint32)
        ix = np.zeros(n, np.uint32)
        self.hash_and_index(prm, pos, h, ix)
        if nt:
            self.hash_and_index_polysphere(prm, h, ix, npt, sphere)
        cs = np.zeros(ncell, np.uint32)
        ce = np.zeros(ncell, np.uint32)
        so = np.zeros(n, np.uint32)
        self.reorder(h, ix, cs, ce, so, n, ncell)
        return h, ix, cs, ce, so

    def vv_position(self, prm, pos, vel, acc):
        self.set_params(prm)
        self.lib.xdref_vv_update_position(_p(pos), _p(vel), _p(acc), _u(pos.shape[0]))

    def vv_velocity(self, prm, vel, acc, omega, alpha, force, moment, mass, inertia):
        self.set_params(prm)
        self.lib.xdref_vv_update_velocity(_p(vel), _p(acc), _p(omega), _p(alpha), _p(force),
                                          _p(moment), _p(mass), _p(inertia), _u(mass.shape[0]))

    def p2p(self, prm, pos, vel, omega, force, moment, mass, sorted_, cstart, cend, cp):
        self.set_params(prm)
        self.lib.xdref_calculate_p2p(C.c_int(1), _p(pos), _p(vel), _p(omega), _p(force),
                                     _p(moment), _p(mass), _p(sorted_), _p(cstart), _p(cend),
                                     _p(cp), _u(pos.shape[0]))

    def cylinder(self, prm, cyl, pos, vel, omega, force, moment, mass, cp, mpos, mf, mm):
        self.set_params(prm)
        self.lib.xdref_cylinder_contact_force(_p(cyl), _p(pos), _p(vel), _p(omega), _p(force), _p(moment),
                                              _p(mass), _u(pos.shape[0]), _p(cp), _p(mpos), _p(mf), _p(mm))

    def plane(self, prm, plane, pos, vel, omega, force, moment, mass, cp):
        self.set_params(prm)
        self.lib.xdref_plane_contact_force(C.c_int(1), _p(plane), _p(pos), _p(vel), _p(omega),
                                           _p(force), _p(moment), _p(mass), _u(pos.shape[0]),
                                           _p(cp))

    def cube(self, prm, planes6, pos, vel, omega, force, moment, mass, cp):
        self.set_params(prm)
        self.lib.xdref_cube_contact_force(C.c_int(1), _p(planes6), _p(pos), _p(vel), _p(omega),
                                          _p(force), _p(moment), _p(mass), _u(pos.shape[0]),
                                          _p(cp))

    def polygon(self, prm, poly, sphere, pmi, pos, vel, omega, force, moment, mass, sorted_,
                cstart, cend, cp):
        self.set_params(prm)
        self.lib.xdref_particle_polygon_collision(C.c_int(1), _p(poly), _p(sphere), _p(pmi),
                                                  _p(pos), _p(vel), _p(omega), _p(force),
                                                  _p(moment), _p(mass), _p(sorted_), _p(cstart),
                                                  _p(cend), _p(cp), _u(pos.shape[0]))

    def update_polygon(self, pmi, vlist, sphere, poly):
        self.lib.xdref_update_polygon_object_data(_p(pmi), _p(vlist), _p(sphere), _p(poly),
                                                  _u(poly.shape[0]))

    # ---- the reference's single-precision kernels (its float launchers, def.cu:254-466)

    def set_params_f(self, prm_f, hash_grid=None):
        """The float parameter block; hash_grid (an FP64 ``PARAMS`` record) sets
        the FP64 block whose grid size the reference's calcGridHash reads."""
        self.lib.xdref_set_params_f(_p(prm_f))
        if hash_grid is not None:
            self.lib.xdref_set_params(_p(hash_grid))

    def vv_position_f(self, pos, vel, acc):
        self.lib.xdref_vv_update_position_f(_p(pos), _p(vel), _p(acc), _u(pos.shape[0]))

    def vv_velocity_f(self, vel, acc, omega, alpha, force, moment, mass, inertia):
        self.lib.xdref_vv_update_velocity_f(_p(vel), _p(acc), _p(omega), _p(alpha), _p(force),
                                            _p(moment), _p(mass), _p(inertia), _u(mass.shape[0]))

    def detection_f(self, prm_f, pos, sphere=None):
        npt = pos.shape[0]
        nt = 0 if sphere is None else sphere.shape[0]
        n = npt + nt
        ncell = int(prm_f["ncell"])
        h = np.zeros(n, np.uint32)
        ix = np.zeros(n, np.uint32)
        self.lib.xdref_calculate_hash_and_index_f(_p(h), _p(ix), _p(pos), _u(npt))
        if nt:
            self.lib.xdref_calculate_hash_and_index_polysphere_f(_p(h), _p(ix), _u(npt), _u(nt),
                                                                 _p(sphere))
        cs = np.zeros(ncell, np.uint32)
        ce = np.zeros(ncell, np.uint32)
        so = np.zeros(n, np.uint32)
        self.lib.xdref_reorder_and_find_cell_start_f(_p(h), _p(ix), _p(cs), _p(ce), _p(so), _u(n),
                                                     _u(ncell))
        return h, ix, cs, ce, so

    def p2p_f(self, pos, vel, omega, force, moment, mass, sorted_, cstart, cend, cp):
        self.lib.xdref_calculate_p2p_f(_p(pos), _p(vel), _p(omega), _p(force), _p(moment),
                                       _p(mass), _p(sorted_), _p(cstart), _p(cend), _p(cp),
                                       _u(pos.shape[0]))

    def plane_f(self, plane, pos, vel, omega, force, moment, mass, cp):
        self.lib.xdref_plane_contact_force_f(_p(plane), _p(pos), _p(vel), _p(omega), _p(force),
                                             _p(moment), _p(mass), _u(pos.shape[0]), _p(cp))

    def cube_f(self, planes6, pos, vel, omega, force, moment, mass, cp):
        self.lib.xdref_cube_contact_force_f(_p(planes6), _p(pos), _p(vel), _p(omega), _p(force),
                                            _p(moment), _p(mass), _u(pos.shape[0]), _p(cp))

    def polygon_f(self, poly, sphere, pmi, pos, vel, omega, force, moment, mass, sorted_, cstart,
                  cend, cp):
        self.lib.xdref_particle_polygon_collision_f(_p(poly), _p(sphere), _p(pmi), _p(pos),
                                                    _p(vel), _p(omega), _p(force), _p(moment),
                                                    _p(mass), _p(sorted_), _p(cstart), _p(cend),
                                                    _p(cp), _u(pos.shape[0]))

    def step(self, sc):
        """One whole step in the reference's order, on the reference's kernels."""
        prm = sc.params
        self.vv_position(prm, sc.pos, sc.vel, sc.acc)
        h, ix, cs, ce, so = self.detection(prm, sc.pos, sc.sphere if sc.ntri else None)
        self.p2p(prm, sc.pos, sc.vel, sc.omega, sc.force, sc.moment, sc.mass, so, cs, ce, sc.cp_pp)
        for i in range(sc.planes.shape[0]):
            self.plane(prm, sc.planes[i:i + 1], sc.pos, sc.vel, sc.omega, sc.force, sc.moment,
                       sc.mass, sc.cp_planes[i:i + 1])
        if sc.ntri:
            self.polygon(prm, sc.poly, sc.sphere, sc.pmi, sc.pos, sc.vel, sc.omega, sc.force,
                         sc.moment, sc.mass, so, cs, ce, sc.cp_poly)
        self.vv_velocity(prm, sc.vel, sc.acc, sc.omega, sc.alpha, sc.force, sc.moment, sc.mass,
                         sc.inertia)
        return h, ix, cs, ce, so


class LegacyRefKernels:
    """The reference's legacy kernels (include/cu_dem_impl.cuh), compiled as
    host code (oracle/_ref/libxdref_legacy.so).  Arrays in the legacy layouts:
    pos, vel, acc, omega, alpha double4 rows, force and moment double3."""

    def __init__(self, path: str = LIB_REF_LEGACY):
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.lib = C.CDLL(path)
        for s_ in ("params", "plane", "polygon", "mass_info"):
            getattr(self.lib, "xdrefl_sizeof_" + s_).restype = _u
        for f in ("cube_hertzian_contact_force", "shape_hertzian_contact_force"):
            getattr(self.lib, "xdrefl_" + f).restype = None

    @staticmethod
    def available(path: str = LIB_REF_LEGACY) -> bool:
        return os.path.exists(path)

    def sizes(self):
        return {s_: getattr(self.lib, "xdrefl_sizeof_" + s_)() for s_ in ("params", "plane", "polygon", "mass_info")}

    def set_params(self, prm):
        self.lib.xdrefl_set_params(_p(prm))

    def vv_position(self, pos, vel, acc, np_):
        self.lib.xdrefl_vv_update_position(_p(pos), _p(vel), _p(acc), _u(np_))

    def vv_velocity(self, vel, acc, omega, alpha, force, moment, np_):
        self.lib.xdrefl_vv_update_velocity(_p(vel), _p(acc), _p(omega), _p(alpha), _p(force), _p(moment), _u(np_))

    def mergedata(self, data, pos, np_, vertice, snp):
        self.lib.xdrefl_mergedata(_p(data), _p(pos), _u(np_), _p(vertice), _u(snp))

    def hash_and_index(self, hash_, index, pos, n):
        self.lib.xdrefl_calculate_hash_and_index(_p(hash_), _p(index), _p(pos), _u(n))

    def reorder(self, hash_, index, cstart, cend, sorted_, n, nc):
        self.lib.xdrefl_reorder_and_find_cell_start(_p(hash_), _p(index), _p(cstart), _p(cend), _p(sorted_),
                                                    _u(n), _u(nc))

    def p2p(self, pos, vel, acc, omega, alpha, force, moment, sorted_, cstart, cend, np_):
        self.lib.xdrefl_calculate_p2p(_p(pos), _p(vel), _p(acc), _p(omega), _p(alpha), _p(force), _p(moment),
                                      _p(sorted_), _p(cstart), _p(cend), _u(np_), _u(0))

    def cube(self, planes, kn, vn, ks, vs, mu, line, pos, vel, omega, force, moment, np_):
        d = C.c_double
        self.lib.xdrefl_cube_hertzian_contact_force(_p(planes), d(kn), d(vn), d(ks), d(vs), d(mu), _p(line),
                                                    _p(pos), _p(vel), _p(omega), _p(force), _p(moment),
                                                    _u(np_))

    def shape(self, minfo, polygons, id_set, poly_start, poly_end, kn, vn, ks, vs, mu, line, pos, vel, omega,
              force, moment, np_, sorted_, cstart, cend):
        d = C.c_double
        out = np.zeros(3)
        self.lib.xdrefl_shape_hertzian_contact_force(_p(minfo), _p(polygons), _p(id_set), _p(poly_start),
                                                     _p(poly_end), d(kn), d(vn), d(ks), d(vs), d(mu), _p(line),
                                                     _p(pos), _p(vel), _p(omega), _p(force), _p(moment),
                                                     _u(np_), _p(sorted_), _p(cstart), _p(cend), _p(out))
        return out

    def update_polygons_position(self, mpos, A, local_vertice, pos):
        self.lib.xdrefl_update_polygons_position(_p(mpos), _p(A), _p(local_vertice), _u(local_vertice.shape[0]),
                                                 _p(pos))

    def update_polygons_information(self, polygons, indice, pos):
        self.lib.xdrefl_update_polygons_information(_p(polygons), _p(indice), _p(pos), _u(indice.shape[0]))
