"""Host-side mirror of the reference's DEM interface, on top of libxdem.

Class and method names follow the reference so that code (and tests) written
against it read the same:

* ``NeighborhoodCell``  grid_base / neighborhood_cell (grid_base.h:7-64,
  neighborhood_cell.cpp:91-107): ``detection(pos, spos, np, snp)``,
  ``sortedID()``, ``cellStart()``, ``cellEnd()``.
* ``VelocityVerlet``    dem_integrator / velocity_verlet (dem_integrator.h:6-32,
  velocity_verlet.cpp:18-67): ``updatePosition``, ``updateVelocity``.
* ``ContactParticlesParticles``, ``ContactParticlesPlane``,
  ``ContactParticlesCube``, ``ContactParticlesPolygonObjects`` and
  ``ContactManager.runCollision`` (contactManager.cpp:82-185).
* ``DemSimulation``     dem_simulation (dem_simulation.cpp:204-469):
  ``initialize(scene)``, ``oneStepAnalysis()``.

Device memory comes from PyTorch (CUDA tensors); every compute call goes
through the C ABI of libxdem.  Struct arguments are the byte layouts of
metakonga_gb300.layouts, uploaded as uint8 tensors.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib
from ._lib import call, ptr
from .layouts import PARAMS

DEV = "cuda"


def stream_handle(stream=None) -> int:
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream


def to_dev(a: np.ndarray) -> torch.Tensor:
    """Copy a numpy array (any dtype, including structured) to a CUDA tensor."""
    a = np.ascontiguousarray(a)
    if a.dtype.names is not None or a.dtype == np.dtype("u1"):
        t = torch.from_numpy(a.view(np.uint8).reshape(-1).copy())
    else:
        t = torch.from_numpy(a.copy())
    return t.to(DEV)


def from_dev(t: torch.Tensor, like: np.ndarray = None) -> np.ndarray:
    out = t.detach().cpu().numpy()
    if like is not None and like.dtype.names is not None:
        return out.view(like.dtype).reshape(like.shape)
    return out


def set_symbolic_parameter(params: np.ndarray) -> None:
    """setSymbolicParameter (mphysics_cuda_def.cu:13-16)."""
    p = np.ascontiguousarray(params.reshape(()) if params.shape else params)
    assert p.dtype == PARAMS
    call("xd_set_symbolic_parameter", p.ctypes.data)


class NeighborhoodCell:
    """grid_base + neighborhood_cell (GPU branch of detection)."""

    def __init__(self):
        self.wo = (0.0, 0.0, 0.0)
        self.cs = 0.0
        self.gs = (0, 0, 0)
        self.ng = 0
        self.nse = 0

    def setWorldOrigin(self, wo):
        self.wo = tuple(float(v) for v in wo)

    def setCellSize(self, cs):
        self.cs = float(cs)

    def setGridSize(self, gs):
        self.gs = tuple(int(v) for v in gs)

    def nCell(self) -> int:
        return self.ng

    def initialize(self, n: int):
        """grid_base::initialize -> cuAllocMemory (grid_base.cpp:79-114)."""
        self.ng = self.gs[0] * self.gs[1] * self.gs[2]
        self.nse = n
        z = lambda m: torch.zeros(max(m, 1), dtype=torch.int32, device=DEV)
        self.d_cell_id = z(n)
        self.d_body_id = z(n)
        self.d_sorted_id = z(n)
        self.d_cell_start = z(self.ng)
        self.d_cell_end = z(self.ng)

    def detection(self, pos, spos=None, np_: int = 0, snp: int = 0, stream=None):
        """neighborhood_cell::detection (neighborhood_cell.cpp:91-107)."""
        s = stream_handle(stream)
        call("xd_calculate_hash_and_index", ptr(self.d_cell_id), ptr(self.d_body_id), ptr(pos), np_, s)
        if snp and spos is not None:
            call("xd_calculate_hash_and_index_polysphere", ptr(self.d_cell_id), ptr(self.d_body_id),
                 np_, snp, ptr(spos), s)
        call("xd_reorder_and_find_cell_start", ptr(self.d_cell_id), ptr(self.d_body_id),
             ptr(self.d_cell_start), ptr(self.d_cell_end), ptr(self.d_sorted_id), np_ + snp,
             self.ng, s)

    def sortedID(self):
        return self.d_sorted_id

    def cellStart(self):
        return self.d_cell_start

    def cellEnd(self):
        return self.d_cell_end

    def cellID(self):
        return self.d_cell_id

    def bodyID(self):
        return self.d_body_id


class VelocityVerlet:
    """velocity_verlet (GPU branch, velocity_verlet.cpp:18-43)."""

    VELOCITY_VERLET = 0

    def integrationType(self):
        return self.VELOCITY_VERLET

    def updatePosition(self, dpos, dvel, dacc, np_: int, stream=None):
        call("xd_vv_update_position", ptr(dpos), ptr(dvel), ptr(dacc), np_, stream_handle(stream))

    def updateVelocity(self, dvel, dacc, domega, dalpha, dforce, dmoment, dmass, dinertia,
                       np_: int, stream=None):
        call("xd_vv_update_velocity", ptr(dvel), ptr(dacc), ptr(domega), ptr(dalpha), ptr(dforce),
             ptr(dmoment), ptr(dmass), ptr(dinertia), np_, stream_handle(stream))


class ContactParticlesParticles:
    """contact_particles_particles::cuda_collision (contact_particles_particles.cpp:129-136)."""

    def __init__(self, cp: np.ndarray):
        self.dcp = to_dev(cp)

    def cuda_collision(self, pos, vel, omega, mass, force, moment, sorted_id, cell_start, cell_end,
                       np_: int, stream=None):
        call("xd_calculate_p2p", 1, ptr(pos), ptr(vel), ptr(omega), ptr(force), ptr(moment),
             ptr(mass), ptr(sorted_id), ptr(cell_start), ptr(cell_end), ptr(self.dcp), np_,
             stream_handle(stream))


class ContactParticlesPlane:
    """contact_particles_plane::cuda_collision (contact_particles_plane.cpp:33-51)."""

    def __init__(self, plane: np.ndarray, cp: np.ndarray):
        self.dpi = to_dev(plane)
        self.dcp = to_dev(cp)

    def cuda_collision(self, pos, vel, omega, mass, force, moment, sorted_id, cell_start, cell_end,
                       np_: int, stream=None):
        call("xd_plane_contact_force", 1, ptr(self.dpi), ptr(pos), ptr(vel), ptr(omega),
             ptr(force), ptr(moment), ptr(mass), np_, ptr(self.dcp), stream_handle(stream))


class ContactParticlesCube:
    """contact_particles_cube::cuda_collision (contact_particles_cube.cpp:36-43)."""

    def __init__(self, planes6: np.ndarray, cp: np.ndarray):
        assert planes6.shape[0] == 6
        self.dpi = to_dev(planes6)
        self.dcp = to_dev(cp)

    def cuda_collision(self, pos, vel, omega, mass, force, moment, sorted_id, cell_start, cell_end,
                       np_: int, stream=None):
        call("xd_cube_contact_force", 1, ptr(self.dpi), ptr(pos), ptr(vel), ptr(omega),
             ptr(force), ptr(moment), ptr(mass), np_, ptr(self.dcp), stream_handle(stream))


class ContactParticlesPolygonObjects:
    """contact_particles_polygonObjects (contact_particles_polygonObjects.cpp:47-123, 439-482)."""

    def __init__(self, poly: np.ndarray, sphere: np.ndarray, vlist: np.ndarray, pmi: np.ndarray,
                 cp: np.ndarray):
        self.npoly = poly.shape[0]
        self.nbodies = pmi.shape[0]
        self.dpi = to_dev(poly)
        self.dsphere = to_dev(sphere)
        self.dvlist = to_dev(vlist)
        self.dpmi = to_dev(pmi)
        self.dcp = to_dev(cp)
        self._pmi_dtype = pmi.dtype

    def SphereData(self):
        return self.dsphere

    def cuda_collision(self, pos, vel, omega, mass, force, moment, sorted_id, cell_start, cell_end,
                       np_: int, stream=None):
        call("xd_particle_polygon_collision", 1, ptr(self.dpi), ptr(self.dsphere), ptr(self.dpmi),
             ptr(pos), ptr(vel), ptr(omega), ptr(force), ptr(moment), ptr(mass), ptr(sorted_id),
             ptr(cell_start), ptr(cell_end), ptr(self.dcp), np_, self.nbodies,
             stream_handle(stream))

    def updatePolygonObjectData(self, pmi: np.ndarray = None, stream=None):
        """contact_particles_polygonObjects::updatePolygonObjectData (:258-328)."""
        if pmi is not None:
            self.dpmi.copy_(to_dev(pmi))
        call("xd_update_polygon_object_data", ptr(self.dpmi), ptr(self.dvlist), ptr(self.dsphere),
             ptr(self.dpi), self.npoly, stream_handle(stream))

    def bodies(self) -> np.ndarray:
        return from_dev(self.dpmi).view(self._pmi_dtype)


class ContactManager:
    """contactManager::runCollision -> deviceCollision (contactManager.cpp:82-185):
    particle-particle, then plane/cube contacts in name order, then polygons."""

    def __init__(self, cpp=None, cots=(), cppoly=None):
        self.cpp = cpp
        self.cots = list(cots)
        self.cppoly = cppoly

    def SphereData(self):
        return self.cppoly.SphereData() if self.cppoly else None

    def runCollision(self, pos, vel, omega, mass, force, moment, sorted_id, cell_start, cell_end,
                     np_: int, stream=None):
        if self.cpp:
            self.cpp.cuda_collision(pos, vel, omega, mass, force, moment, sorted_id, cell_start,
                                    cell_end, np_, stream)
        for c in self.cots:
            c.cuda_collision(pos, vel, omega, mass, force, moment, sorted_id, cell_start, cell_end,
                             np_, stream)
        if self.cppoly:
            self.cppoly.cuda_collision(pos, vel, omega, mass, force, moment, sorted_id, cell_start,
                                       cell_end, np_, stream)


class DemSimulation:
    """dem_simulation on the GPU (double precision), driven through the C ABI."""

    def initialize(self, scene):
        """dem_simulation::initialize (dem_simulation.cpp:204-325) from a
        metakonga_gb300.scenes.Scene (state already carries m g in force)."""
        self.np = scene.np_
        self.nPolySphere = scene.ntri
        self.dpos = to_dev(scene.pos)
        self.dvel = to_dev(scene.vel)
        self.dacc = to_dev(scene.acc)
        self.davel = to_dev(scene.omega)
        self.daacc = to_dev(scene.alpha)
        self.dforce = to_dev(scene.force)
        self.dmoment = to_dev(scene.moment)
        self.dmass = to_dev(scene.mass)
        self.diner = to_dev(scene.inertia)
        prm = scene.params
        self.dtor = NeighborhoodCell()
        self.dtor.setWorldOrigin(prm["world_origin"])
        self.dtor.setGridSize(prm["grid"])
        self.dtor.setCellSize(prm["cell_size"])
        self.dtor.initialize(self.np + self.nPolySphere)
        self.itor = VelocityVerlet()
        cots = [ContactParticlesPlane(scene.planes[i:i + 1], scene.cp_planes[i:i + 1])
                for i in range(scene.planes.shape[0])]
        cppoly = None
        if scene.ntri:
            cppoly = ContactParticlesPolygonObjects(scene.poly, scene.sphere, scene.vlist,
                                                    scene.pmi, scene.cp_poly)
        self.cm = ContactManager(ContactParticlesParticles(scene.cp_pp), cots, cppoly)
        p = scene.params.copy()
        p["np"] = self.np
        set_symbolic_parameter(p)
        return True

    def oneStepAnalysis(self, stream=None):
        """dem_simulation::oneStepAnalysis (dem_simulation.cpp:447-469)."""
        self.itor.updatePosition(self.dpos, self.dvel, self.dacc, self.np, stream)
        self.dtor.detection(self.dpos, self.cm.SphereData(), self.np, self.nPolySphere, stream)
        self.cm.runCollision(self.dpos, self.dvel, self.davel, self.dmass, self.dforce,
                             self.dmoment, self.dtor.sortedID(), self.dtor.cellStart(),
                             self.dtor.cellEnd(), self.np, stream)
        self.itor.updateVelocity(self.dvel, self.dacc, self.davel, self.daacc, self.dforce,
                                 self.dmoment, self.dmass, self.diner, self.np, stream)
        return True

    def state(self) -> dict:
        return {k: from_dev(getattr(self, d)) for k, d in
                (("pos", "dpos"), ("vel", "dvel"), ("acc", "dacc"), ("omega", "davel"),
                 ("alpha", "daacc"), ("force", "dforce"), ("moment", "dmoment"))}
