"""Result and restart files: the reference's two formats, plus an exact checkpoint.

* ``part%04d.bin`` -- one output frame, written by ``dem_simulation::saveResult``
  (source/simulation/dem_simulation.cpp:491-519; single precision ``saveResult_f``
  :521-549): ``double ct``, ``uint32 np``, then ``pos[np][4]`` (x, y, z, r) in
  double, or in float for a single-precision model.
* ``<name>_final.bfr`` -- the restart file, written by
  ``xDynamicsSolver::saveFinalResult`` (source/xDynamicsSolver.cpp:111-130) and
  ``dem_simulation::saveFinalResult`` (dem_simulation.cpp:551-566): ``double ct``,
  ``int32 precision`` (2 double, 1 float), ``int32 flag`` (1), then
  ``pos[np][4]``, ``vel[np][3]``, ``avel[np][3]``.  The reader
  (``startingModel::setDEMData``, source/startingModel.cpp:32-66) takes np from
  the model, not from the file.  Neither file keeps the accelerations, so a run
  resumed from it restarts velocity Verlet with a = 0.
* checkpoint -- this library's own file: the whole scene state (positions,
  velocities, accelerations, angular velocities and accelerations, the force
  and moment arrays -- which hold m g and 0 between FP64 steps -- masses and
  inertias) in double, so that a resumed FP64 scene continues bit for bit.

All files are little-endian with no padding, as the reference writes them on
x86 Windows.
"""
from __future__ import annotations

import os
import struct

import numpy as np

_F64 = np.dtype("<f8")
_F32 = np.dtype("<f4")


def _prec_dtype(precision: int) -> np.dtype:
    if precision == 2:
        return _F64
    if precision == 1:
        return _F32
    raise ValueError(f"precision must be 2 (double) or 1 (float), got {precision}")


def part_name(directory: str, part: int) -> str:
    """The reference's frame path ``<directory>/part%04d.bin``."""
    return os.path.join(directory, "part%04d.bin" % part)


def write_part(path: str, ct: float, pos: np.ndarray, precision: int = 2) -> None:
    """One output frame in the reference's ``part%04d.bin`` layout."""
    dt = _prec_dtype(precision)
    pos = np.ascontiguousarray(pos, dtype=dt).reshape(-1, 4)
    with open(path, "wb") as f:
        f.write(struct.pack("<dI", float(ct), pos.shape[0]))
        f.write(pos.tobytes())


def read_part(path: str, precision: int = 2):
    """(ct, pos[np][4]) of a ``part%04d.bin`` frame."""
    dt = _prec_dtype(precision)
    with open(path, "rb") as f:
        head = f.read(12)
        if len(head) != 12:
            raise ValueError(f"{path}: truncated header")
        ct, np_ = struct.unpack("<dI", head)
        body = f.read()
    want = np_ * 4 * dt.itemsize
    if len(body) != want:
        raise ValueError(f"{path}: {len(body)} bytes of positions, expected {want} for np = {np_}")
    return ct, np.frombuffer(body, dtype=dt).reshape(np_, 4).copy()


def write_final(path: str, ct: float, pos: np.ndarray, vel: np.ndarray, avel: np.ndarray,
                precision: int = 2) -> None:
    """The reference's restart file ``<name>_final.bfr``."""
    dt = _prec_dtype(precision)
    pos = np.ascontiguousarray(pos, dtype=dt).reshape(-1, 4)
    n = pos.shape[0]
    vel = np.ascontiguousarray(vel, dtype=dt).reshape(n, 3)
    avel = np.ascontiguousarray(avel, dtype=dt).reshape(n, 3)
    with open(path, "wb") as f:
        f.write(struct.pack("<dii", float(ct), precision, 1))
        f.write(pos.tobytes())
        f.write(vel.tobytes())
        f.write(avel.tobytes())


def read_final(path: str, np_: int):
    """(ct, precision, pos, vel, avel) of a ``_final.bfr`` restart file holding
    np_ particles (the count comes from the model, as in the reference).  A
    file whose flag is not 1 carries no particle data: pos, vel and avel are None."""
    with open(path, "rb") as f:
        head = f.read(16)
        if len(head) != 16:
            raise ValueError(f"{path}: truncated header")
        ct, precision, flag = struct.unpack("<dii", head)
        if flag != 1:
            return ct, precision, None, None, None
        dt = _prec_dtype(precision)
        sizes = (np_ * 4, np_ * 3, np_ * 3)
        out = []
        for cnt in sizes:
            b = f.read(cnt * dt.itemsize)
            if len(b) != cnt * dt.itemsize:
                raise ValueError(f"{path}: truncated data for np = {np_}")
            out.append(np.frombuffer(b, dtype=dt).copy())
    return ct, precision, out[0].reshape(np_, 4), out[1].reshape(np_, 3), out[2].reshape(np_, 3)


_CKPT_MAGIC = b"XDEMCKP1"
_CKPT_FIELDS = (("pos", 4), ("vel", 3), ("acc", 3), ("omega", 3), ("alpha", 3), ("force", 3),
                ("moment", 3), ("mass", 1), ("inertia", 1))


def write_checkpoint(path: str, ct: float, state: dict, mass: np.ndarray, inertia: np.ndarray) -> None:
    """Exact checkpoint: ``XDEMCKP1``, double ct, uint64 np, then pos[4], vel,
    acc, omega, alpha, force, moment [3] and mass, inertia [1] per particle,
    all double.  ``state`` is a DeviceScene download."""
    pos = np.ascontiguousarray(state["pos"], dtype=_F64).reshape(-1, 4)
    n = pos.shape[0]
    arrays = {"pos": pos, "mass": mass, "inertia": inertia}
    for k in ("vel", "acc", "omega", "alpha", "force", "moment"):
        arrays[k] = state[k]
    with open(path, "wb") as f:
        f.write(_CKPT_MAGIC)
        f.write(struct.pack("<dQ", float(ct), n))
        for k, w in _CKPT_FIELDS:
            a = np.ascontiguousarray(arrays[k], dtype=_F64).reshape(n * w)
            f.write(a.tobytes())


def read_checkpoint(path: str):
    """(ct, dict of pos, vel, acc, omega, alpha, force, moment, mass, inertia)
    of a checkpoint."""
    with open(path, "rb") as f:
        if f.read(8) != _CKPT_MAGIC:
            raise ValueError(f"{path}: not a checkpoint of this library")
        ct, n = struct.unpack("<dQ", f.read(16))
        out = {}
        for k, w in _CKPT_FIELDS:
            b = f.read(n * w * 8)
            if len(b) != n * w * 8:
                raise ValueError(f"{path}: truncated {k}")
            a = np.frombuffer(b, dtype=_F64).copy()
            out[k] = a.reshape(n, w) if w > 1 else a
    return ct, out


def resume(scene, ct_path: str, mode: int):
    """A DeviceScene of `scene` (walls, meshes, parameters) with the state of
    checkpoint ``ct_path``; returns (scene object, ct)."""
    from . import engine
    ct, st = read_checkpoint(ct_path)
    sc = scene
    for k in ("pos", "vel", "acc", "omega", "alpha", "force", "moment", "mass", "inertia"):
        setattr(sc, k, st[k])
    return engine.DeviceScene(sc, mode=mode), ct
