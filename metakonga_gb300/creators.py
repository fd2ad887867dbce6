"""Particle creators of the reference's model files (particleManager): the
cube lattice, and the plane and circle creators whose layers are the groups
of a real-time emitter.

Each creator follows its reference function's layout arithmetic.  Two things
differ on purpose:

- ``frand()`` (C ``rand() / RAND_MAX``) is a seeded MT19937 stream here, drawn
  per particle in x, y, z order (the reference's draw order is the
  compiler's argument order and its seed the clock);
- a polydisperse plane or circle shape redraws the radii of its own
  particles only; the reference's loop runs over the manager's whole count
  from the shape's first particle, past the shape's end when it is not the
  first shape (particleManager.cpp:366-372, :481-487).
A stored initial-position file (the MAKING line's ``.par`` name) is not read.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np


def _u(x: float) -> int:
    """C++ ``static_cast<unsigned int>`` of a non-negative double."""
    return int(math.floor(x))


@dataclasses.dataclass
class Created:
    """Particles of one creator: positions (x, y, z, r) and the emitter
    groups it adds (empty for the cube)."""
    pos: np.ndarray
    groups: list


def _check_dims(nd, what):
    if any(v <= 0 for v in nd):
        raise ValueError(f"{what}: the shape is smaller than two particle diameters along an axis")


def cube_particles(dx, dy, dz, lx, ly, lz, min_radius, max_radius, rng) -> Created:
    """CreateCubeParticle (particleManager.cpp:214-298): a lattice of
    ndim = floor(dim / d) - 1 particles per axis (d = 2 r) from the start
    point, gaps ``space = (dim - d ndim) / (ndim + 1)``, each particle jittered
    by ``r space frand()`` per axis.  A polydisperse cube makes no particle
    (the reference lays out only min_radius == max_radius)."""
    if min_radius != max_radius:
        return Created(np.zeros((0, 4)), [])
    r = float(min_radius)
    d = 2.0 * r
    dim = np.array([dx, dy, dz], dtype=np.float64)
    nd = [_u(v / d) - 1 for v in dim]
    _check_dims(nd, "cube creator")
    ndv = np.array(nd, dtype=np.float64)
    space = (dim - d * ndv) / (ndv + 1.0)
    gab = d + space
    ran = r * space
    start = np.array([lx + r + space[0], ly + r + space[1], lz + r + space[2]])
    n = nd[0] * nd[1] * nd[2]
    pos = np.empty((n, 4))
    c = 0
    for z in range(nd[2]):
        for y in range(nd[1]):
            for x in range(nd[0]):
                f = rng.random(3)
                pos[c, 0] = start[0] + x * gab[0] + ran[0] * f[0]
                pos[c, 1] = start[1] + y * gab[1] + ran[1] * f[1]
                pos[c, 2] = start[2] + z * gab[2] + ran[2] * f[2]
                pos[c, 3] = r
                c += 1
    return Created(pos, [])


def plane_particles(dx, ny, dz, lx, ly, lz, min_radius, max_radius, rng) -> Created:
    """CreatePlaneParticle (particleManager.cpp:300-419): ``ny`` layers, all
    at height ly, of floor(dx / d) - 1 by floor(dz / d) - 1 particles
    (d = 2 max_radius) from (lx + space.x, lz + space.z), jittered by
    ``100 r space frand()`` in x and z; each layer is one emitter group.  A
    polydisperse shape draws its radii as min + (max - min) frand()."""
    r = float(max_radius)
    d = 2.0 * r
    nx, nz = _u(dx / d) - 1, _u(dz / d) - 1
    _check_dims((nx, nz), "plane creator")
    space_x = (dx - d * nx) / (nx + 1.0)
    space_z = (dz - d * nz) / (nz + 1.0)
    gab_x, gab_z = d + space_x, d + space_z
    ran_x, ran_z = 100.0 * r * space_x, 100.0 * r * space_z
    n = nx * int(ny) * nz
    pos = np.empty((n, 4))
    c = 0
    for _ in range(int(ny)):
        for z in range(nz):
            for x in range(nx):
                f = rng.random(2)
                pos[c] = (lx + space_x + x * gab_x + ran_x * f[0], ly,
                          lz + space_z + z * gab_z + ran_z * f[1], r)
                c += 1
    if min_radius != max_radius:
        pos[:, 3] = min_radius + (max_radius - min_radius) * rng.random(n)
    return Created(pos, [nx * nz] * int(ny))


def circle_particles(dia, ny, lx, ly, lz, min_radius, max_radius, rng) -> Created:
    """CreateCircleParticle (particleManager.cpp:421-510): ``ny`` layers, all
    at (lx, ly, lz), of a centre particle and nr = floor(R / d) - 1 rings
    (R = dia / 2, d = 2 max_radius); ring i has radius i (d + space) with
    space = (R - d nr - r) / (nr + 1) and floor(2 pi / dth) particles,
    dth = (d + space) / (i (d + space)).  A layer's emitter group counts its
    ring particles only, as the reference's does (the centre is not counted:
    the last ny particles are never emitted)."""
    r = float(max_radius)
    cr = 0.5 * dia
    nr = _u(cr / (2.0 * r)) - 1
    _check_dims((nr,), "circle creator")
    rr = 2.0 * r * nr + r
    space = (cr - rr) / (nr + 1)
    rows = []
    npg_layer = 0
    ring = []
    for i in range(1, nr + 1):
        _r = i * (2.0 * r + space)
        dth = (2.0 * r + space) / _r
        npr = _u((2.0 * math.pi) / dth)
        dth = (2.0 * math.pi) / npr
        ring.append((_r, dth, npr))
        npg_layer += npr
    for _ in range(int(ny)):
        rows.append((lx, ly, lz, r))
        for _r, dth, npr in ring:
            for j in range(npr):
                rows.append((lx + _r * math.cos(dth * j), ly, lz + _r * math.sin(dth * j), r))
    pos = np.array(rows, dtype=np.float64).reshape(-1, 4)
    if min_radius != max_radius:
        pos[:, 3] = min_radius + (max_radius - min_radius) * rng.random(pos.shape[0])
    return Created(pos, [npg_layer] * int(ny))


def circle_count(dia, ny, max_radius) -> int:
    """calculateNumCircleParticles (particleManager.cpp:184-199)."""
    r = float(max_radius)
    cr = 0.5 * dia
    nr = _u(cr / (2.0 * r)) - 1
    rr = 2.0 * r * nr + r
    space = (cr - rr) / (nr + 1)
    cnt = 1
    for i in range(1, nr + 1):
        dth = (2.0 * r + space) / (i * (2.0 * r + space))
        cnt += _u((2.0 * math.pi) / dth)
    return cnt * int(ny)
