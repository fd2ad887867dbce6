"""A particle cloud around one tilted, moving cylinder (device_cylinder_info),
for the cylinder contact tests: particles sampled along the axis past both
ends and out to the radius plus 1.2 r, so that lateral, end-cap and rim
contacts all occur (particle_cylinder_contact_detection, impl:652-719)."""
import math

import numpy as np

from metakonga_gb300.layouts import CONTACT_PROPERTY, CYLINDER, make_params, make_contact_property


def frame(ep):
    """Rows A1..A3 of the Euler-parameter matrix (makeTFM_1..3, impl:624-637)."""
    x, y, z, w = ep
    return np.array([[2 * (x * x + y * y - 0.5), 2 * (y * z - x * w), 2 * (y * w + x * z)],
                     [2 * (y * z + x * w), 2 * (x * x + z * z - 0.5), 2 * (z * w - x * y)],
                     [2 * (y * w - x * z), 2 * (z * w + x * y), 2 * (x * x + w * w - 0.5)]])


def cylinder(origin=(0.1, 0.2, -0.05), length=0.2, radius=0.05, angle=0.3, axis=(1.0, 0.0, 1.0),
             vel=(0.1, 0.0, 0.0), omega=(0.0, 1.0, 0.5)):
    a = np.asarray(axis) / np.linalg.norm(axis)
    ep = np.concatenate([[math.cos(angle / 2)], math.sin(angle / 2) * a])
    A = frame(ep)
    ax = A[:, 1]                      # the local y axis in world coordinates
    c = np.zeros(1, CYLINDER)
    c["len"], c["rbase"], c["rtop"] = length, radius, radius
    c["origin"] = origin
    c["pbase"] = np.asarray(origin) - 0.5 * length * ax
    c["ptop"] = np.asarray(origin) + 0.5 * length * ax
    c["vel"], c["omega"], c["ep"] = vel, omega, ep
    return c, A


def cloud(n=6000, seed=11):
    cyl, A = cylinder()
    rng = np.random.Generator(np.random.MT19937(seed))
    r = rng.uniform(0.002, 0.004, n)
    t = rng.uniform(-0.03, 1.03, n)
    rho = rng.uniform(0.0, 0.05 + 1.2 * r)
    th = rng.uniform(0.0, 2 * math.pi, n)
    base, top = cyl["pbase"][0], cyl["ptop"][0]
    p = base + t[:, None] * (top - base) + rho[:, None] * (np.cos(th)[:, None] * A[:, 0] +
                                                           np.sin(th)[:, None] * A[:, 2])
    pos = np.concatenate([p, r[:, None]], axis=1)
    vel = rng.normal(0.0, 0.1, (n, 3))
    omega = rng.normal(0.0, 10.0, (n, 3))
    mass = 2500.0 * 4.0 / 3.0 * math.pi * r ** 3
    cp = np.array([make_contact_property(E_i=1e7, E_j=2e11, nu_i=0.3, nu_j=0.3, rest=0.6, fric=0.4, sratio=0.8)],
                  dtype=CONTACT_PROPERTY)
    prm = make_params(np_=n, ncell=8, grid=(2, 2, 2), dt=1e-5, cell_size=0.1, world_origin=(-1, -1, -1),
                      gravity=(0, -9.81, 0))
    mpos = np.array([0.1, 0.15, -0.05])
    return dict(cyl=cyl, pos=pos, vel=vel, omega=omega, mass=mass, cp=cp, prm=prm, mpos=mpos)
