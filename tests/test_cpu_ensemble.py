"""The ensemble statistics (metakonga_gb300.ensemble) on states with known answers."""
import math

import numpy as np

from metakonga_gb300 import ensemble


def test_kinetic_energy_closed_form():
    vel = np.array([[1.0, 0.0, 0.0], [0.0, 2.0, 0.0]])
    omega = np.array([[0.0, 0.0, 3.0], [0.0, 0.0, 0.0]])
    mass = np.array([2.0, 0.5])
    inertia = np.array([0.1, 0.2])
    # 1/2 2 1 + 1/2 0.5 4 + 1/2 0.1 9
    assert math.isclose(ensemble.kinetic_energy(vel, omega, mass, inertia), 1.0 + 1.0 + 0.45)


def test_packing_fraction_of_touching_simple_cubic_lattice():
    r, k = 0.005, 20
    g = (np.arange(k) + 0.5) * 2 * r
    x, y, z = np.meshgrid(g, g, g, indexing="ij")
    pos = np.stack([x.ravel(), y.ravel(), z.ravel(), np.full(k ** 3, r)], axis=1)
    # a box of whole lattice cells: pi / 6
    phi = ensemble.packing_fraction(pos, (0.0, 0.0, 0.0), (2 * r * k,) * 3)
    assert math.isclose(phi, math.pi / 6, rel_tol=1e-12)
    lo, hi = ensemble.bed_box(pos, (0, 0, 0), (2 * r * k,) * 3, margin_radii=4.0, top_quantile=1.0)
    assert np.all(lo > 0) and hi[2] < g.max()


def test_coordination_counts_each_contact_once():
    # a chain 0-1-2-3 listed from both sides, with a repeat
    pairs = np.array([[0, 1], [1, 0], [1, 2], [2, 1], [2, 3], [3, 2], [0, 1]])
    assert ensemble.coordination(pairs, 4) == 2 * 3 / 4
    assert ensemble.coordination(np.zeros((0, 2)), 4) == 0.0


def test_log_band_ignores_samples_below_the_floor():
    a = np.array([10.0, 1.0, 1e-9])
    b = np.array([12.0, 0.5, 1e-12])
    assert math.isclose(ensemble.log_band(a, b, floor=1e-6), math.log10(2.0))
