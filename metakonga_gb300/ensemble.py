"""Ensemble statistics of a granular state.

Granular trajectories are chaotic: two runs whose forces differ by rounding
separate after a few thousand steps, so long runs of two precision forms are
compared through statistics of the state rather than particle by particle.
The long-run comparisons use these three:

* kinetic energy (translational + rotational) -- sampled over a run it gives
  the decay curve of a settling bed;
* packing fraction -- solid volume of the spheres whose centres lie in a box,
  over the box's volume (a box inside the bed, away from walls and the free
  surface, measures the bed's density);
* mean coordination number -- particle-particle contacts per particle, from a
  pair list (each contact counted for both partners).

All functions take host arrays in the reference's layouts (pos (N, 4) with
the radius in column 3, vel/omega (N, 3), mass/inertia (N,)).
"""
from __future__ import annotations

import math

import numpy as np


def kinetic_energy(vel, omega, mass, inertia) -> float:
    """sum_i m_i |v_i|^2 / 2 + I_i |w_i|^2 / 2 (J)."""
    vel = np.asarray(vel, np.float64)
    omega = np.asarray(omega, np.float64)
    return float(0.5 * (np.asarray(mass) * (vel * vel).sum(axis=1)).sum()
                 + 0.5 * (np.asarray(inertia) * (omega * omega).sum(axis=1)).sum())


def packing_fraction(pos, lo, hi) -> float:
    """Volume of the spheres whose centres lie in the box [lo, hi) over the
    box's volume (the sphere counted whole: a box much larger than a sphere
    keeps the edge error small)."""
    pos = np.asarray(pos, np.float64)
    lo = np.asarray(lo, np.float64)
    hi = np.asarray(hi, np.float64)
    inside = np.all((pos[:, :3] >= lo) & (pos[:, :3] < hi), axis=1)
    vol = (4.0 / 3.0) * math.pi * np.power(pos[inside, 3], 3.0).sum()
    return float(vol / np.prod(hi - lo))


def bed_box(pos, walls_lo, walls_hi, margin_radii: float = 3.0, top_quantile: float = 0.9):
    """An interior box of a settled bed in an axis-aligned container: the
    container's floor and sides moved in by ``margin_radii`` largest radii, the
    top at the ``top_quantile`` height of the centres less the same margin."""
    pos = np.asarray(pos, np.float64)
    m = margin_radii * float(pos[:, 3].max())
    lo = np.asarray(walls_lo, np.float64) + m
    hi = np.asarray(walls_hi, np.float64) - m
    hi[2] = float(np.quantile(pos[:, 2], top_quantile)) - m
    return lo, hi


def coordination(pairs, n: int) -> float:
    """Mean particle-particle contacts per particle from a pair list of
    (i, j) rows, each unordered contact listed once or from both sides."""
    pairs = np.asarray(pairs)
    if pairs.size == 0 or n == 0:
        return 0.0
    a = np.minimum(pairs[:, 0], pairs[:, 1]).astype(np.int64)
    b = np.maximum(pairs[:, 0], pairs[:, 1]).astype(np.int64)
    uniq = np.unique(a * (int(n) + 1) + b)
    return 2.0 * uniq.size / n


def log_band(a, b, floor: float) -> float:
    """max |log10(a) - log10(b)| over the samples where either exceeds floor
    (samples below it are at the noise level of a bed at rest)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    keep = np.maximum(a, b) > floor
    if not keep.any():
        return 0.0
    return float(np.abs(np.log10(np.maximum(a[keep], floor)) - np.log10(np.maximum(b[keep], floor))).max())
