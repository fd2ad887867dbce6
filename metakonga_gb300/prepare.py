"""Settled initial states: a bed poured and settled before the timed run.

A hopper-discharge or settle benchmark starts from a packed bed, but the
synthetic scenes start as loose lattices (no overlaps): at the configured
time step (5e-6 s) the lattice takes 0.15-0.3 s of simulated time (30,000-
60,000 steps) to fall together.  ``settle`` runs that preparation in the
mixed form at a coarser time step -- the velocity-Verlet update is stable
while a step stays well below the Hertz contact time of the smallest sphere
pair (about 7e-4 s for 2 mm spheres of E = 1e7 Pa at 0.1 m/s, so 4e-5 s gives
some 17 steps per contact) -- and writes the settled state (positions,
velocities, accelerations, spins) back into the scenes, whose own time step
is untouched.  The preparation is initial-condition generation, like the
lattice itself: the runs that are measured or compared use the scenes'
configured constants from the settled state on.

Gated hoppers (``scenes.hopper(gate=True)``) settle with the orifice closed;
``open_gates`` then removes the gate for the discharge.
"""
from __future__ import annotations

import numpy as np

from . import engine, scenes as _scenes


def _with_dt(sc, dt: float):
    s = sc.copy()
    s.params["dt"] = dt
    s.params["half2dt"] = 0.5 * dt * dt
    s.dt = dt
    return s


def settle(scs, steps: int, dt: float = 4e-5, stream: int = 0, batch: bool = True) -> list:
    """Advance each scene of ``scs`` (a Scene or a list of them) by ``steps``
    steps of ``dt`` in the mixed form (one batch) and store the reached state
    in the scene objects.  Returns the scenes."""
    single = not isinstance(scs, (list, tuple))
    scs = [scs] if single else list(scs)
    prep = [_with_dt(sc, dt) for sc in scs]
    ds = [engine.DeviceScene(p, mode=engine.MODE_MIXED) for p in prep]
    try:
        if batch and len(ds) > 1:
            b = engine.Batch(ds)
            try:
                b.step(steps, check=True, stream=stream)
            finally:
                b.close()
        else:
            for d in ds:
                d.step(steps, check=True, stream=stream)
        for sc, d in zip(scs, ds):
            st = d.download(stream)
            for k in ("pos", "vel", "acc", "omega", "alpha"):
                getattr(sc, k)[:] = st[k]
            # the step's contact force is recomputed from the state by the
            # first step of the next run; gravity alone is the reference's
            # starting value (dem_simulation.cpp:232-251)
            sc.force[:] = sc.mass[:, None] * np.asarray(sc.params["gravity"])[None, :]
            sc.moment[:] = 0.0
            if sc.ntri:
                sc.pmi[:] = d.get_bodies(stream)
                sc.pmi["force"] = 0.0
                sc.pmi["moment"] = 0.0
    finally:
        for d in ds:
            d.close()
    return scs[0] if single else scs


def open_gates(scs) -> None:
    """Gated hoppers: the gate moved out of the way (orifice open), in place."""
    for sc in (scs if isinstance(scs, (list, tuple)) else [scs]):
        if "gate" in sc.plane_names:
            sc.planes = _scenes.open_gate(sc)
