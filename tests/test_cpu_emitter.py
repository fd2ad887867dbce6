"""Particle emitter in the oracle (xdo_emitter, the reference's real-time
creation: dem_simulation.cpp:210-222, :321-322, :449-450 and
particleManager.cpp:132-145): the schedule, free fall of an emitted particle
in closed form, and staged particles left alone."""
import numpy as np

from metakonga_gb300 import scenes
from oracle.pyoracle import Emitter

from .cases import emitter_column


def _sequence(oracle, sc, em, steps):
    out = []
    for _ in range(steps):
        oracle.run(sc, 1, emitter=em)
        out.append(em.active)
    return out


def test_emitter_schedule_groups(oracle):
    sc = emitter_column(n=10)
    em = Emitter(period=3, groups=[2, 5, 1])
    # creations before steps 1, 4, 7; the groups are used up after that
    assert _sequence(oracle, sc, em, 11) == [2, 2, 2, 7, 7, 7, 8, 8, 8, 8, 8]


def test_emitter_schedule_one_by_one_and_clamp(oracle):
    sc = emitter_column(n=4)
    em = Emitter(period=2)
    assert _sequence(oracle, sc, em, 10) == [1, 1, 2, 2, 3, 3, 4, 4, 4, 4]
    sc = emitter_column(n=5)
    em = Emitter(period=1, groups=[3, 3, 3])
    assert _sequence(oracle, sc, em, 3) == [3, 5, 5]


def test_emitted_particle_falls_from_rest_and_staged_ones_stay(oracle):
    """A particle emitted before step k has, m steps later (its own steps),
    x = x0 + g dt^2 m (m - 1) / 2 and v = g dt (m - 1/2): velocity-Verlet
    from rest with a = 0 at the start and F = m g (the upload's force).  The
    staged particles keep their uploaded state bit for bit."""
    sc = emitter_column(n=6)
    ref0 = sc.copy()
    em = Emitter(period=4, groups=[1, 1, 1, 1, 1, 1])
    steps = 13
    oracle.run(sc, steps, emitter=em)
    assert em.active == 4
    g = np.asarray(scenes.GRAVITY)
    dt = sc.dt
    for i in range(em.active):
        m = steps - 4 * i            # particle i joins before step 4 i + 1
        x = ref0.pos[i, :3] + g * dt * dt * m * (m - 1) / 2.0
        v = g * dt * (m - 0.5)
        assert np.allclose(sc.pos[i, :3], x, rtol=0, atol=1e-15), i
        assert np.allclose(sc.vel[i], v, rtol=1e-12, atol=0), i
    for k in ("pos", "vel", "acc", "omega", "force", "moment"):
        assert np.array_equal(getattr(sc, k)[em.active:], getattr(ref0, k)[em.active:]), k


def test_staged_particles_do_not_touch(oracle):
    """An active particle overlapping a staged one feels nothing."""
    sc = emitter_column(n=3)
    sc.pos[1, :3] = sc.pos[0, :3] + (1.5 * sc.pos[0, 3], 0.0, 0.0)   # overlaps particle 0
    ref = sc.copy()
    em = Emitter(period=100, groups=[1, 1, 1])
    oracle.run(sc, 3, emitter=em)
    free = emitter_column(n=1)
    free.pos[0] = ref.pos[0]
    oracle.run(free, 3)
    assert np.array_equal(sc.pos[0], free.pos[0]) and np.array_equal(sc.vel[0], free.vel[0])
    assert np.array_equal(sc.pos[1:], ref.pos[1:])
