"""The FP64 form with a grid of its own for the particles
(xd_scene_set_particle_grid): particle pairs searched in cells of the
particles' size, triangles on the scene's grid of circumsphere-sized cells.
Each step from the oracle's own state (the reference's single grid): the
per-particle force within 1e-12 of max(|F|, m g) (the pair sums run in another
order) and the position update bit-exact, on a hopper bed whose cone
triangles make the scene's cells three times the particles' size."""
import numpy as np
import pytest

from metakonga_gb300 import engine, prepare, scenes
from metakonga_gb300._lib import XdemError

from .conftest import force_error

pytestmark = pytest.mark.gpu
FP64_TOL = 1e-12


def test_particle_grid_equals_oracle_every_step(cuda, oracle):
    sc = scenes.hopper(n=6000, seed=12, gate=True)
    prepare.settle(sc, 3000, dt=4e-5)
    prepare.open_gates(sc)
    ds = engine.DeviceScene(sc, mode=engine.MODE_FP64)
    grid, cell, origin = ds.set_particle_grid()
    assert cell < 0.5 * float(sc.params["cell_size"])      # the particles' cells are much smaller
    ref = sc.copy()
    worst = 0.0
    touching = 0
    for _ in range(10):
        ds.upload(ref)
        ds.step(1, check=True)
        got = ds.download()
        oracle.run(ref, 1)
        f_got, f_ref = got["acc"] * sc.mass[:, None], ref.acc * sc.mass[:, None]
        worst = max(worst, force_error(f_got, f_ref, sc.mass))
        contact = np.linalg.norm(f_ref - sc.mass[:, None] * np.array(scenes.GRAVITY), axis=1)
        touching = max(touching, int((contact > 1e-3 * sc.mass * 9.81).sum()))
        assert np.array_equal(got["pos"], ref.pos)
    ds.close()
    assert touching > 4000, touching
    assert worst <= FP64_TOL, worst


def test_particle_grid_checks(cuda):
    sc = scenes.settle_box(n_side=4)
    d = engine.DeviceScene(sc, mode=engine.MODE_FP64)
    with pytest.raises(XdemError):
        d.set_particle_grid([12, 16, 16], 0.01, [0.0, 0.0, 0.0])     # not a power of two
    d.close()
    m = engine.DeviceScene(sc, mode=engine.MODE_MIXED)
    with pytest.raises(XdemError):
        m.set_particle_grid([16, 16, 16], 0.01, [0.0, 0.0, 0.0])     # FP64 scenes only
    m.close()
