"""Moving walls (xd_scene_set_planes, the reference's re-upload of a moving
plane's device_plane_info, collision/contact_particles_plane.cpp:33-51): the
floor of a packed box pushed up between calls, in both forms, against the
oracle given the same planes between the same steps."""
import numpy as np
import pytest

from metakonga_gb300 import engine

from .cases import packed_scene
from .test_gpu_step import _state_err

pytestmark = pytest.mark.gpu


def _raised(planes, names, dz):
    out = planes.copy()
    k = names.index("wall_floor")
    for f in ("xw", "w2", "w3", "w4"):
        out[k][f][2] += dz
    return out


@pytest.mark.parametrize("mode", [engine.MODE_FP64, engine.MODE_MIXED])
def test_floor_pushed_up_between_calls(cuda, oracle, mode):
    sc = packed_scene(n_side=8)
    ref = sc.copy()
    still = sc.copy()
    oracle.run(still, 16)
    ds = engine.DeviceScene(sc, mode=mode)
    planes = sc.planes.copy()
    for k in range(3):
        oracle.run(ref, 4)
        ds.step(4, check=True)
        planes = _raised(planes, sc.plane_names, 1e-4)
        ref.planes[:] = planes
        ds.set_planes(planes)
    oracle.run(ref, 4)
    ds.step(4, check=True)
    got = ds.download()
    ds.close()
    # the raised floor changed the motion (against the walls left in place)
    assert np.abs(ref.vel - still.vel).max() > 1e-3 * np.abs(still.vel).max()
    if mode == engine.MODE_FP64:
        err = _state_err(got, ref.__dict__, sc.mass)
        assert err["pos"] <= 1e-13 and err["vel"] <= 1e-9 and err["force"] <= 1e-9, err
    else:
        vs = np.abs(ref.vel).max()
        assert np.abs(got["vel"] - ref.vel).max() <= 1e-4 * vs
        assert np.abs(got["pos"] - ref.pos).max() <= 1e-9


def test_set_planes_checks_the_count(cuda):
    sc = packed_scene(n_side=4)
    ds = engine.DeviceScene(sc, mode=engine.MODE_MIXED)
    with pytest.raises(ValueError):
        ds.set_planes(sc.planes[:2])
    ds.close()
