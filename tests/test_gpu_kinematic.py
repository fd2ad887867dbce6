"""Kinematic polygon bodies (an extension: the reference moves bodies through
its multibody solver on the host) on the GPU against the oracle's
restatement (closed forms in tests/test_cpu_history.py): a spinning,
translating drum, 8 steps.  FP64 form: the FP64 step tolerances and the body
pose within 1e-13; mixed form: the pose within 1e-13 and the state within
the mixed form's trajectory bands."""
import numpy as np
import pytest

from metakonga_gb300 import engine

from .cases import small_drum
from .test_gpu_step import _state_err

pytestmark = pytest.mark.gpu


def _spinning_drum():
    sc = small_drum()
    sc.pmi["omega"] = (0.0, 20.0, 0.0)
    sc.pmi["vel"] = (0.01, -0.02, 0.005)
    return sc


@pytest.mark.parametrize("mode", [engine.MODE_FP64, engine.MODE_MIXED])
def test_kinematic_drum_matches_oracle(cuda, oracle, mode):
    sc = _spinning_drum()
    ref = sc.copy()
    oracle.run(ref, 8, kinematic=True)
    ds = engine.DeviceScene(sc, mode=mode)
    ds.set_kinematic_bodies(True)
    ds.step(3)
    ds.step(5, check=True)
    got = ds.download()
    pmi = ds.get_bodies()
    ds.close()
    for k in ("ep", "origin"):
        assert np.abs(pmi[k] - ref.pmi[k]).max() <= 1e-13, k
    assert np.abs(ref.pmi["ep"][0] - sc.pmi["ep"][0]).max() > 1e-4, "the drum did not turn"
    if mode == engine.MODE_FP64:
        err = _state_err(got, ref.__dict__, sc.mass)
        assert err["pos"] <= 1e-13 and err["vel"] <= 1e-9 and err["force"] <= 1e-9, err
        # the body reaction of the moving mesh
        scale = np.abs(ref.pmi["force"]).max()
        assert np.abs(pmi["force"] - ref.pmi["force"]).max() <= 1e-9 * scale
    else:
        vs = np.abs(ref.vel).max()
        assert np.abs(got["vel"] - ref.vel).max() <= 1e-4 * vs
        assert np.abs(got["pos"] - ref.pos).max() <= 1e-9
        scale = np.abs(ref.pmi["force"]).max()
        assert np.abs(pmi["force"] - ref.pmi["force"]).max() <= 1e-4 * scale


def test_kinematic_mixed_rebins_as_the_mesh_sweeps(cuda):
    """A fast spin moves the vertices past half the skin: the mixed form
    re-bins during the call, on the device."""
    sc = _spinning_drum()
    sc.pmi["omega"] = (0.0, 400.0, 0.0)
    ds = engine.DeviceScene(sc, mode=engine.MODE_MIXED)
    ds.set_kinematic_bodies(True)
    ds.step(2, check=True)
    r0 = ds.rebuilds()[0]
    ds.step(40, check=True)
    assert ds.rebuilds()[0] > r0
    ds.close()
