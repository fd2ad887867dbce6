"""Tangential-spring history on the GPU against the oracle's restatement
(tests/test_cpu_history.py pins the oracle to closed forms).

FP64 form: the same steps as the oracle with history on; states within the
FP64 form's step tolerances (pos 1e-13, vel 1e-9 relative), the contact
tables equal (same keys in the same entries) and the springs within 1e-9 of
their scale."""
import numpy as np
import pytest

from metakonga_gb300 import engine
from oracle.pyoracle import HIST_EMPTY, History

from .cases import packed_scene, small_drum
from .test_gpu_step import _state_err

pytestmark = pytest.mark.gpu
SLOTS = 16


def _squeezed_drum():
    sc = small_drum()
    return sc


@pytest.mark.parametrize("case", ["packed", "drum"])
def test_fp64_history_steps_match_oracle(cuda, oracle, case):
    sc = packed_scene(n_side=8) if case == "packed" else _squeezed_drum()
    ref = sc.copy()
    hist = History(ref.np_, SLOTS)
    oracle.run(ref, 8, history=hist)
    ds = engine.DeviceScene(sc)
    ds.set_tangential_history(SLOTS)
    ds.step(3)
    ds.step(5, check=True)
    got = ds.download()
    keys, delta, overflow = ds.download_history()
    ds.close()
    err = _state_err(got, ref.__dict__, sc.mass)
    assert err["pos"] <= 1e-13 and err["vel"] <= 1e-9 and err["force"] <= 1e-9, err
    assert overflow == 0 and hist.overflow == 0
    assert np.array_equal(keys, hist.key)
    live = hist.key != HIST_EMPTY
    assert live.sum() > 50, "case has too few lasting contacts"
    scale = np.abs(hist.delta[live]).max()
    assert np.abs(delta - hist.delta).max() <= 1e-9 * scale


def test_fp64_history_off_is_the_reference_model(cuda, oracle):
    sc = packed_scene(n_side=6)
    a = engine.DeviceScene(sc)
    b = engine.DeviceScene(sc)
    b.set_tangential_history(SLOTS)
    b.set_tangential_history(0)
    a.step(4, check=True)
    b.step(4, check=True)
    ga, gb = a.download(), b.download()
    a.close()
    b.close()
    for k in ("pos", "vel", "omega"):
        assert np.array_equal(ga[k], gb[k]), k
