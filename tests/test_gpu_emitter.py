"""Particle emitter on the GPU (xd_scene_set_emitter) against the oracle's
restatement (xdo_emitter; closed forms in tests/test_cpu_emitter.py).

The scene is the plane emitter of tests/cases.EMITTER_MODEL read by the model
loader, its six layers restacked 7.9 mm apart above the floor (touching each
other and the floor) and emitted one layer every 8 steps, so that 60 steps
cover every emission, staged particles next to active ones, contacts between
layers that joined at different steps, and calls that end between
emissions.  FP64 form: the FP64 step tolerances; mixed form: its trajectory
bands.  Staged particles come back exactly as uploaded."""
import numpy as np
import pytest

from metakonga_gb300 import engine
from oracle.pyoracle import Emitter, History

from .cases import emitter_box
from .test_gpu_step import _state_err

pytestmark = pytest.mark.gpu


def _stacked(layers=6, period=8):
    sc, em = emitter_box(layers=layers, drop_speed=0.5)
    per = em["groups"][0]
    for k in range(layers):
        sc.pos[k * per:(k + 1) * per, 1] = 0.0039 + 0.0079 * k
    return sc, dict(em, period=period)


def _check(mode, got, ref, sc, staged_from=None):
    if mode == engine.MODE_FP64:
        err = _state_err(got, ref.__dict__, sc.mass)
        assert err["pos"] <= 1e-13 and err["vel"] <= 1e-9 and err["force"] <= 1e-9, err
    else:
        vs = np.abs(ref.vel).max()
        assert np.abs(got["vel"] - ref.vel).max() <= 1e-4 * vs
        assert np.abs(got["pos"] - ref.pos).max() <= 1e-9
    if staged_from is not None:
        for k in ("pos", "vel", "omega"):
            assert np.array_equal(got[k][staged_from:], getattr(sc, k)[staged_from:]), k


@pytest.mark.parametrize("mode", [engine.MODE_FP64, engine.MODE_MIXED])
def test_emitter_matches_oracle(cuda, oracle, mode):
    sc, em = _stacked()
    ref = sc.copy()
    e = Emitter(em["period"], em["groups"], em["active"])
    oracle.run(ref, 36, emitter=e)
    ds = engine.DeviceScene(sc, mode=mode)
    ds.set_emitter(em["period"], em["groups"], em["active"])
    assert ds.active() == 0
    for k in (7, 13, 16):          # calls that end between emissions
        ds.step(k, check=True)
    assert ds.active() == e.active == 5 * em["groups"][0]
    got = ds.download()
    _check(mode, got, ref, sc, staged_from=e.active)
    # the rest: the last emission, then a call long enough for the graphs
    oracle.run(ref, 44, emitter=e)
    ds.step(44, check=True)
    assert ds.active() == e.active == sc.np_
    got = ds.download()
    ds.close()
    _check(mode, got, ref, sc)


@pytest.mark.parametrize("mode", [engine.MODE_FP64, engine.MODE_MIXED])
def test_emitter_same_alone_and_in_a_batch(cuda, mode):
    """A scene with an emitter gives the same bits stepped alone and side by
    side with others (engine.step_many), in any split of its steps."""
    outs = []
    for split, batch in (((40,), False), ((9, 31), True)):
        sc, em = _stacked()
        ds = engine.DeviceScene(sc, mode=mode)
        ds.set_emitter(em["period"], em["groups"], em["active"])
        others = [engine.DeviceScene(_stacked()[0], mode=mode) for _ in range(2)] if batch else []
        for k in split:
            if batch:
                engine.step_many([ds] + others, [k] * 3, check=True)
            else:
                ds.step(k, check=True)
        outs.append(ds.download())
        for d in [ds] + others:
            d.close()
    for k in ("pos", "vel", "omega"):
        assert np.array_equal(outs[0][k], outs[1][k]), k


def test_emitter_set_after_steps_with_history(cuda, oracle):
    """Setting an emitter on a mixed scene that has re-binned puts its
    particles back in id order, springs included: stepping on equals the
    oracle's uninterrupted run."""
    sc, _ = _stacked()
    ref = sc.copy()
    h = History(sc.np_, 12)
    oracle.run(ref, 40, history=h)
    ds = engine.DeviceScene(sc, mode=engine.MODE_MIXED)
    ds.set_tangential_history(12)
    ds.step(20, check=True)
    ds.set_emitter(0, None, active=sc.np_)      # every particle, no creation
    ds.step(20, check=True)
    got = ds.download()
    ds.close()
    _check(engine.MODE_MIXED, got, ref, sc)
