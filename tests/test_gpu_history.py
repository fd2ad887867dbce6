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


def _pairs_by_id(keys, delta):
    """{(i, key): spring} of a table in original order."""
    out = {}
    s_idx, i_idx = np.nonzero(keys != HIST_EMPTY)
    for s, i in zip(s_idx, i_idx):
        out[(int(i), int(keys[s, i]))] = delta[s, i]
    return out


@pytest.mark.parametrize("case", ["packed", "drum"])
def test_mixed_history_matches_oracle(cuda, oracle, case):
    """The mixed form with springs: the same contacts hold springs as in the
    oracle (keys per particle as sets: the mixed form visits contacts in its
    own order), the springs within 2e-5 of the largest spring, and the state
    close to the oracle's over 8 steps."""
    sc = packed_scene(n_side=8) if case == "packed" else small_drum()
    ref = sc.copy()
    hist = History(ref.np_, SLOTS)
    oracle.run(ref, 8, history=hist)
    ds = engine.DeviceScene(sc, mode=engine.MODE_MIXED)
    ds.set_tangential_history(SLOTS)
    ds.step(3)
    ds.step(5, check=True)
    got = ds.download()
    keys, delta, overflow = ds.download_history()
    ds.close()
    assert overflow == 0
    a, b = _pairs_by_id(keys, delta), _pairs_by_id(hist.key, hist.delta)
    assert set(a) == set(b)
    assert len(b) > 50
    scale = max(np.abs(v).max() for v in b.values())
    assert max(np.abs(a[k] - b[k]).max() for k in b) <= 2e-5 * scale
    vs = np.abs(ref.vel).max()
    assert np.abs(got["vel"] - ref.vel).max() <= 1e-4 * vs
    assert np.abs(got["pos"] - ref.pos).max() <= 1e-9


def test_mixed_history_forces_match_oracle(cuda, oracle):
    """Contact forces with springs (read-only evaluation) against the oracle's
    next-step forces on the same state and tables, 2e-5 of max(sum |F_c|, m g)."""
    from metakonga_gb300.scenes import GRAVITY
    from .test_gpu_mixed import FORCE_TOL, _norm_err
    sc = packed_scene(n_side=8)
    ds = engine.DeviceScene(sc, mode=engine.MODE_MIXED)
    ds.set_tangential_history(SLOTS)
    ds.step(6, check=True)
    st = ds.download()
    keys, delta, _ = ds.download_history()
    f, m = ds.eval_contacts()
    ds.close()
    # the oracle evaluates the same state with the same tables
    p = sc.params.copy()
    p["np"] = sc.np_
    pos = np.ascontiguousarray(st["pos"])
    vel = np.ascontiguousarray(st["vel"])
    om = np.ascontiguousarray(st["omega"])
    h, ix, cs, ce, so = oracle.detection(p, pos)
    H = History(sc.np_, SLOTS)
    H.key[:] = keys
    H.delta[:] = delta
    fr = np.zeros((sc.np_, 3))
    mr = np.zeros((sc.np_, 3))
    oracle.hist_p2p(p, pos, vel, om, fr, mr, sc.mass, so, cs, ce, sc.cp_pp, H)
    oracle.hist_planes(p, sc.planes, sc.cp_planes, pos, vel, om, fr, mr, sc.mass, H)
    mag = oracle.contact_magnitudes(p, pos, vel, om, sc.mass, so, cs, ce, sc.cp_pp, sc.planes,
                                    sc.cp_planes)
    assert np.abs(fr).max() > 0
    assert _norm_err(f, fr, mag, sc.mass) <= FORCE_TOL
    r = sc.pos[:, 3:4]
    assert _norm_err(m / r, mr / r, mag, sc.mass) <= FORCE_TOL
