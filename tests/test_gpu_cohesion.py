"""Cohesion (cohesionForce, mphysics_cuda_impl.cuh:259-279) in both forms.

The particle-pair DHS force adds coh pi rc^2, rc^3 = 3 Req (-fsn) Eeq / 4
(impl:386).  The reference's polygon kernel passes a cohesion of zero
(impl:1000) and its plane kernel passes the property's cohesion with zero radii
and moduli (impl:613), which makes the plane force NaN when it is set: polygon
cohesion is accepted and has no effect, plane cohesion is refused by the mixed
form.  Cohesion 1e6 Pa halves the largest contact force of the packed lattice,
so the elastic, cohesive and damping terms cancel in many contacts."""
import numpy as np
import pytest

from metakonga_gb300 import engine

from .cases import packed_scene, small_hopper
from .test_gpu_mixed import FORCE_TOL, _norm_err, _oracle_view, _pairset
from .test_gpu_step import _state_err

pytestmark = pytest.mark.gpu


def _cohesive(coh, n_side=10):
    sc = packed_scene(n_side=n_side)      # walls keep the property without cohesion
    sc.cp_pp["coh"] = coh
    return sc


@pytest.mark.parametrize("coh", [1e5, 1e6])
def test_mixed_cohesion_pairs_and_forces(cuda, oracle, coh):
    sc = _cohesive(coh, n_side=12)
    ds = engine.DeviceScene(sc, mode=engine.MODE_MIXED)
    ds.step(2)
    st = ds.download()
    pairs_ref, f_ref, m_ref, mag = _oracle_view(oracle, sc, st)
    assert _pairset(ds.pair_list(cap=48)) == _pairset(pairs_ref)
    f, m = ds.eval_contacts()
    ds.close()
    r = sc.pos[:, 3:4]
    assert _norm_err(f, f_ref, mag, sc.mass) <= FORCE_TOL
    assert _norm_err(m / r, m_ref / r, mag, sc.mass) <= FORCE_TOL


def test_fp64_cohesion_matches_oracle(cuda, oracle):
    sc = _cohesive(1e6)
    ref = sc.copy()
    oracle.run(ref, 20)
    ds = engine.DeviceScene(sc, mode=engine.MODE_FP64)
    ds.step(20)
    got = ds.download()
    ds.close()
    err = _state_err(got, ref.__dict__, sc.mass)
    assert err["pos"] <= 1e-13 and err["vel"] <= 1e-9 and err["force"] <= 1e-9, err


def test_mixed_cohesion_tracks_fp64(cuda):
    sc = _cohesive(1e6)
    a = engine.DeviceScene(sc, mode=engine.MODE_FP64)
    b = engine.DeviceScene(sc, mode=engine.MODE_MIXED)
    a.step(20)
    b.step(20)
    sa, sb = a.download(), b.download()
    a.close()
    b.close()
    assert np.abs(sa["pos"] - sb["pos"]).max() < 1e-9
    assert np.abs(sa["vel"] - sb["vel"]).max() < 1e-4 * np.abs(sa["vel"]).max()


def test_polygon_cohesion_has_no_effect(cuda):
    outs = []
    for coh in (0.0, 1e6):
        sc = small_hopper()
        sc.cp_poly["coh"] = coh
        ds = engine.DeviceScene(sc, mode=engine.MODE_MIXED)
        ds.step(30)
        outs.append(ds.download())
        ds.close()
    for k in ("pos", "vel", "omega"):
        assert np.array_equal(outs[0][k], outs[1][k]), k


def test_mixed_refuses_plane_cohesion(cuda):
    sc = _cohesive(0.0, n_side=6)
    sc.cp_planes["coh"] = 1e5
    with pytest.raises(Exception, match="plane cohesion"):
        engine.DeviceScene(sc, mode=engine.MODE_MIXED)
