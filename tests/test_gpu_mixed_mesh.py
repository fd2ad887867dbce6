"""Triangle meshes in the mixed form against the FP64 oracle.

The drum case presses spheres against a coarse cylinder mesh (face, edge and
vertex contacts); the hopper case presses them against a 4,096-triangle cone
above a plane floor.  Gates: particle pair lists equal the oracle's; per-particle
contact force (pairs + triangles) within 2e-5 of max(sum_c |F_c|, m g), the sum
over every contact of the particle, triangles included; the reaction on the
polygon body after one step within 1e-6 of its scale (the mixed form's
triangle forces are FP32, each within about 1e-7 of the FP64 force; the
reaction is their sum); a mesh moved by xd_scene_set_bodies is seen at its
new pose."""
import numpy as np
import pytest

from metakonga_gb300 import engine
from metakonga_gb300.scenes import euler_parameters_about_y

from .cases import small_drum, small_hopper
from .test_gpu_mixed import FORCE_TOL, _norm_err, _pairset

pytestmark = pytest.mark.gpu


def _oracle_mesh_view(oracle, sc, st, poly=None, sphere=None):
    p = sc.params.copy()
    p["np"] = sc.np_
    poly = sc.poly if poly is None else poly
    sphere = sc.sphere if sphere is None else sphere
    pos = np.ascontiguousarray(st["pos"])
    vel = np.ascontiguousarray(st["vel"])
    om = np.ascontiguousarray(st["omega"])
    h, ix, cs, ce, so = oracle.detection(p, pos, sphere)
    pairs = oracle.pair_list(p, pos, so, cs, ce)
    f = np.zeros((sc.np_, 3))
    m = np.zeros((sc.np_, 3))
    oracle.p2p(p, pos, vel, om, f, m, sc.mass, so, cs, ce, sc.cp_pp)
    for i in range(sc.planes.shape[0]):
        oracle.plane(p, sc.planes[i:i + 1], pos, vel, om, f, m, sc.mass, sc.cp_planes[i:i + 1])
    pmi = sc.pmi.copy()
    pmi["force"] = 0
    pmi["moment"] = 0
    ft = np.zeros((sc.np_, 3))
    mt = np.zeros((sc.np_, 3))
    oracle.polygon(p, poly, sphere, pmi, pos, vel, om, ft, mt, sc.mass, so, cs, ce, sc.cp_poly)
    # sum_c |F_c| over pair and plane contacts, plus the magnitude of the
    # triangle force (at most the sum of the triangle contacts' magnitudes)
    mag = oracle.contact_magnitudes(p, pos, vel, om, sc.mass, so, cs, ce, sc.cp_pp, sc.planes,
                                    sc.cp_planes) + np.linalg.norm(ft, axis=1)
    return pairs, f + ft, m + mt, mag, pmi


def test_mixed_drum_pairs_and_forces(cuda, oracle):
    sc = small_drum()
    ds = engine.DeviceScene(sc, mode=engine.MODE_MIXED)
    ds.step(2)
    st = ds.download()
    pairs_ref, f_ref, m_ref, mag, _ = _oracle_mesh_view(oracle, sc, st)
    # the case must exercise the mesh: compare against forces without triangles
    assert np.abs(f_ref).max() > 0
    pairs = ds.pair_list(cap=48)
    f, m = ds.eval_contacts()
    ds.close()
    assert _pairset(pairs) == _pairset(pairs_ref)
    assert _norm_err(f, f_ref, mag, sc.mass) <= FORCE_TOL
    r = sc.pos[:, 3:4]
    assert _norm_err(m / r, m_ref / r, mag, sc.mass) <= FORCE_TOL


def test_mixed_hopper_pairs_and_forces(cuda, oracle):
    sc = small_hopper()
    ds = engine.DeviceScene(sc, mode=engine.MODE_MIXED)
    ds.step(2)
    st = ds.download()
    pairs_ref, f_ref, m_ref, mag, pmi = _oracle_mesh_view(oracle, sc, st)
    # the case must exercise the cone: the body takes a reaction
    assert np.abs(pmi["force"]).max() > 0
    pairs = ds.pair_list(cap=48)
    f, m = ds.eval_contacts()
    ds.close()
    assert _pairset(pairs) == _pairset(pairs_ref)
    assert _norm_err(f, f_ref, mag, sc.mass) <= FORCE_TOL
    r = sc.pos[:, 3:4]
    assert _norm_err(m / r, m_ref / r, mag, sc.mass) <= FORCE_TOL


def test_mixed_drum_body_reaction_one_step(cuda, oracle):
    """One step from the uploaded state: the reaction added to the body equals
    the oracle step's within 1e-6 of its scale (FP32 triangle forces summed)."""
    sc = small_drum()
    sc.pmi["force"] = 0
    sc.pmi["moment"] = 0
    ds = engine.DeviceScene(sc, mode=engine.MODE_MIXED)
    ds.step(1)
    got = ds.get_bodies()
    ds.close()
    ref = small_drum()
    ref.pmi["force"] = 0
    ref.pmi["moment"] = 0
    oracle.run(ref, 1)
    fs = np.abs(ref.pmi["force"]).max()
    ms = np.abs(ref.pmi["moment"]).max()
    assert fs > 0
    assert np.abs(got["force"] - ref.pmi["force"]).max() <= 1e-6 * fs
    assert np.abs(got["moment"] - ref.pmi["moment"]).max() <= 1e-6 * ms


def test_mixed_mesh_follows_set_bodies(cuda, oracle):
    """A pose set between calls moves the triangles (and re-bins when the move
    exceeds half the skin); contacts are those of the moved mesh."""
    sc = small_drum()
    ds = engine.DeviceScene(sc, mode=engine.MODE_MIXED)
    ds.step(2)
    pmi = ds.get_bodies()
    pmi["ep"] = euler_parameters_about_y(0.05)
    pmi["origin"] = (0.0005, -0.0003, 0.0004)
    r0 = ds.rebuilds()[0]
    ds.set_bodies(pmi)
    f, m = ds.eval_contacts()
    st = ds.download()
    assert ds.rebuilds()[0] > r0
    ds.close()
    poly, sphere = sc.poly.copy(), sc.sphere.copy()
    oracle.update_polygon(pmi, sc.vlist, sphere, poly)
    sc.pmi = pmi
    _, f_ref, _, mag, _ = _oracle_mesh_view(oracle, sc, st, poly=poly, sphere=sphere)
    assert _norm_err(f, f_ref, mag, sc.mass) <= FORCE_TOL
