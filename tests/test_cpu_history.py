"""Tangential-spring history (an extension: the reference's DHSModel keeps no
state between steps) in the oracle, against closed forms.

The model, per contact and step, with u the contact normal and vt the
tangential relative velocity:  d <- d - (d.u)u rescaled to |d|;
d <- d + vt dt;  Ft = ks d + vs vt;  if |Ft| > mu |Fn|: Ft <- mu |Fn| Ft/|Ft|
and d <- (Ft - vs vt) / ks.  A new contact starts from d = 0."""
import math

import numpy as np
import pytest

from metakonga_gb300 import scenes
from metakonga_gb300.layouts import make_params
from oracle.pyoracle import HIST_EMPTY, HIST_PLANE, History

from .cases import packed_scene

R = 0.005
DT = 1e-5


def _constants(r_eq, m_eq, fric=scenes.FRICTION):
    E, nu, e = scenes.E_YOUNG, scenes.POISSON, scenes.RESTITUTION
    eeq = (E * E) / (E * (1 - nu * nu) + E * (1 - nu * nu))
    beta = math.pi / math.log(e)
    kn = (4.0 / 3.0) * eeq * math.sqrt(r_eq)
    vn = math.sqrt((4.0 * m_eq * kn) / (1.0 + beta * beta))
    return kn, vn, kn * scenes.STIFFNESS_RATIO, vn * scenes.STIFFNESS_RATIO, fric


def _pair(overlap, vj, fric=scenes.FRICTION):
    """Sphere 0 at the origin, sphere 1 on +x overlapping by `overlap`, moving at vj."""
    pos = np.array([[0.0, 0.0, 0.0, R], [2 * R - overlap, 0.0, 0.0, R]])
    vel = np.array([[0.0, 0.0, 0.0], list(vj)])
    m, _ = scenes.mass_inertia(pos[:, 3])
    prm = make_params(np_=2, ncell=128 ** 3, grid=(128, 128, 128), dt=DT, cell_size=2 * R,
                      world_origin=(-1, -1, -1), gravity=(0, 0, -9.81))
    cp = scenes._default_property(fric=fric)
    return pos, vel, m, prm, cp


def _p2p_steps(oracle, pos, vel, m, prm, cp, hist, n):
    h, ix, cs, ce, so = oracle.detection(prm, pos)
    om = np.zeros((2, 3))
    out = []
    for _ in range(n):
        f = np.zeros((2, 3))
        mo = np.zeros((2, 3))
        oracle.hist_p2p(prm, pos, vel, om, f, mo, m, so, cs, ce, cp, hist)
        out.append((f.copy(), mo.copy()))
    return out


def test_sliding_pair_spring_grows_then_caps(oracle):
    overlap, v = 1e-4, 0.002
    pos, vel, m, prm, cp = _pair(overlap, (0.0, v, 0.0))
    hist = History(2, slots=4)
    steps = _p2p_steps(oracle, pos, vel, m, prm, cp, hist, 100)
    kn, vn, ks, vs, mu = _constants(R / 2, m[0] / 2)
    fn = kn * overlap ** 1.5
    capped = 0
    for n, (f, mo) in enumerate(steps, start=1):
        # particle 0: normal force along -x, tangential force along +y (dragged by 1)
        assert f[0, 0] == pytest.approx(-fn, rel=1e-12)
        ft = min(ks * n * v * DT + vs * v, mu * fn)
        capped += ks * n * v * DT + vs * v > mu * fn
        assert f[0, 1] == pytest.approx(ft, rel=1e-11)
        assert abs(f[0, 2]) < 1e-12 * fn
        # moment (R u) x Ft = R Ft z
        assert mo[0, 2] == pytest.approx(R * ft, rel=1e-11)
        # particle 1 sees the mirror force
        assert f[1, 1] == pytest.approx(-ft, rel=1e-11)
    assert 10 < capped < 90
    # at the cap the spring holds (Ft - vs vt) / ks
    d = hist.contacts(0)[1]
    assert d[1] == pytest.approx((mu * fn - vs * v) / ks, rel=1e-10)
    assert hist.overflow == 0


def test_first_step_equals_reference_dhs(oracle):
    """From empty tables, one step with history gives the reference's step."""
    a = packed_scene(n_side=6)
    b = a.copy()
    oracle.run(a, 1)
    oracle.run(b, 1, history=History(b.np_, slots=16))
    for k in ("pos", "vel", "omega"):
        scale = np.abs(getattr(a, k)).max()
        assert np.abs(getattr(a, k) - getattr(b, k)).max() <= 1e-12 * scale, k


def test_history_changes_later_steps_and_is_deterministic(oracle):
    a = packed_scene(n_side=6)
    b, c = a.copy(), a.copy()
    oracle.run(a, 5)
    hb, hc = History(b.np_, 16), History(c.np_, 16)
    oracle.run(b, 5, history=hb)
    oracle.run(c, 5, history=hc)
    assert np.array_equal(b.vel, c.vel) and np.array_equal(hb.delta, hc.delta)
    assert np.abs(a.vel - b.vel).max() > 0
    assert (hb.key != HIST_EMPTY).sum() > 0 and hb.overflow == 0
    # planes of the box keep springs too
    assert ((hb.key & 0xC0000000) == HIST_PLANE).sum() > 0


def test_spring_turns_with_the_contact_plane(oracle):
    """A spring built along y, then the contact normal turned by 30 degrees
    with no tangential motion: the spring keeps its length, lies in the new
    tangent plane, and gives Ft = ks d."""
    overlap, v = 2e-5, 0.01
    pos, vel, m, prm, cp = _pair(overlap, (0.0, v, 0.0), fric=10.0)
    hist = History(2, slots=4)
    _p2p_steps(oracle, pos, vel, m, prm, cp, hist, 10)
    d0 = hist.contacts(0)[1]
    th = math.radians(30.0)
    dist = 2 * R - overlap
    pos2 = pos.copy()
    pos2[1, :3] = (dist * math.cos(th), dist * math.sin(th), 0.0)
    (f, _), = _p2p_steps(oracle, pos2, np.zeros((2, 3)), m, prm, cp, hist, 1)
    d1 = hist.contacts(0)[1]
    u = np.array([math.cos(th), math.sin(th), 0.0])
    assert np.linalg.norm(d1) == pytest.approx(np.linalg.norm(d0), rel=1e-12)
    assert abs(d1 @ u) < 1e-12 * np.linalg.norm(d1)
    kn, vn, ks, vs, mu = _constants(R / 2, m[0] / 2, fric=10.0)
    fn_vec = -kn * overlap ** 1.5 * u
    assert np.allclose(f[0], fn_vec + ks * d1, rtol=0, atol=1e-10 * np.linalg.norm(f[0]))


def test_separation_frees_the_entry(oracle):
    pos, vel, m, prm, cp = _pair(1e-4, (0.0, 0.002, 0.0))
    hist = History(2, slots=4)
    _p2p_steps(oracle, pos, vel, m, prm, cp, hist, 5)
    assert 1 in hist.contacts(0)
    apart = pos.copy()
    apart[1, 0] += 1e-4
    _p2p_steps(oracle, apart, vel, m, prm, cp, hist, 1)
    assert hist.contacts(0) == {} and hist.contacts(1) == {}
    (f, _), = _p2p_steps(oracle, pos, vel, m, prm, cp, hist, 1)
    kn, vn, ks, vs, mu = _constants(R / 2, m[0] / 2)
    assert f[0, 1] == pytest.approx(ks * 0.002 * DT + vs * 0.002, rel=1e-11)


def test_sphere_sliding_on_a_plane(oracle):
    overlap, v = 1e-4, 0.002
    pos = np.array([[0.0, 0.0, R - overlap, R]])
    vel = np.array([[v, 0.0, 0.0]])
    m, _ = scenes.mass_inertia(pos[:, 3])
    prm = make_params(np_=1, ncell=128 ** 3, grid=(128, 128, 128), dt=DT, cell_size=2 * R,
                      world_origin=(-1, -1, -1), gravity=(0, 0, -9.81), rolling=False)
    planes, _ = scenes.box_walls((-0.1, -0.1, 0.0), (0.1, 0.1, 0.1))
    floor = planes[:1]
    cp = np.array([scenes._default_property()])
    hist = History(1, slots=2)
    kn, vn, ks, vs, mu = _constants(R, m[0])
    fn = kn * overlap ** 1.5
    capped = 0
    for n in range(1, 60):
        capped += ks * n * v * DT + vs * v > mu * fn
        f = np.zeros((1, 3))
        mo = np.zeros((1, 3))
        oracle.hist_planes(prm, floor, cp, pos, vel, np.zeros((1, 3)), f, mo, m, hist)
        assert f[0, 2] == pytest.approx(fn, rel=1e-12)
        # the floor drags the sphere back: Ft along -x
        assert f[0, 0] == pytest.approx(-min(ks * n * v * DT + vs * v, mu * fn), rel=1e-11)
        assert np.all(mo == 0)   # ir = 0 for walls, as in the reference
    assert 10 < capped < 50
    assert list(hist.contacts(0)) == [HIST_PLANE | 0]


def test_full_table_falls_back_to_fresh_springs(oracle):
    pos = np.array([[0.0, 0.0, 0.0, R], [2 * R - 2e-5, 0.0, 0.0, R], [-(2 * R - 2e-5), 0.0, 0.0, R]])
    vel = np.array([[0.0, 0.0, 0.0], [0.0, 0.01, 0.0], [0.0, 0.0, 0.01]])
    m, _ = scenes.mass_inertia(pos[:, 3])
    prm = make_params(np_=3, ncell=128 ** 3, grid=(128, 128, 128), dt=DT, cell_size=2 * R,
                      world_origin=(-1, -1, -1), gravity=(0, 0, -9.81))
    cp = scenes._default_property()
    hist = History(3, slots=1)
    h, ix, cs, ce, so = oracle.detection(prm, pos)
    for _ in range(3):
        oracle.hist_p2p(prm, pos, vel, np.zeros((3, 3)), np.zeros((3, 3)), np.zeros((3, 3)), m,
                        so, cs, ce, cp, hist)
    assert hist.overflow == 3      # particle 0's second contact, each step
    assert len(hist.contacts(0)) == 1


def test_kinematic_body_turns_and_moves_as_prescribed(oracle):
    """Prescribed body motion (an extension): after n steps at omega about y
    and velocity v, the Euler parameters are those of the rotation by
    omega n dt about y, and the origin has moved by v n dt."""
    from metakonga_gb300.layouts import POLYGON_MASS
    pmi = np.zeros(1, dtype=POLYGON_MASS)
    pmi["ep"] = (1.0, 0.0, 0.0, 0.0)
    pmi["omega"] = (0.0, 2.0, 0.0)
    pmi["vel"] = (0.01, 0.0, -0.02)
    dt, n = 5e-6, 4000
    for _ in range(n):
        oracle.advance_bodies(pmi, dt)
    th = 2.0 * n * dt
    assert np.allclose(pmi["ep"][0], (math.cos(th / 2), 0.0, math.sin(th / 2), 0.0), atol=1e-12)
    assert np.allclose(pmi["origin"][0], (0.01 * n * dt, 0.0, -0.02 * n * dt), atol=1e-15)
    assert abs(np.linalg.norm(pmi["ep"][0]) - 1.0) < 1e-15


def test_kinematic_drum_moves_its_mesh(oracle):
    """With kinematic bodies the oracle moves the triangles every step: a
    vertex of the drum turns about the axis by omega n dt."""
    from .cases import small_drum
    sc = small_drum()
    sc.pmi["vel"] = 0.0
    sc.pmi["omega"] = (0.0, 3.0, 0.0)
    p0 = sc.poly["P"][0].copy()
    oracle.run(sc, 10, kinematic=True)
    th = 3.0 * 10 * sc.dt
    # rotation about y by th: x' = x cos + z sin, z' = -x sin + z cos
    x, y, z = p0
    want = (x * math.cos(th) + z * math.sin(th), y, -x * math.sin(th) + z * math.cos(th))
    assert np.allclose(sc.poly["P"][0], want, atol=1e-12)
