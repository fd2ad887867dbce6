"""Known answers worked by hand for the oracle (no GPU): two equal spheres of
the 8,000-sphere settle's material meeting head on, one sphere against one
triangle in its face, edge and vertex regions, and the grid hash on cell
faces, below the grid's origin and beyond its end.

getConstant with TCM = 1 (mphysics_cuda_impl.cuh:238-246): Eeq = Ei Ej /
(Ei (1 - nuj^2) + Ej (1 - nui^2)), kn = 4/3 Eeq sqrt(Req), beta = pi / ln e,
vn = sqrt(4 Meq kn / (1 + beta^2)); DHSModel (impl:379-401) with no slip:
Fn = (-kn cdist^1.5 + vn (dv . u)) u, u from the particle to its partner."""
import math

import numpy as np
import pytest

from metakonga_gb300 import scenes
from metakonga_gb300.layouts import POLYGON_MASS, make_contact_property, make_params

E, NU, REST, FRIC, SRATIO = 1e7, 0.3, 0.7, 0.3, 0.8


def _cp():
    return np.array([make_contact_property(E_i=E, E_j=E, nu_i=NU, nu_j=NU, rest=REST, fric=FRIC,
                                           sratio=SRATIO)])


def _hertz(req, meq):
    eeq = E * E / (E * (1 - NU * NU) + E * (1 - NU * NU))
    kn = 4.0 / 3.0 * eeq * math.sqrt(req)
    beta = math.pi / math.log(REST)
    return kn, math.sqrt(4.0 * meq * kn / (1.0 + beta * beta))


def test_two_equal_spheres_head_on(oracle):
    r, delta, v = 0.005, 1e-4, 0.2
    pos = np.array([[0.0, 0.0, 0.0, r], [2 * r - delta, 0.0, 0.0, r]])
    vel = np.array([[v / 2, 0.0, 0.0], [-v / 2, 0.0, 0.0]])
    omega = np.zeros((2, 3))
    m, _ = scenes.mass_inertia(pos[:, 3])
    force, moment = np.zeros((2, 3)), np.zeros((2, 3))
    prm = make_params(np_=2, ncell=128 ** 3, grid=(128, 128, 128), dt=1e-5, cell_size=0.01,
                      world_origin=(-1, -1, -1), gravity=(0, 0, -9.81))
    _, _, cs, ce, so = oracle.detection(prm, pos)
    oracle.p2p(prm, pos, vel, omega, force, moment, m, so, cs, ce, _cp())
    kn, vn = _hertz(r / 2, m[0] / 2)
    # the 8,000-sphere settle's constants: m = 1.309e-3 kg, Eeq = 5.4945e6 Pa,
    # kn = 3.663e5 N/m^1.5, vn = 3.49 N s/m
    assert m[0] == pytest.approx(1.309e-3, rel=1e-3)
    assert kn == pytest.approx(3.663e5, rel=1e-3) and vn == pytest.approx(3.49, rel=2e-3)
    fn = kn * delta ** 1.5 + vn * v
    np.testing.assert_allclose(force[0], (-fn, 0.0, 0.0), rtol=1e-12, atol=1e-12 * fn)
    np.testing.assert_allclose(force[1], (fn, 0.0, 0.0), rtol=1e-12, atol=1e-12 * fn)
    assert np.all(moment == 0.0)     # no slip: no tangential force, no moment


def test_sphere_on_a_triangle_face_edge_and_vertex(oracle):
    """Triangle P (0,0,0), Q (L,0,0), R (0,L,0); spheres of radius r overlap
    it by delta at the face, at the middle of edge PQ and at vertex P, each
    falling at w.  The reference's polygon kernel (impl:923-1021) takes the
    overlap from the closest point (closestPtPointTriangle, impl:837-899) and
    the direction from the face winding, u = -(Q - P) x (R - P) / |.| = -z:
    every sphere gets Fz = kn delta^1.5 + vn w with Req = r and Meq = m, and
    the body the opposite."""
    r, delta, w, L = 0.005, 1e-4, 0.3, 0.1
    d = r - delta
    tri = np.array([[[0.0, 0.0, 0.0], [L, 0.0, 0.0], [0.0, L, 0.0]]])
    poly, sphere, _ = scenes._mesh_arrays(tri)
    pos = np.array([[0.25 * L, 0.25 * L, d, r],                                   # face
                    [0.5 * L, -d / math.sqrt(2), d / math.sqrt(2), r],             # edge PQ
                    [-d / math.sqrt(3), -d / math.sqrt(3), d / math.sqrt(3), r]])  # vertex P
    n = pos.shape[0]
    vel = np.zeros((n, 3))
    vel[:, 2] = -w
    omega = np.zeros((n, 3))
    m, _ = scenes.mass_inertia(pos[:, 3])
    force, moment = np.zeros((n, 3)), np.zeros((n, 3))
    pmi = np.zeros(1, dtype=POLYGON_MASS)
    pmi["ep"] = (1.0, 0.0, 0.0, 0.0)
    prm = make_params(np_=n, ncell=16 ** 3, grid=(16, 16, 16), dt=1e-5, cell_size=0.15,
                      world_origin=(-1, -1, -1), gravity=(0, 0, -9.81), nsphere=1)
    _, _, cs, ce, so = oracle.detection(prm, pos, sphere)
    oracle.polygon(prm, poly, sphere, pmi, pos, vel, omega, force, moment, m, so, cs, ce, _cp())
    kn, vn = _hertz(r, m[0])
    fz = kn * delta ** 1.5 + vn * w
    for i in range(n):
        np.testing.assert_allclose(force[i], (0.0, 0.0, fz), rtol=1e-9, atol=1e-9 * fz)
    assert np.all(moment == 0.0)
    np.testing.assert_allclose(pmi["force"][0], (0.0, 0.0, -n * fz), rtol=1e-9, atol=1e-9 * fz)


def test_grid_hash_on_cell_faces_below_and_beyond_the_grid(oracle):
    """calcGridPos / calcGridHash (impl:65-83): c = floor((p - wo) / cs),
    hash = (cz & (gz-1)) gy gx + (cy & (gy-1)) gx + (cx & (gx-1)).  Cells of
    0.25 m from wo = -1 m on a 128^3 grid: a coordinate on a cell face falls
    in the cell above it, one below the origin wraps to cell 127, and one
    128 cells up wraps to cell 0."""
    g = 128
    prm = make_params(np_=5, ncell=g ** 3, grid=(g, g, g), dt=1e-5, cell_size=0.25,
                      world_origin=(-1, -1, -1), gravity=(0, 0, -9.81))
    pos = np.array([[-1.0, -1.0, -1.0, 0.01],      # the origin: cell (0, 0, 0)
                    [-0.75, -0.5, 0.0, 0.01],      # faces: cells (1, 2, 4)
                    [-1.25, -1.0, -1.0, 0.01],     # below the origin: cx = -1 -> 127
                    [31.0, -0.875, -1.0, 0.01],    # 128 cells up: cx = 128 -> 0; cy = 0
                    [-1.0, -1.0, -1.0 - 1e-12, 0.01]])   # just below a face: cz = -1 -> 127
    cells = [(0, 0, 0), (1, 2, 4), (127, 0, 0), (0, 0, 0), (0, 0, 127)]
    want = np.array([cz * g * g + cy * g + cx for cx, cy, cz in cells], dtype=np.uint32)
    h = np.zeros(5, np.uint32)
    ix = np.zeros(5, np.uint32)
    oracle.hash_and_index(prm, pos, h, ix)
    assert np.array_equal(h, want)
    assert np.array_equal(ix, np.arange(5, dtype=np.uint32))
