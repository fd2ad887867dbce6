"""FP64 contact forces on the GPU against the oracle.

Tolerance: the FP64 form may differ from the oracle only through the
last-place differences of sqrt-based x^1.5 vs pow and of the device log, so
per-particle force and torque errors are held to 1e-12 of the particle's own
force scale (max(|F_ref|, m g)); pair lists are bit-exact."""
import numpy as np
import pytest
import torch

from metakonga_gb300 import dem
from metakonga_gb300._lib import call, ptr

from .cases import packed_scene, small_drum
from .conftest import force_error

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _upload(sc):
    d = {k: dem.to_dev(getattr(sc, k)) for k in
         ("pos", "vel", "acc", "omega", "alpha", "force", "moment", "mass", "inertia")}
    return d


def _grid(sc, oracle):
    sphere = sc.sphere if sc.ntri else None
    return oracle.detection(sc.params, sc.pos, sphere)


def _dev_u32(a):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int32).copy()).cuda()


def test_p2p_matches_oracle(cuda, oracle):
    sc = packed_scene()
    p = sc.params.copy()
    p["np"] = sc.np_
    h, ix, cs, ce, so = _grid(sc, oracle)
    f_ref, m_ref = sc.force.copy(), sc.moment.copy()
    oracle.p2p(p, sc.pos, sc.vel, sc.omega, f_ref, m_ref, sc.mass, so, cs, ce, sc.cp_pp)
    d = _upload(sc)
    dem.set_symbolic_parameter(p)
    cpp = dem.ContactParticlesParticles(sc.cp_pp)
    cpp.cuda_collision(d["pos"], d["vel"], d["omega"], d["mass"], d["force"], d["moment"],
                       _dev_u32(so), _dev_u32(cs), _dev_u32(ce), sc.np_)
    torch.cuda.synchronize()
    f = d["force"].cpu().numpy()
    m = d["moment"].cpu().numpy()
    assert np.abs(f_ref - sc.force).max() > 1e-3, "test case has no contacts"
    assert force_error(f, f_ref, sc.mass) <= TOL
    # torque scale: |M| ~ r |Ft|
    assert force_error(m / sc.pos[:, 3:4], m_ref / sc.pos[:, 3:4], sc.mass) <= TOL


def test_pair_list_bit_exact(cuda, oracle):
    sc = packed_scene(n_side=10)
    p = sc.params.copy()
    p["np"] = sc.np_
    h, ix, cs, ce, so = _grid(sc, oracle)
    ref = oracle.pair_list(p, sc.pos, so, cs, ce)
    dem.set_symbolic_parameter(p)
    n = sc.np_
    counts = torch.zeros(n, dtype=torch.int32, device="cuda")
    cap = 40 * n
    pairs = torch.zeros((cap, 2), dtype=torch.int32, device="cuda")
    import ctypes as C
    total = C.c_ulonglong(0)
    # keep every device buffer referenced until the kernels have run
    dpos, dso, dcs, dce = dem.to_dev(sc.pos), _dev_u32(so), _dev_u32(cs), _dev_u32(ce)
    call("xd_pair_list", ptr(dpos), ptr(dso), ptr(dcs), ptr(dce), n, ptr(counts), ptr(pairs), cap,
         C.addressof(total), dem.stream_handle())
    got = pairs[: total.value].cpu().numpy().view(np.uint32)
    assert total.value == ref.shape[0] and total.value > n
    assert np.array_equal(got, ref)


def test_planes_match_oracle(cuda, oracle):
    """Six walls hugging a packed lattice: face, edge and corner regions."""
    sc = packed_scene(n_side=9)
    p = sc.params.copy()
    p["np"] = sc.np_
    f_ref, m_ref = sc.force.copy(), sc.moment.copy()
    for i in range(sc.planes.shape[0]):
        oracle.plane(p, sc.planes[i:i + 1], sc.pos, sc.vel, sc.omega, f_ref, m_ref, sc.mass,
                     sc.cp_planes[i:i + 1])
    assert np.abs(f_ref - sc.force).max() > 1e-3, "no wall contacts"
    # one call per plane (the reference launcher)
    d = _upload(sc)
    dem.set_symbolic_parameter(p)
    for i in range(sc.planes.shape[0]):
        dem.ContactParticlesPlane(sc.planes[i:i + 1], sc.cp_planes[i:i + 1]).cuda_collision(
            d["pos"], d["vel"], d["omega"], d["mass"], d["force"], d["moment"], None, None, None,
            sc.np_)
    torch.cuda.synchronize()
    assert force_error(d["force"].cpu().numpy(), f_ref, sc.mass) <= TOL
    assert np.array_equal(d["moment"].cpu().numpy(), m_ref)
    # all planes in one pass
    d2 = _upload(sc)
    dpl, dcp = dem.to_dev(sc.planes), dem.to_dev(sc.cp_planes)
    call("xd_planes_contact_force", 1, ptr(dpl), ptr(dcp), sc.planes.shape[0], ptr(d2["pos"]), ptr(d2["vel"]), ptr(d2["omega"]), ptr(d2["force"]),
         ptr(d2["moment"]), ptr(d2["mass"]), sc.np_, dem.stream_handle())
    torch.cuda.synchronize()
    assert force_error(d2["force"].cpu().numpy(), f_ref, sc.mass) <= TOL


def test_plane_regions_known_answer(cuda, oracle):
    """Single spheres placed in each region of one finite plane (face, four
    corners, four edges) give the oracle's forces; the face case also matches
    the closed-form Hertz + dashpot force.  The edge along u2 at x = 0 is the
    reference's unreachable branch (mphysics_cuda_impl.cuh:549 tests
    wp.x > 0 && wp.x < 0), so that sphere gets no force."""
    from metakonga_gb300 import scenes
    from metakonga_gb300.layouts import define_plane, make_params, make_contact_property
    pl = np.array([define_plane((0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0))])
    r = 0.01
    d = 0.002     # overlap
    s = (r - d) / np.sqrt(2.0)
    s3 = (r - d) / np.sqrt(3.0)
    pts = [(0.5, 0.5, r - d), (-s3, -s3, s3), (1 + s3, -s3, s3), (1 + s3, 1 + s3, s3),
           (-s3, 1 + s3, s3), (0.5, -s, s), (0.5, 1 + s, s), (1 + s, 0.5, s), (-s, 0.5, s)]
    pos = np.array([[x, y, z, r] for x, y, z in pts])
    n = pos.shape[0]
    m, inertia = scenes.mass_inertia(pos[:, 3])
    vel = np.zeros((n, 3))
    vel[:, 2] = -0.1
    omega = np.zeros((n, 3))
    omega[:, 0] = 3.0
    force = np.zeros((n, 3))
    moment = np.zeros((n, 3))
    cp = np.array([make_contact_property(E_i=1e7, E_j=1e7, nu_i=0.3, nu_j=0.3, rest=0.7, fric=0.3,
                                         sratio=0.8)])
    prm = make_params(np_=n, ncell=8, grid=(2, 2, 2), dt=1e-5, cell_size=0.1,
                      world_origin=(-1, -1, -1), gravity=(0, 0, -9.81))
    f_ref = force.copy()
    m_ref = moment.copy()
    oracle.plane(prm, pl, pos, vel, omega, f_ref, m_ref, m, cp)
    fmag = np.linalg.norm(f_ref, axis=1)
    assert np.all(fmag[:-1] > 0), "a region test sphere is not in contact"
    assert fmag[-1] == 0.0
    # closed form for the face case: Fn = kn d^1.5 + vn v (sphere vs rigid wall, Req = r, Meq = m)
    E, nu, e = 1e7, 0.3, 0.7
    Eeq = E * E / (E * (1 - nu * nu) + E * (1 - nu * nu))
    kn = 4.0 / 3.0 * Eeq * np.sqrt(r)
    beta = np.pi / np.log(e)
    vn = np.sqrt(4.0 * m[0] * kn / (1.0 + beta * beta))
    assert f_ref[0, 2] == pytest.approx(kn * d ** 1.5 + vn * 0.1, rel=1e-12)
    dem.set_symbolic_parameter(prm)
    dp = dem.to_dev(pos)
    dv = dem.to_dev(vel)
    do = dem.to_dev(omega)
    dm = dem.to_dev(m)
    df = dem.to_dev(force)
    dmo = dem.to_dev(moment)
    dem.ContactParticlesPlane(pl, cp).cuda_collision(dp, dv, do, dm, df, dmo, None, None, None, n)
    torch.cuda.synchronize()
    assert force_error(df.cpu().numpy(), f_ref, m) <= TOL


def test_cube_matches_oracle(cuda, oracle):
    sc = packed_scene(n_side=8)
    p = sc.params.copy()
    p["np"] = sc.np_
    planes6 = np.ascontiguousarray(sc.planes[:6])
    f_ref, m_ref = sc.force.copy(), sc.moment.copy()
    oracle.cube(p, planes6, sc.pos, sc.vel, sc.omega, f_ref, m_ref, sc.mass, sc.cp_pp)
    d = _upload(sc)
    dem.set_symbolic_parameter(p)
    dem.ContactParticlesCube(planes6, sc.cp_pp).cuda_collision(
        d["pos"], d["vel"], d["omega"], d["mass"], d["force"], d["moment"], None, None, None, sc.np_)
    torch.cuda.synchronize()
    assert force_error(d["force"].cpu().numpy(), f_ref, sc.mass) <= TOL


@pytest.mark.parametrize("nbodies_arg", [1, 0])
def test_polygon_matches_oracle(cuda, oracle, nbodies_arg):
    sc = small_drum()
    p = sc.params.copy()
    p["np"] = sc.np_
    h, ix, cs, ce, so = _grid(sc, oracle)
    f_ref, m_ref = sc.force.copy(), sc.moment.copy()
    pmi_ref = sc.pmi.copy()
    oracle.polygon(p, sc.poly, sc.sphere, pmi_ref, sc.pos, sc.vel, sc.omega, f_ref, m_ref, sc.mass,
                   so, cs, ce, sc.cp_poly)
    assert np.abs(f_ref - sc.force).max() > 1e-3, "no triangle contacts"
    d = _upload(sc)
    dem.set_symbolic_parameter(p)
    cpo = dem.ContactParticlesPolygonObjects(sc.poly, sc.sphere, sc.vlist, sc.pmi, sc.cp_poly)
    cpo.nbodies = nbodies_arg            # 0: the shim's "unknown body count" path (atomics)
    cpo.cuda_collision(d["pos"], d["vel"], d["omega"], d["mass"], d["force"], d["moment"],
                       _dev_u32(so), _dev_u32(cs), _dev_u32(ce), sc.np_)
    torch.cuda.synchronize()
    assert force_error(d["force"].cpu().numpy(), f_ref, sc.mass) <= TOL
    assert np.array_equal(d["moment"].cpu().numpy(), m_ref)
    got = cpo.bodies()
    scale = np.abs(f_ref - sc.force).sum()
    assert np.abs(got["force"] - pmi_ref["force"]).max() <= TOL * scale
    mscale = scale * 0.2
    assert np.abs(got["moment"] - pmi_ref["moment"]).max() <= TOL * mscale


def test_update_polygon_matches_oracle(cuda, oracle):
    from metakonga_gb300.scenes import euler_parameters_about_y
    sc = small_drum(n=50)
    pmi = sc.pmi.copy()
    pmi["ep"] = euler_parameters_about_y(0.37)
    pmi["origin"] = (0.01, -0.02, 0.03)
    poly_ref, sph_ref = sc.poly.copy(), sc.sphere.copy()
    oracle.update_polygon(pmi, sc.vlist, sph_ref, poly_ref)
    cpo = dem.ContactParticlesPolygonObjects(sc.poly, sc.sphere, sc.vlist, sc.pmi, sc.cp_poly)
    cpo.updatePolygonObjectData(pmi)
    torch.cuda.synchronize()
    poly = dem.from_dev(cpo.dpi, sc.poly)
    sph = cpo.dsphere.cpu().numpy()
    for f in ("P", "Q", "R"):
        assert np.array_equal(poly[f], poly_ref[f]), f
    assert np.abs(sph - sph_ref).max() <= 1e-15


def test_reduction_d3(cuda):
    rng = np.random.Generator(np.random.MT19937(1))
    a = rng.normal(size=(123_457, 3))
    out = np.zeros(3)
    call("xd_reduction_d3", ptr(dem.to_dev(a)), a.shape[0], out.ctypes.data, dem.stream_handle())
    assert np.allclose(out, a.sum(axis=0), rtol=1e-12, atol=1e-9)
