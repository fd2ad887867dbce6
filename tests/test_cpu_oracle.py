"""CPU tests: the oracle against the golden fixtures and the reference pin,
struct layouts, host-side logic, and the C ABI's exports (no GPU needed)."""
import glob
import os
import re

import numpy as np
import pytest

from metakonga_gb300 import layouts, scenes

from .cases import packed_scene, random_positions, small_drum

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
GOLDEN = sorted(p for p in glob.glob(os.path.join(HERE, "golden", "*.npz"))
                if not os.path.basename(p).startswith(("f32_", "legacy_")))
GOLDEN_F32 = sorted(glob.glob(os.path.join(HERE, "golden", "f32_*.npz")))
GOLDEN_LEGACY = sorted(glob.glob(os.path.join(HERE, "golden", "legacy_*.npz")))
STATE = ("pos", "vel", "acc", "omega", "alpha", "force", "moment", "mass", "inertia")


def struct_equal(a, b):
    """Field-by-field equality of structured arrays (padding bytes ignored)."""
    return all(np.array_equal(a[f], b[f]) for f in a.dtype.names)


def _scene_from_golden(z):
    sc = scenes.settle_box(n_side=2)
    for k in STATE:
        setattr(sc, k, z["in_" + k].copy())
    sc.params = z["params"].view(layouts.PARAMS).reshape(()).copy()
    sc.cp_pp = z["cp_pp"].view(layouts.CONTACT_PROPERTY).reshape(()).copy()
    sc.planes = z["planes"].view(layouts.PLANE).copy()
    sc.cp_planes = z["cp_planes"].view(layouts.CONTACT_PROPERTY).copy()
    if "poly" in z:
        sc.poly = z["poly"].view(layouts.POLYGON).copy()
        sc.sphere = z["sphere"].copy()
        sc.vlist = z["vlist"].copy()
        sc.pmi = z["pmi"].view(layouts.POLYGON_MASS).copy()
        sc.cp_poly = z["cp_poly"].view(layouts.CONTACT_PROPERTY).copy()
    else:
        sc.poly = sc.sphere = sc.vlist = sc.pmi = sc.cp_poly = None
    return sc


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def test_oracle_reproduces_golden(oracle, path):
    """The C restatement reproduces the reference kernels' outputs bit for bit."""
    z = np.load(path)
    sc = _scene_from_golden(z)
    work = oracle.run(sc, int(z["steps"]))
    for k in STATE:
        assert np.array_equal(getattr(sc, k), z["out_" + k]), k
    assert np.array_equal(work["sorted"], z["out_sorted"])
    assert np.array_equal(work["hash"], z["out_hash"])
    cells = z["out_cells"]
    assert np.array_equal(np.flatnonzero(work["cstart"] != 0xFFFFFFFF), cells)
    assert np.array_equal(work["cstart"][cells], z["out_cstart"])
    assert np.array_equal(work["cend"][cells], z["out_cend"])
    if "out_pmi" in z:
        assert struct_equal(sc.pmi, z["out_pmi"].view(layouts.POLYGON_MASS))


def test_golden_fixtures_present():
    assert len(GOLDEN) >= 2
    assert len(GOLDEN_F32) == 3


def test_fp32_golden_reproduced_by_reference_kernels(tmp_path, monkeypatch):
    """The single-precision fixtures are what the reference's float kernels
    give now (regenerated into a temporary folder and compared bit for bit)."""
    _ref()
    from tests.golden import make_golden_fp32 as gen
    monkeypatch.setattr(gen, "HERE", str(tmp_path))
    gen.main()
    for path in GOLDEN_F32:
        a = np.load(path)
        b = np.load(os.path.join(tmp_path, os.path.basename(path)))
        assert sorted(a.files) == sorted(b.files)
        for k in a.files:
            assert np.array_equal(a[k], b[k]), (path, k)


def test_legacy_golden_reproduced_by_reference_kernels(tmp_path, monkeypatch):
    """The legacy-interface fixtures are what the reference's legacy kernels
    give now (regenerated into a temporary folder and compared bit for bit)."""
    from oracle.pyoracle import LegacyRefKernels
    if not LegacyRefKernels.available():
        pytest.skip("legacy reference kernels not built here (oracle/_ref needs the reference tree)")
    assert len(GOLDEN_LEGACY) == 2
    from tests.golden import make_golden_legacy as gen
    monkeypatch.setattr(gen, "HERE", str(tmp_path))
    gen.main()
    for path in GOLDEN_LEGACY:
        a = np.load(path)
        b = np.load(os.path.join(tmp_path, os.path.basename(path)))
        assert sorted(a.files) == sorted(b.files)
        for k in a.files:
            assert np.array_equal(a[k], b[k]), (path, k)


def test_legacy_layouts_match_reference_structs():
    from oracle.pyoracle import LegacyRefKernels
    if not LegacyRefKernels.available():
        pytest.skip("legacy reference kernels not built here")
    sz = LegacyRefKernels().sizes()
    assert sz == {"params": layouts.LEGACY_PARAMS.itemsize, "plane": layouts.LEGACY_PLANE.itemsize,
                  "polygon": layouts.LEGACY_POLYGON.itemsize, "mass_info": layouts.LEGACY_MASS_INFO.itemsize}


def test_fp32_layouts_match_reference_structs():
    """The float records have the reference's sizes (mphysics_cuda_dec.cuh:165-246),
    also as compiled into the reference kernels' host build when present."""
    from metakonga_gb300 import _lib
    L = _lib.lib()
    for name, dt in (("device_parameters_f", layouts.PARAMS_F),
                     ("device_contact_property_f", layouts.CONTACT_PROPERTY_F),
                     ("device_plane_info_f", layouts.PLANE_F),
                     ("device_polygon_info_f", layouts.POLYGON_F),
                     ("device_polygon_mass_info_f", layouts.POLYGON_MASS_F)):
        assert L.xd_sizeof(name.encode()) == dt.itemsize, name
    from oracle.pyoracle import RefKernels
    if RefKernels.available():
        import ctypes as C
        lib = C.CDLL(RefKernels().lib._name)
        lib.xdref_sizeof_params_f.restype = C.c_uint
        assert lib.xdref_sizeof_params_f() == layouts.PARAMS_F.itemsize


def _ref():
    from oracle.pyoracle import RefKernels
    if not RefKernels.available():
        pytest.skip("reference kernels not built here (oracle/_ref needs the reference tree)")
    return RefKernels()


@pytest.mark.parametrize("case", ["packed", "drum", "wrapped", "cohesion", "no_rolling", "polydisperse"])
def test_oracle_matches_reference_kernels(oracle, case):
    """Pin: the restatement equals the reference's own kernels (host build)
    on fresh seeded inputs, step by step: packed overlaps with the box's
    planes, triangle contacts in a drum, the grid's wrap, cohesion
    (cohesionForce, impl:259-279), the relative velocity without rolling
    (impl:455-457), and radii of a spread (getConstant's Req and Meq)."""
    ref = _ref()
    if case == "packed":
        sc = packed_scene(n_side=9)
    elif case == "drum":
        sc = small_drum(n=300)
    elif case == "cohesion":
        sc = packed_scene(n_side=7)        # the planes keep their property without cohesion
        sc.cp_pp["coh"] = 1e5
    elif case == "no_rolling":
        sc = packed_scene(n_side=7)
        sc.params["rolling"] = 0
    elif case == "polydisperse":
        sc = packed_scene(n_side=8)
        rng = np.random.Generator(np.random.MT19937(17))
        sc.pos[:, 3] = rng.uniform(0.0048, 0.0062, sc.np_)
        sc.mass[:], sc.inertia[:] = scenes.mass_inertia(sc.pos[:, 3])
        sc.force[:] = sc.mass[:, None] * np.array(scenes.GRAVITY)
        sc.params["cell_size"] = 2.0 * sc.pos[:, 3].max()
    else:
        sc = packed_scene(n_side=7)
        sc.pos[:, :3] += np.array([1.7, -1.3, 0.9])      # beyond 128 cells: exercises the wrap
        for f in ("xw", "w2", "w3", "w4"):
            sc.planes[f] += np.array([1.7, -1.3, 0.9])
    a, b = sc.copy(), sc.copy()
    for _ in range(4):
        wa = oracle.run(a, 1)
        h, ix, cs, ce, so = ref.step(b)
        assert np.array_equal(wa["sorted"], so)
        assert np.array_equal(wa["cstart"], cs) and np.array_equal(wa["cend"], ce)
        for k in STATE:
            assert np.array_equal(getattr(a, k), getattr(b, k)), k
    if sc.ntri:
        assert struct_equal(a.pmi, b.pmi)


def test_oracle_cube_matches_reference(oracle):
    """Pin: cu_cube_contact_force (six plane launches, mphysics_cuda_def.cu:158-179)
    against the reference's kernels on a packed lattice whose outer spheres
    overlap the walls: the same bits."""
    ref = _ref()
    sc = packed_scene(n_side=8)
    p = sc.params.copy()
    p["np"] = sc.np_
    assert sc.planes.shape[0] == 6
    planes6 = np.ascontiguousarray(sc.planes)
    out = []
    for fn in (oracle.cube, ref.cube):
        f, m = sc.force.copy(), sc.moment.copy()
        fn(p, planes6, sc.pos, sc.vel, sc.omega, f, m, sc.mass, sc.cp_pp)
        out.append((f, m))
    assert np.abs(out[0][0] - sc.force).max() > 1e-3, "no wall contacts"
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


def test_oracle_update_polygon_matches_reference(oracle):
    ref = _ref()
    sc = small_drum(n=20)
    pmi = sc.pmi.copy()
    pmi["ep"] = scenes.euler_parameters_about_y(0.71)
    pmi["origin"] = (0.003, 0.0, -0.002)
    pa, sa = sc.poly.copy(), sc.sphere.copy()
    pb, sb = sc.poly.copy(), sc.sphere.copy()
    oracle.update_polygon(pmi, sc.vlist, sa, pa)
    ref.update_polygon(pmi, sc.vlist, sb, pb)
    assert struct_equal(pa, pb)
    assert np.array_equal(sa, sb)


def test_oracle_pair_list_consistent(oracle):
    sc = packed_scene(n_side=8)
    p = sc.params.copy()
    p["np"] = sc.np_
    h, ix, cs, ce, so = oracle.detection(p, sc.pos)
    pairs = oracle.pair_list(p, sc.pos, so, cs, ce)
    # brute force: every overlapping pair appears exactly once per side
    d = np.linalg.norm(sc.pos[:, None, :3] - sc.pos[None, :, :3], axis=2)
    ov = (sc.pos[:, None, 3] + sc.pos[None, :, 3]) - d > 0
    np.fill_diagonal(ov, False)
    brute = set(zip(*np.nonzero(ov)))
    got = set(map(tuple, pairs.tolist()))
    assert got == brute


def test_cpu_path_runs_and_differs_as_documented(oracle):
    """The reference CPU path (timed baseline) runs and keeps its documented
    divergences from the GPU path (different VV association, plane contacts
    assigned instead of added)."""
    sc = packed_scene(n_side=6)
    a, b = sc.copy(), sc.copy()
    oracle.run(a, 3, cpu_path=True)
    oracle.run(b, 3, cpu_path=False)
    assert np.all(np.isfinite(a.pos))
    assert np.abs(a.pos - b.pos).max() < 1e-4
    assert not np.array_equal(a.vel, b.vel)


def test_cpu_path_polygon_contact_closed_form(oracle):
    """The reference CPU path's polygon contact (cppolyCollision): a sphere at
    rest overlapping one horizontal triangle by delta gets the Hertz force
    kn delta^1.5 along the face normal (Req = r, kn = 4/3 Eeq sqrt(r)), and
    the body the opposite reaction."""
    from metakonga_gb300.layouts import POLYGON_MASS
    sc = scenes.settle_box(n_side=1)
    r, delta = 0.005, 1e-4
    sc.pos[:] = (0.0, 0.0, r - delta, r)
    sc.vel[:] = 0.0
    sc.acc[:] = 0.0
    sc.planes, sc.cp_planes, sc.plane_names = sc.planes[:0], sc.cp_planes[:0], []
    tri = np.array([[[-0.01, -0.01, 0.0], [0.01, -0.01, 0.0], [0.0, 0.01, 0.0]]])
    sc.poly, sc.sphere, sc.vlist = scenes._mesh_arrays(tri)
    sc.pmi = np.zeros(1, dtype=POLYGON_MASS)
    sc.pmi["ep"] = (1.0, 0.0, 0.0, 0.0)
    sc.cp_poly = sc.cp_pp.reshape(1).copy()
    sc.params["cell_size"] = 0.025
    oracle.run(sc, 1, cpu_path=True)
    cp = sc.cp_poly[0]
    eeq = cp["Ei"] * cp["Ej"] / (cp["Ei"] * (1 - cp["prj"] ** 2) + cp["Ej"] * (1 - cp["pri"] ** 2))
    fn = 4.0 / 3.0 * eeq * np.sqrt(r) * delta ** 1.5
    m = sc.mass[0]
    np.testing.assert_allclose(sc.acc[0], (0.0, 0.0, fn / m - 9.81), rtol=1e-12, atol=1e-9)
    np.testing.assert_allclose(sc.pmi["force"][0], (0.0, 0.0, -fn), rtol=1e-12, atol=1e-12 * fn)


def test_struct_layouts(oracle):
    expect = {"params": 112, "plane": 232, "polygon": 152, "polygon_mass": 160,
              "contact_property": 88}
    assert oracle.sizes() == expect
    assert layouts.PARAMS.itemsize == 112 and layouts.POLYGON_MASS.fields["ep"][1] == 32


def test_plane_definition_matches_reference_formulas():
    pl = layouts.define_plane((0, 0, 0), (2, 0, 0), (2, 3, 0), (0, 3, 0))
    assert pl["l1"] == 2 and pl["l2"] == 3
    assert np.array_equal(pl["uw"], [0, 0, 1])
    assert np.array_equal(pl["w3"], [2, 3, 0])


def test_scene_generators():
    sc = scenes.settle_box()
    assert sc.np_ == 8000 and sc.planes.shape[0] == 5
    d = np.diff(np.sort(sc.pos[:, 0]))
    assert sc.pos[:, 3].min() == 0.005
    pb = scenes.polydisperse_box(n=20_000)
    from scipy.spatial import cKDTree
    pairs = cKDTree(pb.pos[:, :3]).query_pairs(0.008, output_type="ndarray")
    dist = np.linalg.norm(pb.pos[pairs[:, 0], :3] - pb.pos[pairs[:, 1], :3], axis=1)
    assert np.all(dist >= pb.pos[pairs[:, 0], 3] + pb.pos[pairs[:, 1], 3])
    assert 0.002 <= pb.pos[:, 3].min() and pb.pos[:, 3].max() <= 0.004
    m, inertia = scenes.mass_inertia(np.array([0.005]))
    assert m[0] == pytest.approx(1.3089969e-3, rel=1e-6)


def test_drum_mesh_winding_and_count():
    tri = scenes.cylinder_mesh(0.5, 0.4, 242, 20, 30)
    assert tri.shape[0] == 20480
    n = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
    c = tri.mean(axis=1)
    side = np.abs(c[:, 1]) < 0.2 - 1e-9
    # side normals point at the axis, cap normals into the drum
    assert np.all(np.einsum("ij,ij->i", n[side][:, [0, 2]], -c[side][:, [0, 2]]) > 0)
    assert np.all(n[~side][:, 1] * c[~side][:, 1] < 0)


def test_abi_library_exports_every_declared_symbol():
    """libxdem loads without a GPU and exports every function include/xdem.h and
    include/xdem_legacy.h declare."""
    from metakonga_gb300 import _lib
    lib = _lib.lib()
    decl = "".join(open(os.path.join(ROOT, "include", h)).read() for h in ("xdem.h", "xdem_legacy.h"))
    names = set(re.findall(r"\b(xd_[a-z0-9_]+)\s*\(", decl))
    assert len(names) > 25
    for n in sorted(names):
        assert hasattr(lib, n), n
    assert set(_lib.exported_symbols()) == names
    assert lib.xd_version() == b"0.1.0"
    for s, size in (("device_parameters", 112), ("device_plane_info", 232),
                    ("device_polygon_info", 152), ("device_polygon_mass_info", 160),
                    ("device_contact_property", 88)):
        assert lib.xd_sizeof(s.encode()) == size


def test_abi_argument_errors_without_gpu():
    """Argument checks run before any CUDA call and report XD_ERR_INVALID."""
    from metakonga_gb300 import _lib
    lib = _lib.lib()
    lib.xd_clear_error()
    bad = np.zeros((), layouts.PARAMS)
    bad["grid"] = (3, 4, 4)
    bad["cell_size"] = 0.01
    assert lib.xd_set_symbolic_parameter(bad.ctypes.data) == 1
    import ctypes as C
    buf = C.create_string_buffer(256)
    assert lib.xd_last_error(buf, 256) == 1 and b"powers of two" in buf.value
    lib.xd_clear_error()
    assert lib.xd_reduction_d3(None, 10, None, None) == 1
    lib.xd_clear_error()
