"""The legacy DEM interface (cu_dem_dec.cuh) on the GPU against the
reference's own legacy kernels (fixtures from tests/golden/make_golden_legacy.py).

Gates: hashes, sorted indices and occupied cells' ranges bit-exact; contact
forces and moments within 1e-12 of max(|F_ref|, m g) per particle (FP64; the
device pow and the reference's host pow may differ in the last place);
positions 1e-13 and velocities 1e-9 relative after the steps; the mesh
placement within 1e-15 of the mesh's extent; face/edge flags equal; the shape
call's force sum within 1e-12 of the summed force magnitudes."""
import ctypes as C
import os

import numpy as np
import pytest
import torch

from metakonga_gb300._lib import call
from metakonga_gb300.layouts import LEGACY_PARAMS, LEGACY_POLYGON

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL = 1e-12


def _dev(a):
    a = np.ascontiguousarray(a)
    if a.dtype == np.uint32:
        a = a.view(np.int32)
    if a.dtype == np.bool_:
        a = a.view(np.uint8)
    return torch.from_numpy(a.copy()).cuda()


def _h(t, dtype=None):
    a = t.cpu().numpy()
    return a.view(dtype) if dtype is not None else a


def _err(f, f_ref, mass, g=9.81):
    den = np.maximum(np.linalg.norm(f_ref, axis=1), mass * g)
    return float((np.linalg.norm(f - f_ref, axis=1) / den).max())


def _params(d):
    p = np.frombuffer(d["params"].tobytes(), dtype=LEGACY_PARAMS).copy()
    call("xd_legacy_set_symbolic_parameter", p.ctypes.data)
    return p[0]


def test_legacy_packed_steps_match_reference(cuda):
    d = np.load(os.path.join(GOLDEN, "legacy_packed_512_cube.npz"))
    p = _params(d)
    n, nc = int(p["np"]), int(p["ncell"])
    S = {k: _dev(d["in_" + k]) for k in ("pos", "vel", "acc", "omega", "alpha")}
    S["force"] = torch.zeros((n, 3), dtype=torch.float64, device="cuda")
    S["moment"] = torch.zeros_like(S["force"])
    planes = _dev(d["planes"])
    cend = torch.zeros(nc, dtype=torch.int32, device="cuda")
    line = torch.zeros(n, dtype=torch.uint8, device="cuda")
    mass = d["in_acc"][:, 3]
    kn, vn, ks, vs, mu = (float(x) for x in d["wall"])
    P = lambda k: S[k].data_ptr()   # noqa: E731
    for t in range(int(d["steps"])):
        call("xd_legacy_vv_update_position", P("pos"), P("vel"), P("acc"), n, None)
        h = torch.zeros(n, dtype=torch.int32, device="cuda")
        ix = torch.zeros_like(h)
        call("xd_legacy_calculate_hash_and_index", h.data_ptr(), ix.data_ptr(), P("pos"), n, None)
        cs = torch.zeros(nc, dtype=torch.int32, device="cuda")
        so = torch.zeros_like(h)
        call("xd_legacy_reorder_and_find_cell_start", h.data_ptr(), ix.data_ptr(), cs.data_ptr(), cend.data_ptr(),
             so.data_ptr(), n, nc, None)
        S["force"].zero_()
        S["moment"].zero_()
        call("xd_legacy_calculate_p2p", P("pos"), P("vel"), P("acc"), P("omega"), P("alpha"), P("force"),
             P("moment"), so.data_ptr(), cs.data_ptr(), cend.data_ptr(), n, 0, None)
        torch.cuda.synchronize()
        assert _err(_h(S["force"]), d[f"s{t}_p2p_force"], mass) <= TOL
        assert _err(_h(S["moment"]) / 0.0057, d[f"s{t}_p2p_moment"] / 0.0057, mass) <= TOL
        call("xd_legacy_cube_hertzian_contact_force", planes.data_ptr(), kn, vn, ks, vs, mu, line.data_ptr(),
             P("pos"), P("vel"), P("omega"), P("force"), P("moment"), n, None)
        torch.cuda.synchronize()
        assert _err(_h(S["force"]), d[f"s{t}_force"], mass) <= TOL
        assert _err(_h(S["moment"]) / 0.0057, d[f"s{t}_moment"] / 0.0057, mass) <= TOL
        call("xd_legacy_vv_update_velocity", P("vel"), P("acc"), P("omega"), P("alpha"), P("force"),
             P("moment"), n, None)
        torch.cuda.synchronize()
        cs_h, ce_h = _h(cs, np.uint32), _h(cend, np.uint32)
        occ = np.flatnonzero(cs_h != 0xFFFFFFFF)
        assert np.array_equal(_h(h, np.uint32), d[f"s{t}_hash"])
        assert np.array_equal(_h(so, np.uint32), d[f"s{t}_sorted"])
        assert np.array_equal(occ, d[f"s{t}_cells"])
        assert np.array_equal(cs_h[occ], d[f"s{t}_cstart"]) and np.array_equal(ce_h[occ], d[f"s{t}_cend"])
        for k, tol in (("pos", 1e-13), ("vel", 1e-9)):
            ref = d[f"s{t}_{k}"]
            assert np.abs(_h(S[k]) - ref).max() <= tol * np.abs(ref).max(), (t, k)
        assert np.array_equal(_h(S["acc"])[:, 3], d[f"s{t}_acc"][:, 3])


def test_legacy_shape_matches_reference(cuda):
    d = np.load(os.path.join(GOLDEN, "legacy_drum_600_shape.npz"))
    p = _params(d)
    n, nc, nv = int(p["np"]), int(p["ncell"]), int(p["nsp"])
    verts, A, mpos = _dev(d["verts"]), _dev(d["A"]), _dev(d["mpos"])
    world = torch.zeros((nv, 3), dtype=torch.float64, device="cuda")
    call("xd_legacy_update_polygons_position", mpos.data_ptr(), A.data_ptr(), verts.data_ptr(), nv,
         world.data_ptr(), None)
    ni = d["indice"].shape[0]
    polygons = torch.zeros(ni * LEGACY_POLYGON.itemsize, dtype=torch.uint8, device="cuda")
    indice = _dev(d["indice"])
    call("xd_legacy_update_polygons_information", polygons.data_ptr(), indice.data_ptr(),
         world.data_ptr(), ni, None)
    pos = _dev(d["pos"])
    data = torch.zeros((n + nv, 4), dtype=torch.float64, device="cuda")
    call("xd_legacy_mergedata", data.data_ptr(), pos.data_ptr(), n, world.data_ptr(), nv, None)
    h = torch.zeros(n + nv, dtype=torch.int32, device="cuda")
    ix = torch.zeros_like(h)
    call("xd_legacy_calculate_hash_and_index", h.data_ptr(), ix.data_ptr(), data.data_ptr(), n + nv, None)
    cs = torch.zeros(nc, dtype=torch.int32, device="cuda")
    ce = torch.zeros_like(cs)
    so = torch.zeros_like(h)
    call("xd_legacy_reorder_and_find_cell_start", h.data_ptr(), ix.data_ptr(), cs.data_ptr(), ce.data_ptr(),
         so.data_ptr(), n + nv, nc, None)
    force = torch.zeros((n, 3), dtype=torch.float64, device="cuda")
    moment = torch.zeros_like(force)
    line = torch.zeros(n, dtype=torch.uint8, device="cuda")
    total = np.zeros(3)
    kn, vn, ks, vs, mu = (float(x) for x in d["wall"])
    # device copies held in variables: a tensor freed right after data_ptr()
    # would let the next one take its memory before the call runs
    T = {k: _dev(d[k]) for k in ("minfo", "id_set", "poly_start", "poly_end", "vel", "omega")}
    call("xd_legacy_shape_hertzian_contact_force", T["minfo"].data_ptr(), polygons.data_ptr(),
         T["id_set"].data_ptr(), T["poly_start"].data_ptr(), T["poly_end"].data_ptr(),
         kn, vn, ks, vs, mu, line.data_ptr(), pos.data_ptr(), T["vel"].data_ptr(),
         T["omega"].data_ptr(), force.data_ptr(), moment.data_ptr(), None, n, so.data_ptr(), cs.data_ptr(),
         ce.data_ptr(), total.ctypes.data, None)
    torch.cuda.synchronize()
    ext = np.abs(d["out_world"]).max()
    assert np.abs(_h(world) - d["out_world"]).max() <= 1e-15 * ext
    pg, pr = np.frombuffer(_h(polygons).tobytes(), LEGACY_POLYGON), d["out_polygons"].view(LEGACY_POLYGON)
    for k in LEGACY_POLYGON.names:
        assert np.abs(pg[k] - pr[k]).max() <= 1e-15 * max(ext, np.abs(pr[k]).max()), k
    assert np.array_equal(_h(data), d["out_data"])
    assert np.array_equal(_h(h, np.uint32), d["out_hash"])
    assert np.array_equal(_h(so, np.uint32), d["out_sorted"])
    cs_h = _h(cs, np.uint32)
    occ = np.flatnonzero(cs_h != 0xFFFFFFFF)
    assert np.array_equal(occ, d["out_cells"]) and np.array_equal(cs_h[occ], d["out_cstart"])
    assert np.array_equal(_h(line).astype(bool), d["out_line"])
    mass = np.pi * 4 / 3 * 2500.0 * d["pos"][:, 3] ** 3
    assert _err(_h(force), d["out_force"], mass) <= TOL
    r = d["pos"][:, 3:4]
    assert _err(_h(moment) / r, d["out_moment"] / r, mass) <= TOL
    assert np.abs(total - d["out_total"]).max() <= TOL * np.abs(d["out_force"]).sum()


def test_legacy_api_program_matches_reference(cuda, tmp_path):
    """A program using only the reference's legacy names (tests/cpp/legacy_step.cpp),
    linked with libxdem_legacy.so, reproduces the fixture's two steps."""
    import shutil
    import subprocess
    here = os.path.dirname(os.path.abspath(__file__))
    root = os.path.dirname(here)
    pkg = os.path.join(root, "metakonga_gb300")
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    cr = os.path.dirname(os.path.dirname(nvcc))
    exe = tmp_path / "legacy_step"
    subprocess.run(["g++", "-O2", "-std=c++17", os.path.join(here, "cpp", "legacy_step.cpp"),
                    "-I", os.path.join(root, "include"), "-I", os.path.join(cr, "include"),
                    "-L", pkg, "-lxdem_legacy", "-lxdem", "-L", os.path.join(cr, "lib64"), "-lcudart",
                    "-Wl,-rpath," + pkg, "-Wl,-rpath," + os.path.join(cr, "lib64"), "-o", str(exe)], check=True)
    d = np.load(os.path.join(GOLDEN, "legacy_packed_512_cube.npz"))
    n = d["in_pos"].shape[0]
    with open(tmp_path / "in.bin", "wb") as f:
        f.write(np.array([n, int(d["steps"])], np.uint32).tobytes())
        f.write(d["params"].tobytes())
        f.write(d["planes"].tobytes())
        f.write(np.asarray(d["wall"], np.float64).tobytes())
        for k in ("pos", "vel", "acc", "omega", "alpha"):
            f.write(np.ascontiguousarray(d["in_" + k]).tobytes())
    r = subprocess.run([str(exe), str(tmp_path / "in.bin"), str(tmp_path / "out.bin")], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr
    buf = open(tmp_path / "out.bin", "rb").read()
    t = int(d["steps"]) - 1
    off = 0
    for k, tol in (("pos", 1e-13), ("vel", 1e-9), ("acc", 1e-9), ("omega", 1e-9), ("alpha", 1e-9)):
        a = np.frombuffer(buf, np.float64, 4 * n, off).reshape(n, 4)
        off += 32 * n
        ref = d[f"s{t}_{k}"]
        assert np.abs(a - ref).max() <= tol * np.abs(ref).max(), k
    assert np.array_equal(np.frombuffer(buf, np.uint32, n, off), d[f"s{t}_sorted"])
