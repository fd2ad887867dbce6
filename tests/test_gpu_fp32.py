"""The single-precision twins of the live API against the reference's own
float kernels (fixtures from tests/golden/make_golden_fp32.py).

Gates: cell hashes, sorted indices and occupied cells' ranges bit-exact;
per-particle contact force and torque / r within 1e-5 of max(|F_ref|, m g)
(float arithmetic in the same order; the ulps of the device powf, logf and
sqrt are the only differences); positions and velocities after the steps
within 1e-6 relative; the body reaction within 1e-4 of its scale (the
reference adds it in thread order, this library per block in a fixed order)."""
import os

import numpy as np
import pytest
import torch

from metakonga_gb300._lib import call
from metakonga_gb300.layouts import CONTACT_PROPERTY_F, PARAMS, PARAMS_F, PLANE_F, POLYGON_MASS_F

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FORCE_TOL = 1e-5


def _rec(raw, dtype):
    return np.frombuffer(raw.tobytes(), dtype=dtype).copy()


def _dev(a):
    a = np.ascontiguousarray(a)
    return torch.from_numpy(a.view(np.int32) if a.dtype == np.uint32 else a.copy()).cuda()


def _host(t, dtype=None):
    a = t.cpu().numpy()
    return a.view(dtype) if dtype is not None else a


def _err(f, f_ref, mass, g=9.81):
    den = np.maximum(np.linalg.norm(f_ref, axis=1), mass.astype(np.float64) * g)
    return float((np.linalg.norm(f.astype(np.float64) - f_ref.astype(np.float64), axis=1) / den).max())


def _set_params(d):
    call("xd_set_symbolic_parameter", _rec(d["hash_grid"], PARAMS).ctypes.data)
    call("xd_set_symbolic_parameter_f", _rec(d["params_f"], PARAMS_F).ctypes.data)


def _step(d, S, planes, cps, cp_pp, mesh):
    """One float step through the C ABI in the reference's order."""
    n = S["pos"].shape[0]
    nt = 0 if mesh is None else mesh["sphere"].shape[0]
    ncell = int(_rec(d["params_f"], PARAMS_F)["ncell"][0])
    call("xd_vv_update_position_f", S["pos"].data_ptr(), S["vel"].data_ptr(), S["acc"].data_ptr(), n, 0)
    h = torch.zeros(n + nt, dtype=torch.int32, device="cuda")
    ix = torch.zeros_like(h)
    call("xd_calculate_hash_and_index_f", h.data_ptr(), ix.data_ptr(), S["pos"].data_ptr(), n, 0)
    if nt:
        call("xd_calculate_hash_and_index_polysphere_f", h.data_ptr(), ix.data_ptr(), n, nt,
             mesh["sphere"].data_ptr(), 0)
    cs = torch.zeros(ncell, dtype=torch.int32, device="cuda")
    ce = torch.zeros_like(cs)
    so = torch.zeros_like(h)
    call("xd_reorder_and_find_cell_start_f", h.data_ptr(), ix.data_ptr(), cs.data_ptr(), ce.data_ptr(),
         so.data_ptr(), n + nt, ncell, 0)
    args = [S[k].data_ptr() for k in ("pos", "vel", "omega", "force", "moment", "mass")]
    call("xd_calculate_p2p_f", 1, *args, so.data_ptr(), cs.data_ptr(), ce.data_ptr(), cp_pp.data_ptr(), n, 0)
    for i in range(planes.shape[0]):
        call("xd_plane_contact_force_f", 1, planes[i:i + 1].data_ptr(), *args, n,
             cps[i:i + 1].data_ptr(), 0)
    if nt:
        call("xd_particle_polygon_collision_f", 1, mesh["poly"].data_ptr(), mesh["sphere"].data_ptr(),
             mesh["pmi"].data_ptr(), *args, so.data_ptr(), cs.data_ptr(), ce.data_ptr(),
             mesh["cp"].data_ptr(), n, mesh["nbodies"], 0)
    torch.cuda.synchronize()
    fm = (_host(S["force"]).copy(), _host(S["moment"]).copy())
    call("xd_vv_update_velocity_f", *[S[k].data_ptr() for k in
                                      ("vel", "acc", "omega", "alpha", "force", "moment", "mass", "inertia")],
         n, 0)
    torch.cuda.synchronize()
    cs_h, ce_h = _host(cs, np.uint32), _host(ce, np.uint32)
    occ = np.flatnonzero(cs_h != 0xFFFFFFFF)
    return {"hash": _host(h, np.uint32), "sorted": _host(so, np.uint32), "cells": occ,
            "cstart": cs_h[occ], "cend": ce_h[occ], "contact_force": fm[0], "contact_moment": fm[1]}


def _raw_dev(raw):
    return torch.from_numpy(np.ascontiguousarray(raw).copy()).cuda()


@pytest.mark.parametrize("name", ["f32_packed_512_walls.npz", "f32_drum_600_mesh.npz"])
def test_fp32_steps_match_reference_kernels(cuda, name):
    d = np.load(os.path.join(GOLDEN, name))
    _set_params(d)
    S = {k: _dev(d["in_" + k]) for k in ("pos", "vel", "acc", "omega", "alpha", "force", "moment",
                                         "mass", "inertia")}
    planes = _raw_dev(d["planes"])
    planes = planes.view(-1, PLANE_F.itemsize) if planes.numel() else planes
    cps = _raw_dev(d["cp_planes"])
    cps = cps.view(-1, CONTACT_PROPERTY_F.itemsize) if cps.numel() else cps
    cp_pp = _raw_dev(d["cp_pp"])
    mesh = None
    if "poly" in d.files:
        pmi = _rec(d["pmi"], POLYGON_MASS_F)
        mesh = {"poly": _raw_dev(d["poly"]), "sphere": _dev(d["sphere"]), "pmi": _raw_dev(d["pmi"]),
                "cp": _raw_dev(d["cp_poly"]), "nbodies": int(pmi.shape[0])}
    mass = d["in_mass"]
    r = d["in_pos"][:, 3:4].astype(np.float64)
    for t in range(int(d["steps"])):
        got = _step(d, S, planes, cps, cp_pp, mesh)
        for k in ("hash", "sorted", "cells", "cstart", "cend"):
            assert np.array_equal(got[k], d[f"s{t}_{k}"]), (t, k)
        f_ref = d[f"s{t}_contact_force"]
        assert np.abs(f_ref - d["in_force"]).max() > 0, "case has no contacts"
        assert _err(got["contact_force"], f_ref, mass) <= FORCE_TOL
        assert _err(got["contact_moment"] / r, d[f"s{t}_contact_moment"] / r, mass) <= FORCE_TOL
        for k in ("pos", "vel"):
            ref = d[f"s{t}_{k}"].astype(np.float64)
            assert np.abs(_host(S[k]) - ref).max() <= 1e-6 * max(np.abs(ref).max(), 1e-3), (t, k)
        if mesh is not None:
            got_pmi = np.frombuffer(_host(mesh["pmi"]).tobytes(), dtype=POLYGON_MASS_F)
            ref_pmi = _rec(d[f"s{t}_pmi"], POLYGON_MASS_F)
            for k in ("force", "moment"):
                scale = np.abs(ref_pmi[k]).max()
                assert scale > 0
                assert np.abs(got_pmi[k] - ref_pmi[k]).max() <= 1e-4 * scale, k


def test_fp32_cube_matches_reference_kernels(cuda):
    d = np.load(os.path.join(GOLDEN, "f32_cube_512.npz"))
    call("xd_set_symbolic_parameter_f", _rec(d["params_f"], PARAMS_F).ctypes.data)
    S = {k: _dev(d[k]) for k in ("pos", "vel", "omega", "force", "moment", "mass")}
    n = d["pos"].shape[0]
    planes6, cp = _raw_dev(d["planes6"]), _raw_dev(d["cp"])   # held until the call has run
    call("xd_cube_contact_force_f", 1, planes6.data_ptr(),
         *[S[k].data_ptr() for k in ("pos", "vel", "omega", "force", "moment", "mass")], n,
         cp.data_ptr(), 0)
    torch.cuda.synchronize()
    assert (d["out_force"] != d["force"]).any()
    assert _err(_host(S["force"]), d["out_force"], d["mass"]) <= FORCE_TOL
    assert np.array_equal(_host(S["moment"]) == 0, d["out_moment"] == 0)


def test_fp32_polygon_atomic_reaction_matches_fixed_order(cuda):
    """nbodies = 0 (the drop-in signature, which carries no body count) adds
    the same reaction with atomics."""
    d = np.load(os.path.join(GOLDEN, "f32_drum_600_mesh.npz"))
    _set_params(d)
    pmis = []
    for nb in (0, int(_rec(d["pmi"], POLYGON_MASS_F).shape[0])):
        S = {k: _dev(d["in_" + k]) for k in ("pos", "vel", "acc", "omega", "alpha", "force", "moment",
                                             "mass", "inertia")}
        mesh = {"poly": _raw_dev(d["poly"]), "sphere": _dev(d["sphere"]), "pmi": _raw_dev(d["pmi"]),
                "cp": _raw_dev(d["cp_poly"]), "nbodies": nb}
        _step(d, S, torch.zeros(0, dtype=torch.uint8, device="cuda"),
              torch.zeros(0, dtype=torch.uint8, device="cuda"), _raw_dev(d["cp_pp"]), mesh)
        pmis.append(np.frombuffer(_host(mesh["pmi"]).tobytes(), dtype=POLYGON_MASS_F))
    for k in ("force", "moment"):
        assert np.abs(pmis[0][k] - pmis[1][k]).max() <= 1e-4 * np.abs(pmis[1][k]).max()


def test_fp32_reduction(cuda):
    rng = np.random.Generator(np.random.MT19937(8))
    a = rng.normal(0.0, 1.0, (100_003, 3)).astype(np.float32)
    out = np.zeros(3, np.float32)
    da = _dev(a)
    call("xd_reduction_f3", da.data_ptr(), a.shape[0], out.ctypes.data, 0)
    ref = a.astype(np.float64).sum(axis=0)
    assert np.abs(out - ref).max() <= 1e-5 * np.abs(a).sum()
