"""xd_cylinder_contact_force (cu_cylinder_hertzian_contact_force) against the
oracle on the cloud of tests/cylinder_case.py: forces, moments and the
per-particle reaction on the cylinder within 1e-12 of each particle's force
scale (the device atan/sin/cos and the oracle's libm may differ in the last
place); the C++ drop-in name gives the same bits."""

import numpy as np
import pytest
import torch

from metakonga_gb300 import dem
from metakonga_gb300._lib import call, ptr

from .conftest import force_error
from .cylinder_case import cloud

pytestmark = pytest.mark.gpu
TOL = 1e-12


def test_cylinder_matches_oracle(cuda, oracle):
    c = cloud()
    n = c["pos"].shape[0]
    f0 = np.tile(c["mass"][:, None] * np.array([0.0, -9.81, 0.0]), 1).reshape(n, 3)
    f, m, mf, mm = f0.copy(), np.zeros((n, 3)), np.zeros((n, 3)), np.zeros((n, 3))
    oracle.cylinder(c["prm"], c["cyl"], c["pos"], c["vel"], c["omega"], f, m, c["mass"], c["cp"], c["mpos"],
                    mf, mm)
    assert np.abs(f - f0).max() > 1e-3, "no contacts"
    d = {k: dem.to_dev(v) for k, v in (("pos", c["pos"]), ("vel", c["vel"]), ("omega", c["omega"]),
                                       ("mass", c["mass"]), ("cyl", c["cyl"]), ("cp", c["cp"]),
                                       ("mpos", c["mpos"]), ("force", f0), ("moment", np.zeros((n, 3))))}
    dmf = torch.full((n, 3), float("nan"), dtype=torch.float64, device="cuda")
    dmm = torch.full((n, 3), float("nan"), dtype=torch.float64, device="cuda")
    dem.set_symbolic_parameter(c["prm"])
    call("xd_cylinder_contact_force", 1, ptr(d["cyl"]), ptr(d["pos"]), ptr(d["vel"]), ptr(d["omega"]),
         ptr(d["force"]), ptr(d["moment"]), ptr(d["mass"]), n, ptr(d["cp"]), ptr(d["mpos"]), ptr(dmf), ptr(dmm),
         dem.stream_handle())
    torch.cuda.synchronize()
    got_f, got_m = d["force"].cpu().numpy(), d["moment"].cpu().numpy()
    assert force_error(got_f, f, c["mass"]) <= TOL
    r = c["pos"][:, 3]
    assert force_error(got_m / r[:, None], m / r[:, None], c["mass"]) <= TOL
    assert force_error(dmf.cpu().numpy(), mf, c["mass"]) <= TOL
    scale = np.abs(mm).max()
    assert np.abs(dmm.cpu().numpy() - mm).max() <= TOL * scale


def test_cylinder_refuses_hmc(cuda):
    from metakonga_gb300._lib import XdemError
    c = cloud(n=8)
    dem.set_symbolic_parameter(c["prm"])
    t = torch.zeros(64, dtype=torch.float64, device="cuda")
    with pytest.raises(XdemError):
        call("xd_cylinder_contact_force", 0, ptr(t), ptr(t), ptr(t), ptr(t), ptr(t), ptr(t), ptr(t), 8, ptr(t),
             ptr(t), ptr(t), ptr(t), dem.stream_handle())
