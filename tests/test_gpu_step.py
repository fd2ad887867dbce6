"""Whole steps on the GPU against the oracle: velocity-Verlet kernels, the
reference-order step through the host mirror (DemSimulation), and the
device-resident scene."""
import numpy as np
import pytest
import torch

from metakonga_gb300 import dem, engine, scenes

from .cases import packed_scene, small_drum
from .conftest import force_error

pytestmark = pytest.mark.gpu


def _state_err(got, ref, mass):
    """Relative state errors; "force" is the last step's force m a (the
    velocity update stores a = F / m and resets F to m g, as the reference's
    kernel does, so the force arrays themselves hold m g after a step)."""
    out = {}
    for k in ("pos", "vel", "omega"):
        a, b = np.asarray(got[k]), np.asarray(ref[k])
        scale = np.abs(b).max() + 1e-300
        out[k] = float(np.abs(a - b).max() / scale)
    m = np.asarray(mass)[:, None]
    out["force"] = force_error(np.asarray(got["acc"]) * m, np.asarray(ref["acc"]) * m, mass)
    return out


def test_vv_bit_exact(cuda, oracle):
    sc = packed_scene(n_side=10)
    rng = np.random.Generator(np.random.MT19937(2))
    sc.acc[:] = rng.normal(size=sc.acc.shape)
    sc.alpha[:] = rng.normal(size=sc.alpha.shape)
    sc.force[:] = rng.normal(size=sc.force.shape) * 1e-2
    sc.moment[:] = rng.normal(size=sc.moment.shape) * 1e-5
    p = sc.params.copy()
    p["np"] = sc.np_
    ref = sc.copy()
    oracle.vv_position(p, ref.pos, ref.vel, ref.acc)
    oracle.vv_velocity(p, ref.vel, ref.acc, ref.omega, ref.alpha, ref.force, ref.moment, ref.mass,
                       ref.inertia)
    d = {k: dem.to_dev(getattr(sc, k)) for k in
         ("pos", "vel", "acc", "omega", "alpha", "force", "moment", "mass", "inertia")}
    dem.set_symbolic_parameter(p)
    vv = dem.VelocityVerlet()
    vv.updatePosition(d["pos"], d["vel"], d["acc"], sc.np_)
    vv.updateVelocity(d["vel"], d["acc"], d["omega"], d["alpha"], d["force"], d["moment"], d["mass"],
                      d["inertia"], sc.np_)
    torch.cuda.synchronize()
    for k in ("pos", "vel", "acc", "omega", "alpha", "force", "moment"):
        assert np.array_equal(d[k].cpu().numpy(), getattr(ref, k)), k


def test_fused_velocity_position_equals_two_calls(cuda, oracle):
    from metakonga_gb300._lib import call, ptr
    sc = packed_scene(n_side=6)
    rng = np.random.Generator(np.random.MT19937(8))
    sc.force[:] = rng.normal(size=sc.force.shape) * 1e-2
    p = sc.params.copy()
    p["np"] = sc.np_
    ref = sc.copy()
    oracle.vv_velocity(p, ref.vel, ref.acc, ref.omega, ref.alpha, ref.force, ref.moment, ref.mass,
                       ref.inertia)
    oracle.vv_position(p, ref.pos, ref.vel, ref.acc)
    d = {k: dem.to_dev(getattr(sc, k)) for k in
         ("pos", "vel", "acc", "omega", "alpha", "force", "moment", "mass", "inertia")}
    dem.set_symbolic_parameter(p)
    call("xd_vv_update_velocity_position", *[ptr(d[k]) for k in
         ("pos", "vel", "acc", "omega", "alpha", "force", "moment", "mass", "inertia")], sc.np_,
         dem.stream_handle())
    torch.cuda.synchronize()
    for k in ("pos", "vel", "acc", "omega", "alpha", "force", "moment"):
        assert np.array_equal(d[k].cpu().numpy(), getattr(ref, k)), k


def test_dem_simulation_steps(cuda, oracle):
    """Five reference-order steps through the host mirror vs the oracle."""
    sc = packed_scene(n_side=10)
    ref = sc.copy()
    oracle.run(ref, 5)
    sim = dem.DemSimulation()
    sim.initialize(sc)
    for _ in range(5):
        sim.oneStepAnalysis()
    torch.cuda.synchronize()
    err = _state_err(sim.state(), ref.__dict__, sc.mass)
    assert err["pos"] <= 1e-13 and err["vel"] <= 1e-9 and err["force"] <= 1e-9, err


@pytest.mark.parametrize("case", ["packed", "drum"])
def test_device_scene_steps(cuda, oracle, case):
    sc = packed_scene(n_side=10) if case == "packed" else small_drum()
    ref = sc.copy()
    work = oracle.run(ref, 8)
    ds = engine.DeviceScene(sc)
    ds.step(3)
    ds.step(5, check=True)
    got = ds.download()
    err = _state_err(got, ref.__dict__, sc.mass)
    assert err["pos"] <= 1e-13 and err["vel"] <= 1e-9 and err["force"] <= 1e-9, err
    grid = ds.download_grid()
    for k in ("sorted", "cstart", "cend"):
        assert np.array_equal(grid[k], work[k]), k
    ds.close()


def test_settle_box_energy_decays(cuda):
    """Ensemble check on the 8,000-sphere settle: after 3,000 steps (0.03 s) the
    spheres have fallen (mean height down) and none has left the box."""
    sc = scenes.settle_box()
    z0 = sc.pos[:, 2].mean()
    ds = engine.DeviceScene(sc)
    ds.step(3000, check=True)
    got = ds.download()
    ds.close()
    z = got["pos"][:, 2]
    assert z.mean() < z0 - 0.004
    assert np.all(np.isfinite(got["pos"]))
    assert z.min() > -0.01


@pytest.mark.parametrize("scene", ["box", "drum"])
def test_fp64_graphs_match_direct_launches(cuda, scene):
    """The FP64 form replays its steps as CUDA graphs (8 steps, 1 step, the
    last step of a call); the state equals the directly launched run (phase
    timing on) bit for bit, across calls of several lengths."""
    sc = packed_scene(n_side=8) if scene == "box" else small_drum(n=300, seed=2)
    a = engine.DeviceScene(sc, mode=engine.MODE_FP64)
    b = engine.DeviceScene(sc, mode=engine.MODE_FP64)
    b.set_timing(True)
    for k in (19, 4, 11):
        a.step(k, check=True)
        b.step(k, check=True)
    sa, sb = a.download(), b.download()
    a.close()
    b.close()
    for k in ("pos", "vel", "omega", "acc", "alpha", "force", "moment"):
        assert np.array_equal(sa[k], sb[k]), k
