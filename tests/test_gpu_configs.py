"""Parity on the benchmark workloads at their stated sizes, in packed states.

The smaller cases of the other test files show the arithmetic; these show it
holds on the workloads the figures are quoted on, once the spheres are piled
into a bed (contacts everywhere, not a falling lattice):

* the 8,000-sphere settle in its box of five walls: the FP64 form equals the
  oracle step after step (per-step force within 1e-12 of max(|F|, m g),
  cell order and ranges bit for bit), from a settled bed;
* one hopper at the batch's largest size (199,583 spheres, the 4,096-triangle
  cone and the floor), settled with the orifice closed, then opened: the
  mixed form's pair list equals the oracle's and its per-particle force is
  within 2e-5 of max(sum_c |F_c|, m g); the FP64 form within 1e-12;
* an axial slab of the rotating drum (the full 20,480-triangle cylinder,
  turning at 1 rad/s) with a settled bed: the same gates;
* a 100,000-sphere window of the polydisperse settle (its box at the same
  density, settled): the same gates.

The beds are prepared by metakonga_gb300.prepare.settle (a coarser time step
for the fall, in the mixed form); the comparisons then evaluate identical
input states.  The oracle is the C restatement of the reference's FP64 path.
"""
import functools

import numpy as np
import pytest

from metakonga_gb300 import engine, prepare, scenes

from .conftest import force_error
from .test_gpu_mixed import FORCE_TOL, _norm_err, _pairset

pytestmark = pytest.mark.gpu
FP64_TOL = 1e-12


def _oracle_view(oracle, sc, st):
    """The oracle's pair list, contact force and moment (no gravity) and the
    normaliser sum_c |F_c| of state st (pairs, planes, triangles)."""
    p = sc.params.copy()
    p["np"] = sc.np_
    pos = np.ascontiguousarray(st["pos"])
    vel = np.ascontiguousarray(st["vel"])
    om = np.ascontiguousarray(st["omega"])
    _, _, cs, ce, so = oracle.detection(p, pos, sc.sphere if sc.ntri else None)
    pairs = oracle.pair_list(p, pos, so, cs, ce)
    f = np.zeros((sc.np_, 3))
    m = np.zeros((sc.np_, 3))
    oracle.p2p(p, pos, vel, om, f, m, sc.mass, so, cs, ce, sc.cp_pp)
    for i in range(sc.planes.shape[0]):
        oracle.plane(p, sc.planes[i:i + 1], pos, vel, om, f, m, sc.mass, sc.cp_planes[i:i + 1])
    mag = oracle.contact_magnitudes(p, pos, vel, om, sc.mass, so, cs, ce, sc.cp_pp, sc.planes, sc.cp_planes)
    if sc.ntri:
        pmi = sc.pmi.copy()
        ft = np.zeros((sc.np_, 3))
        mt = np.zeros((sc.np_, 3))
        oracle.polygon(p, sc.poly, sc.sphere, pmi, pos, vel, om, ft, mt, sc.mass, so, cs, ce, sc.cp_poly)
        f += ft
        m += mt
        mag = mag + np.linalg.norm(ft, axis=1)
    return pairs, f, m, mag


def _state_of(sc):
    return {k: getattr(sc, k) for k in ("pos", "vel", "omega")}


@functools.lru_cache(maxsize=None)
def _settled(name):
    """The packed state of each workload (prepared once per session)."""
    if name == "settle_8000":
        sc = scenes.settle_box()
        prepare.settle(sc, 8000, dt=4e-5)
    elif name == "hopper_max":
        spec = max(scenes.hopper_batch(count=256), key=lambda d: d["n"])
        sc = scenes.hopper(gate=True, **spec)
        prepare.settle(sc, 5000, dt=4e-5)
        prepare.open_gates(sc)
    elif name == "drum_slab":
        sc = scenes.drum_lattice(n=60_000, slab=0.06)
        prepare.settle(sc, 5000, dt=4e-5)
    elif name == "box_window":
        sc = scenes.polydisperse_box(n=100_000, seed=7)
        prepare.settle(sc, 30_000, dt=4e-5)
    else:
        raise KeyError(name)
    return sc


def test_settle_8000_fp64_equals_oracle_every_step(cuda, oracle):
    """The reference's CPU-runnable case at full size: 20 steps from a settled
    bed, each step from the oracle's own state, force within 1e-12 and the
    grid bit for bit."""
    sc = _settled("settle_8000").copy()
    ds = engine.DeviceScene(sc, mode=engine.MODE_FP64)
    ref = sc.copy()
    worst = 0.0
    touching = 0
    for _ in range(20):
        ds.upload(ref)
        ds.step(1, check=True)
        got = ds.download()
        grid = ds.download_grid()
        work = oracle.run(ref, 1)
        # the step's force is m a (the velocity update stores a = F / m and
        # resets F to m g for the next step, as the reference's kernel does)
        f_got, f_ref = got["acc"] * sc.mass[:, None], ref.acc * sc.mass[:, None]
        worst = max(worst, force_error(f_got, f_ref, sc.mass))
        contact = np.linalg.norm(f_ref - sc.mass[:, None] * np.array(scenes.GRAVITY), axis=1)
        touching = max(touching, int((contact > 1e-3 * sc.mass * 9.81).sum()))
        for k in ("sorted", "cstart", "cend"):
            assert np.array_equal(grid[k], work[k]), k
        assert np.array_equal(got["pos"], ref.pos)          # velocity Verlet is bit-exact
    ds.close()
    assert touching > 7000, touching          # a bed: nearly every sphere carries contact force
    assert worst <= FP64_TOL, worst


@pytest.mark.parametrize("name", ["hopper_max", "drum_slab", "box_window"])
def test_workload_packed_state_parity(cuda, oracle, name):
    """Mixed and FP64 forms against the oracle on one packed state of the
    workload: pair lists equal, forces and torques within the forms' gates."""
    sc = _settled(name)
    if name == "drum_slab":
        sc = sc.copy()
        # the drum turning: the wall's velocity enters every wall contact
        sc.pmi["omega"] = (0.0, 1.0, 0.0)
    st = _state_of(sc)
    pairs_ref, f_ref, m_ref, mag = _oracle_view(oracle, sc, st)
    assert pairs_ref.shape[0] > sc.np_, "the state is not packed"
    r = sc.pos[:, 3:4]
    mixed = engine.DeviceScene(sc, mode=engine.MODE_MIXED)
    pairs = mixed.pair_list(cap=32)
    f, m = mixed.eval_contacts()
    mixed.close()
    assert _pairset(pairs) == _pairset(pairs_ref)
    assert _norm_err(f, f_ref, mag, sc.mass) <= FORCE_TOL
    assert _norm_err(m / r, m_ref / r, mag, sc.mass) <= FORCE_TOL
    plain = engine.DeviceScene(sc, mode=engine.MODE_FP64)
    f64, m64 = plain.eval_contacts()
    plain.close()
    assert _norm_err(f64, f_ref, mag, sc.mass) <= FP64_TOL
    assert _norm_err(m64 / r, m_ref / r, mag, sc.mass) <= FP64_TOL
