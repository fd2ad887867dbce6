"""Mixed-precision scene mode against the FP64 oracle.

Gates (per step, on identical input states):
  * contact pair lists equal the oracle's (as sets of (i, k) pairs);
  * per-particle force error |F - F_ref| / max(sum_c |F_c|, m g) <= 2e-5, and
    the same for the torque divided by the radius;
  * over a short run the trajectory stays with the FP64 form, and a settle
    run reaches the same ensemble state (mean height, kinetic energy)."""
import numpy as np
import pytest

from metakonga_gb300 import engine, scenes
from metakonga_gb300.layouts import make_params

from .cases import packed_scene

pytestmark = pytest.mark.gpu
FORCE_TOL = 2e-5


def _oracle_view(oracle, sc, st):
    """Oracle pair list, contact forces and normaliser for state st."""
    p = sc.params.copy()
    p["np"] = sc.np_
    pos = np.ascontiguousarray(st["pos"])
    vel = np.ascontiguousarray(st["vel"])
    om = np.ascontiguousarray(st["omega"])
    h, ix, cs, ce, so = oracle.detection(p, pos)
    pairs = oracle.pair_list(p, pos, so, cs, ce)
    f = np.zeros((sc.np_, 3))
    m = np.zeros((sc.np_, 3))
    oracle.p2p(p, pos, vel, om, f, m, sc.mass, so, cs, ce, sc.cp_pp)
    for i in range(sc.planes.shape[0]):
        oracle.plane(p, sc.planes[i:i + 1], pos, vel, om, f, m, sc.mass, sc.cp_planes[i:i + 1])
    mag = oracle.contact_magnitudes(p, pos, vel, om, sc.mass, so, cs, ce, sc.cp_pp, sc.planes,
                                    sc.cp_planes)
    return pairs, f, m, mag


def _norm_err(a, b, mag, mass, g=9.81):
    den = np.maximum(mag, mass * g)
    return float((np.linalg.norm(a - b, axis=1) / den).max())


def _pairset(p):
    return set(map(tuple, np.asarray(p).tolist()))


@pytest.mark.parametrize("case", ["packed", "polydisperse"])
def test_mixed_pairs_and_forces(cuda, oracle, case):
    if case == "packed":
        sc = packed_scene(n_side=12)
    else:
        sc = scenes.polydisperse_box(n=30_000, seed=21)
        rng = np.random.Generator(np.random.MT19937(4))
        # squeeze the cloud so that there are many contacts, and give it motion
        c = sc.pos[:, :3].mean(axis=0)
        sc.pos[:, :3] = c + (sc.pos[:, :3] - c) * 0.5
        sc.vel[:] = rng.normal(0, 0.2, sc.vel.shape)
        sc.omega[:] = rng.normal(0, 20, sc.omega.shape)
    ds = engine.DeviceScene(sc, mode=engine.MODE_MIXED)
    ds.step(2)
    st = ds.download()
    pairs_ref, f_ref, m_ref, mag = _oracle_view(oracle, sc, st)
    assert pairs_ref.shape[0] > sc.np_, "test state has too few contacts"
    pairs = ds.pair_list(cap=48)
    assert _pairset(pairs) == _pairset(pairs_ref)
    f, m = ds.eval_contacts()
    ef = _norm_err(f, f_ref, mag, sc.mass)
    r = sc.pos[:, 3:4]
    em = _norm_err(m / r, m_ref / r, mag, sc.mass)
    ds.close()
    assert ef <= FORCE_TOL, ef
    assert em <= FORCE_TOL, em


def test_mixed_guard_band_pairs(cuda, oracle):
    """Sphere pairs placed at the touching distance and a few ulp either side:
    the contact decision equals the FP64 oracle's for every one of them."""
    rng = np.random.Generator(np.random.MT19937(17))
    rows = []
    x0 = 0.0
    for k in range(-6, 7):
        for t in range(6):
            ri, rj = rng.uniform(0.002, 0.004, 2)
            d = np.array(rng.normal(size=3))
            d /= np.linalg.norm(d)
            base = np.array([x0, 0.3 + 0.05 * t, 0.4])
            sep = ri + rj
            for _ in range(abs(k)):
                sep = np.nextafter(sep, np.inf if k > 0 else -np.inf)
            rows.append([*base, ri])
            rows.append([*(base + d * sep), rj])
            x0 += 0.03
    pos = np.array(rows)
    n = pos.shape[0]
    sc = scenes.settle_box(n_side=2)
    sc.pos = pos
    for key, val in scenes._state(pos).items():
        setattr(sc, key, val)
    sc.params = make_params(np_=n, ncell=128 ** 3, grid=(128, 128, 128), dt=1e-5, cell_size=0.0081,
                            world_origin=(-1.0, -1.0, -1.0), gravity=(0, 0, -9.81))
    sc.planes = sc.planes[:0]
    sc.cp_planes = sc.cp_planes[:0]
    sc.plane_names = []
    ds = engine.DeviceScene(sc, mode=engine.MODE_MIXED)
    pairs = ds.pair_list(cap=8)
    cnt = ds.counters()
    st = ds.download()
    ds.close()
    p = sc.params.copy()
    h, ix, cs, ce, so = oracle.detection(p, st["pos"])
    ref = oracle.pair_list(p, st["pos"], so, cs, ce)
    assert _pairset(pairs) == _pairset(ref)
    assert cnt["fp64_decisions"] > 0


def test_mixed_tracks_fp64_over_steps(cuda):
    sc = packed_scene(n_side=10)
    a = engine.DeviceScene(sc, mode=engine.MODE_FP64)
    b = engine.DeviceScene(sc, mode=engine.MODE_MIXED)
    a.step(20)
    b.step(20)
    sa, sb = a.download(), b.download()
    a.close()
    b.close()
    assert np.abs(sa["pos"] - sb["pos"]).max() < 1e-9
    vscale = np.abs(sa["vel"]).max()
    assert np.abs(sa["vel"] - sb["vel"]).max() < 1e-4 * vscale


def test_mixed_settle_ensemble(cuda):
    """8,000-sphere settle: 4,000 steps in both forms give the same mean height
    and kinetic energy within the stated bands (trajectories are chaotic, so
    only ensemble statistics are compared)."""
    sc = scenes.settle_box()
    res = {}
    for mode in (engine.MODE_FP64, engine.MODE_MIXED):
        ds = engine.DeviceScene(sc, mode=mode)
        ds.step(4000, check=True)
        st = ds.download()
        ds.close()
        z = st["pos"][:, 2]
        ke = 0.5 * (sc.mass[:, None] * st["vel"] ** 2).sum()
        res[mode] = (z.mean(), ke, z.min())
    (z64, ke64, zmin64), (zmx, kemx, zminmx) = res[engine.MODE_FP64], res[engine.MODE_MIXED]
    assert abs(z64 - zmx) < 2e-4
    assert abs(ke64 - kemx) <= 0.02 * ke64
    assert zminmx > -0.001


def test_mixed_graph_replay_matches_direct_launches(cuda):
    """Steps replayed from the captured CUDA graphs give bit-identical state to
    the same steps launched one by one (phase timing on disables the graphs)."""
    sc = packed_scene(n_side=10)
    a = engine.DeviceScene(sc, mode=engine.MODE_MIXED)
    b = engine.DeviceScene(sc, mode=engine.MODE_MIXED)
    b.set_timing(True)
    for chunk in (1, 7, 4, 9):          # odd and even counts exercise both buffer parities
        a.step(chunk)
        b.step(chunk)
    sa, sb = a.download(), b.download()
    a.close()
    b.close()
    for k in ("pos", "vel", "omega", "acc", "alpha"):
        assert np.array_equal(sa[k], sb[k]), k


def test_mixed_fast_movers_keep_pairs_exact(cuda, oracle):
    """Fast particles cross cells every step (thousands of movers per step,
    several shared-memory tiles in the near-sorted resort): the cell order
    stays right, so pair lists and forces still match the oracle."""
    sc = scenes.polydisperse_box(n=30_000, seed=33)
    rng = np.random.Generator(np.random.MT19937(8))
    c = sc.pos[:, :3].mean(axis=0)
    sc.pos[:, :3] = c + (sc.pos[:, :3] - c) * 0.6
    sc.vel[:] = rng.normal(0, 3.0, sc.vel.shape)
    sc.omega[:] = rng.normal(0, 50, sc.omega.shape)
    sc.params["dt"] = 2e-4
    sc.params["half2dt"] = 0.5 * 2e-4 * 2e-4
    ds = engine.DeviceScene(sc, mode=engine.MODE_MIXED)
    for _ in range(3):
        ds.step(2)
    st = ds.download()
    pairs_ref, f_ref, m_ref, mag = _oracle_view(oracle, sc, st)
    pairs = ds.pair_list(cap=48)
    f, m = ds.eval_contacts()
    ds.close()
    assert _pairset(pairs) == _pairset(pairs_ref)
    assert _norm_err(f, f_ref, mag, sc.mass) <= FORCE_TOL


def test_mixed_crowded_contacts_beyond_list(cuda, oracle):
    """Large spheres each touched by 40 small ones: more contacts than the
    per-particle contact list holds, so the rest come from a second search in
    the same order; pairs and forces still match the oracle."""
    rng = np.random.Generator(np.random.MT19937(23))
    R, r, nshell = 0.004, 0.001, 40
    k = np.arange(nshell) + 0.5
    phi = np.arccos(1.0 - 2.0 * k / nshell)
    th = np.pi * (1.0 + 5.0 ** 0.5) * k
    shell = np.stack([np.cos(th) * np.sin(phi), np.sin(th) * np.sin(phi), np.cos(phi)], axis=1)
    rows = []
    for b in range(6):
        c = np.array([0.03 * b, 0.1, 0.1])
        rows.append([*c, R])
        for d in shell:
            rows.append([*(c + d * (R + r - rng.uniform(1e-6, 3e-5))), r])
    pos = np.array(rows)
    n = pos.shape[0]
    sc = scenes.settle_box(n_side=2)
    sc.pos = pos
    for key, val in scenes._state(pos).items():
        setattr(sc, key, val)
    sc.vel[:] = rng.normal(0, 0.1, sc.vel.shape)
    sc.omega[:] = rng.normal(0, 10, sc.omega.shape)
    sc.params = make_params(np_=n, ncell=128 ** 3, grid=(128, 128, 128), dt=1e-5, cell_size=0.0081,
                            world_origin=(-1.0, -1.0, -1.0), gravity=(0, 0, -9.81))
    sc.planes = sc.planes[:0]
    sc.cp_planes = sc.cp_planes[:0]
    sc.plane_names = []
    ds = engine.DeviceScene(sc, mode=engine.MODE_MIXED)
    pairs = ds.pair_list(cap=64)
    f, m = ds.eval_contacts()
    st = ds.download()
    ds.close()
    pairs_ref, f_ref, m_ref, mag = _oracle_view(oracle, sc, st)
    big = np.flatnonzero(pos[:, 3] == R)
    assert all((np.asarray(pairs_ref)[:, 0] == b).sum() == nshell for b in big)
    assert _pairset(pairs) == _pairset(pairs_ref)
    rr = sc.pos[:, 3:4]
    assert _norm_err(f, f_ref, mag, sc.mass) <= FORCE_TOL
    assert _norm_err(m / rr, m_ref / rr, mag, sc.mass) <= FORCE_TOL


def _fast_scene(n=30_000, seed=33):
    sc = scenes.polydisperse_box(n=n, seed=seed)
    rng = np.random.Generator(np.random.MT19937(8))
    c = sc.pos[:, :3].mean(axis=0)
    sc.pos[:, :3] = c + (sc.pos[:, :3] - c) * 0.6
    sc.vel[:] = rng.normal(0, 3.0, sc.vel.shape)
    sc.omega[:] = rng.normal(0, 50, sc.omega.shape)
    sc.params["dt"] = 2e-4
    sc.params["half2dt"] = 0.5 * 2e-4 * 2e-4
    return sc


def test_mixed_rebinning_in_graphs_matches_direct(cuda, oracle):
    """Fast particles leave their cells' skin within a few steps, so cells are
    re-binned inside the replayed graphs (conditional nodes); the state equals
    the directly launched run bit for bit, and pairs stay exact."""
    sc = _fast_scene()
    a = engine.DeviceScene(sc, mode=engine.MODE_MIXED)
    b = engine.DeviceScene(sc, mode=engine.MODE_MIXED)
    b.set_timing(True)
    a.step(9)
    b.step(9)
    ra, rb = a.rebuilds()[0], b.rebuilds()[0]
    sa, sb = a.download(), b.download()
    pairs = a.pair_list(cap=48)
    a.close()
    b.close()
    assert ra == rb and ra > 2, (ra, rb)
    for k in ("pos", "vel", "omega", "acc", "alpha"):
        assert np.array_equal(sa[k], sb[k]), k
    pairs_ref = _oracle_view(oracle, sc, sa)[0]
    assert _pairset(pairs) == _pairset(pairs_ref)


def test_mixed_static_scene_bins_once(cuda):
    """Particles that stay inside their cells' skin keep their cells: a resting
    packing is binned once, at its first step."""
    sc = packed_scene(n_side=10)
    ds = engine.DeviceScene(sc, mode=engine.MODE_MIXED)
    ds.step(12)
    ds.step(5)
    cnt, each = ds.rebuilds()
    ds.close()
    assert cnt == 1 and each > 2
