"""The mixed form's tuning: any skin width, list capacity and contact block
size gives the oracle's contacts (they change how the contact pass finds
them, not what it finds), and the autotuner picks, times and caches one."""
import numpy as np
import pytest

from metakonga_gb300 import engine, scenes, tune
from metakonga_gb300._lib import XdemError

from .test_gpu_mixed import FORCE_TOL, _norm_err, _oracle_view, _pairset

pytestmark = pytest.mark.gpu


def _packed():
    sc = scenes.polydisperse_box(n=20_000, seed=33)
    rng = np.random.Generator(np.random.MT19937(8))
    c = sc.pos[:, :3].mean(axis=0)
    sc.pos[:, :3] = c + (sc.pos[:, :3] - c) * 0.5
    sc.vel[:] = rng.normal(0, 0.2, sc.vel.shape)
    sc.omega[:] = rng.normal(0, 20, sc.omega.shape)
    return sc


@pytest.mark.parametrize("tuning", [
    {"skin_factor": 0.35, "verlet_cap": 8, "triangle_cap": 4, "contact_threads": 32},   # lists overflow
    {"skin_factor": 0.05, "contact_threads": 128},
    {"skin_factor": 0.2, "verlet_cap": 96},
    {"contact_mode": 0},
    {"contact_mode": 0, "verlet_cap": 8},
])
def test_tuned_settings_give_the_oracle_contacts(cuda, oracle, tuning):
    sc = _packed()
    ds = engine.DeviceScene(sc, mode=engine.MODE_MIXED, tuning=tuning)
    assert ds.tuning() == dict(engine.DEFAULT_TUNING, **tuning)
    ds.step(2)
    st = ds.download()
    pairs_ref, f_ref, m_ref, mag = _oracle_view(oracle, sc, st)
    pairs = ds.pair_list(cap=48)
    f, m = ds.eval_contacts()
    stats = ds.stats()
    ds.close()
    assert _pairset(pairs) == _pairset(pairs_ref)
    assert _norm_err(f, f_ref, mag, sc.mass) <= FORCE_TOL
    r = sc.pos[:, 3:4]
    assert _norm_err(m / r, m_ref / r, mag, sc.mass) <= FORCE_TOL
    if tuning.get("verlet_cap") == 8:
        assert stats["verlet_overflows"] > 0      # the cell-search path ran


def test_tuning_is_checked_and_fixed_after_upload(cuda):
    sc = scenes.settle_box(n_side=4)
    with pytest.raises(XdemError):
        engine.DeviceScene(sc, mode=engine.MODE_MIXED, tuning={"contact_threads": 48})
    with pytest.raises(XdemError):
        engine.DeviceScene(sc, mode=engine.MODE_FP64, tuning={"skin_factor": 0.2})
    d = engine.DeviceScene(sc, mode=engine.MODE_MIXED)
    t = engine.Tuning(**dict(engine.DEFAULT_TUNING, skin_factor=0.2))
    from metakonga_gb300._lib import call
    import ctypes as C
    with pytest.raises(XdemError):
        call("xd_scene_set_tuning", d.handle, C.addressof(t))
    d.close()


def test_autotuner_times_and_caches(cuda, monkeypatch, tmp_path):
    monkeypatch.setenv("XDEM_TUNE_CACHE", str(tmp_path / "tuning.json"))
    sc = scenes.hopper(n=3000, seed=9)
    out = tune.tune(sc, steps=30, warm=5)
    assert out["tuning"] in [c["tuning"] for c in out["candidates"]]
    # the choice is within the tuner's margin of the fastest candidate
    assert out["ms_per_step"] * (1.0 - 0.05) <= min(c["ms_per_step"] for c in out["candidates"]) + 1e-12
    assert tune.tuned(sc) == out["tuning"]
    assert (tmp_path / "tuning.json").exists()
    # the chosen setting runs the scene
    d = engine.DeviceScene(sc, mode=engine.MODE_MIXED, tuning=tune.tuned(sc))
    d.step(10, check=True)
    d.close()


@pytest.mark.parametrize("case", ["packed", "packed_cells", "hopper_bed"])
def test_contact_modes_give_the_same_bits(cuda, case):
    """The warp-cooperative pair pass (contact_mode 1) sums each particle's
    contacts in its list order, as the per-particle pass does: the states
    after 20 steps and the contact forces are the same bits.  packed: up to
    ~30 contacts per sphere (several rounds of kCoopSlots); packed_cells:
    Verlet lists over capacity (the cell search, searched again per round);
    hopper_bed: a settled bed against the cone's triangles and the floor."""
    from metakonga_gb300 import prepare
    extra = {}
    if case == "hopper_bed":
        sc = scenes.hopper(n=6000, seed=12, gate=True)
        prepare.settle(sc, 3000, dt=4e-5)
        prepare.open_gates(sc)
    else:
        sc = _packed()
        if case == "packed_cells":
            extra = {"verlet_cap": 8}
    out = []
    for mode in (0, 1):
        d = engine.DeviceScene(sc, mode=engine.MODE_MIXED, tuning=dict(extra, contact_mode=mode))
        d.step(20, check=True)
        st = d.download()
        f, m = d.eval_contacts()
        stats = d.stats()
        d.close()
        out.append((st, f, m, stats))
    (s0, f0, m0, t0), (s1, f1, m1, t1) = out
    assert np.abs(f0).max() > 0
    for k in ("pos", "vel", "omega"):
        assert np.array_equal(s0[k], s1[k]), k
    assert np.array_equal(f0, f1) and np.array_equal(m0, m1)
    if case == "packed_cells":
        assert t1["verlet_overflows"] > 0

