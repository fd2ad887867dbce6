"""Batched and served scenes: every result equals the scene stepped alone.

Scenes of different kinds and sizes (a packed lattice with walls, a hopper of
triangles over a floor, a polydisperse cloud) are advanced together by
xd_scene_step_many and by the continuous-batching server; each scene's state
must be bit for bit the one a lone xd_scene_step call of the same step count
gives, in both the mixed and the FP64 form."""
import numpy as np
import pytest

from metakonga_gb300 import engine, scenes, serve

from .cases import packed_scene

pytestmark = pytest.mark.gpu

_KEYS = ("pos", "vel", "acc", "omega", "alpha")


def _mix():
    out = [packed_scene(n_side=8),
           scenes.hopper(n=1500, seed=5, orifice=7.0, fric=0.3),
           scenes.polydisperse_box(n=4000, seed=9)]
    rng = np.random.Generator(np.random.MT19937(17))
    for sc in out[1:]:
        sc.vel[:] = rng.normal(0.0, 0.5, sc.vel.shape)
    return out


def _alone(sc, nsteps, mode):
    ds = engine.DeviceScene(sc, mode=mode)
    ds.step(nsteps, check=True)
    st = ds.download()
    ds.close()
    return st


def _same(a, b):
    for k in _KEYS:
        assert np.array_equal(a[k], b[k]), k


@pytest.mark.parametrize("mode", [engine.MODE_MIXED, engine.MODE_FP64])
def test_step_many_equals_each_scene_alone(cuda, mode):
    mix = _mix()
    counts = [5, 9, 2]
    ref = [_alone(sc, c, mode) for sc, c in zip(mix, counts)]
    ds = [engine.DeviceScene(sc, mode=mode) for sc in mix]
    engine.step_many(ds, counts, check=True)
    for d, r in zip(ds, ref):
        _same(d.download(), r)
        d.close()


def test_step_many_in_chunks_equals_one_call(cuda):
    """Steps split over several batched calls give the single call's state."""
    mix = _mix()
    ref = [_alone(sc, 12, engine.MODE_MIXED) for sc in mix]
    ds = [engine.DeviceScene(sc, mode=engine.MODE_MIXED) for sc in mix]
    for c in (5, 4, 3):
        engine.step_many(ds, c, check=True)
    for d, r in zip(ds, ref):
        _same(d.download(), r)
        d.close()


@pytest.mark.parametrize("batch", [False, True, "cohorts"])
def test_served_results_equal_alone(cuda, batch):
    """Served side by side (step_many), as batches of the resident set, or as
    cohorts (finished members riding along in their cohort's batch): the
    results are the scenes' own."""
    mix = _mix()
    steps = [23, 17, 30]
    ref = [_alone(sc, s, engine.MODE_MIXED) for sc, s in zip(mix, steps)]
    srv = serve.Server(budget_bytes=1 << 34, chunk=7, batch=batch is True, cohorts=batch == "cohorts")
    for k, (sc, s) in enumerate(zip(mix, steps)):
        srv.submit(k, sc, s, arrival=0.0)
    done = srv.run()
    assert sorted(r.rid for r in done) == [0, 1, 2]
    for r in done:
        _same(r.result, ref[r.rid])
    rep = srv.report()
    assert rep["requests"] == 3 and rep["p99_ms"] >= rep["p50_ms"] > 0
    assert rep["peak_active"] == 3
    assert (rep["batched_ticks"] > 0) == bool(batch)


def test_memory_estimate_bounds_the_allocation(cuda):
    for sc in _mix():
        for mode in (engine.MODE_MIXED, engine.MODE_FP64):
            ds = engine.DeviceScene(sc, mode=mode)
            got = ds.device_bytes()
            ds.close()
            est = serve.estimate_device_bytes(sc, mode)
            assert got > 0
            assert got <= est <= 3 * got + (8 << 20), (sc.name, mode, got, est)


def test_budget_holds_requests_back(cuda):
    """With room for one scene at a time, requests run one after another and
    the results are still those of the scenes alone."""
    mix = _mix()[:2]
    ref = [_alone(sc, 6, engine.MODE_MIXED) for sc in mix]
    budget = max(serve.estimate_device_bytes(sc) for sc in mix)
    srv = serve.Server(budget_bytes=budget, chunk=4)
    for k, sc in enumerate(mix):
        srv.submit(k, sc, 6, arrival=0.0)
    done = srv.run()
    assert [r.rid for r in done] == [0, 1]
    assert srv.report()["peak_active"] == 1
    assert done[1].admitted >= done[0].done
    for r in done:
        _same(r.result, ref[r.rid])
