"""Host logic of the serving loop, with the device calls replaced by fakes:
first-come-first-served admission under the memory budget, continuous
batching (late arrivals join running scenes), chunked step counts, the
latency report, and the memory estimate's growth with the scene."""
import numpy as np
import pytest

from metakonga_gb300 import engine, scenes, serve

from .cases import packed_scene


class _FakeScene:
    live = 0
    batches = []

    def __init__(self, sc, mode=engine.MODE_MIXED):
        if getattr(sc, "refuse", False):
            raise RuntimeError("scene refused")
        self.sc = sc
        self.steps = 0
        _FakeScene.live += 1

    def download(self, stream=0):
        out = {"steps": self.steps}
        if getattr(self.sc, "blow_up", False):
            out["pos"] = np.array([[0.0, float("nan"), 0.0, 1.0]])
        return out

    def download_async(self, stream=0):
        # the copy is queued in stream order: it sees the steps issued so far
        snap = self.download(stream)
        return lambda: snap

    def close(self):
        # a scene is never freed while a batch holding it is alive
        assert not any(self in b.handles for b in _FakeScene.batches if not b.closed)
        _FakeScene.live -= 1


class _Marks:
    """Tick marks for the fake device: nothing to wait for."""

    def mark(self):
        return None

    def wait(self, mark):
        pass

    def side_after(self, mark):
        return 0


class _Clock:
    """Deterministic clock: each tick of the fake batch advances 1 ms."""

    def __init__(self):
        self.t = 0.0

    def __call__(self):
        return self.t


@pytest.fixture
def fake(monkeypatch):
    clock = _Clock()
    calls = []

    def step_many(handles, counts, check=False, stream=0):
        calls.append([(h.sc.name, c) for h, c in zip(handles, counts)])
        for h, c in zip(handles, counts):
            h.steps += c
        clock.t += 1e-3

    class _FakeBatch:
        def __init__(self, handles):
            self.handles = list(handles)
            self.closed = False
            _FakeScene.batches.append(self)

        def step(self, k, check=False, stream=0):
            assert not self.closed
            step_many(self.handles, [k] * len(self.handles))

        def close(self):
            self.closed = True

    monkeypatch.setattr(engine, "DeviceScene", _FakeScene)
    monkeypatch.setattr(engine, "step_many", step_many)
    monkeypatch.setattr(engine, "Batch", _FakeBatch)
    _FakeScene.batches = []
    monkeypatch.setattr(serve.time, "sleep", lambda s: setattr(clock, "t", clock.t + max(s, 0.0)))
    _FakeScene.live = 0
    return clock, calls


def _named(name, n_side=4):
    sc = packed_scene(n_side=n_side)
    sc.name = name
    return sc


def test_chunks_and_results(fake):
    clock, calls = fake
    srv = serve.Server(budget_bytes=1 << 40, chunk=4, clock=clock, marks=_Marks(), depth=0)
    srv.submit("a", _named("a"), 10)
    srv.submit("b", _named("b"), 3)
    done = srv.run()
    assert [r.rid for r in done] == ["b", "a"]
    assert calls[0] == [("a", 4), ("b", 3)]
    assert calls[1] == [("a", 4)] and calls[2] == [("a", 2)]
    assert all(r.result["steps"] == r.steps for r in done)
    assert _FakeScene.live == 0 and srv.used == 0


def test_late_arrival_joins_running_batch(fake):
    clock, calls = fake
    srv = serve.Server(budget_bytes=1 << 40, chunk=2, clock=clock, marks=_Marks(), depth=0)
    srv.submit("a", _named("a"), 20, arrival=0.0)
    srv.submit("b", _named("b"), 4, arrival=0.0035)
    done = srv.run()
    # b arrives during a's fourth tick and runs beside a from the fifth
    assert calls[3] == [("a", 2)]
    assert calls[4] == [("a", 2), ("b", 2)]
    assert [r.rid for r in done] == ["b", "a"]
    rep = srv.report()
    assert rep["peak_active"] == 2
    b = done[0]
    assert b.admitted == pytest.approx(0.004)
    assert b.done - b.arrival == pytest.approx(0.0025)


def test_pipelined_ticks_retire_depth_ticks_later(fake):
    """With two ticks queued, a finished request is retired (downloaded) when
    two more ticks have been issued; the issued ticks are the same."""
    clock, calls = fake
    srv = serve.Server(budget_bytes=1 << 40, chunk=2, clock=clock, marks=_Marks(), depth=2)
    srv.submit("a", _named("a"), 20, arrival=0.0)
    srv.submit("b", _named("b"), 4, arrival=0.0035)
    done = srv.run()
    assert calls[4] == [("a", 2), ("b", 2)] and calls[5] == [("a", 2), ("b", 2)]
    b = [r for r in done if r.rid == "b"][0]
    assert b.done - b.arrival == pytest.approx(0.0045)
    assert all(r.result["steps"] == r.steps for r in done)
    assert _FakeScene.live == 0


def test_budget_is_first_come_first_served(fake):
    clock, calls = fake
    big, small = _named("big", 6), _named("s2", 3)
    eb, es = serve.estimate_device_bytes(big), serve.estimate_device_bytes(small)
    srv = serve.Server(budget_bytes=eb + es - 1, chunk=5, clock=clock, marks=_Marks(), depth=0)
    srv.submit("s1", _named("s1", 3), 5, arrival=0.0)
    srv.submit("big", big, 5, arrival=0.0)
    srv.submit("s2", small, 5, arrival=0.0)
    done = srv.run()
    # big does not fit beside s1, and s2 may not overtake it
    assert calls[0] == [("s1", 5)]
    assert calls[1] == [("big", 5)]
    assert calls[2] == [("s2", 5)]
    assert [r.rid for r in done] == ["s1", "big", "s2"]
    assert srv.peak_used <= srv.budget


def test_oversized_request_runs_alone(fake):
    clock, calls = fake
    srv = serve.Server(budget_bytes=1, chunk=5, clock=clock, marks=_Marks(), depth=0)
    srv.submit("x", _named("x"), 5)
    srv.submit("y", _named("y"), 5)
    done = srv.run()
    assert [r.rid for r in done] == ["x", "y"]
    assert all(len(c) == 1 for c in calls)


def test_idle_server_waits_for_arrivals(fake):
    clock, calls = fake
    srv = serve.Server(budget_bytes=1 << 40, chunk=5, clock=clock, marks=_Marks(), depth=0)
    srv.submit("late", _named("late"), 5, arrival=2.0)
    done = srv.run()
    assert done[0].admitted >= 2.0
    assert srv.report()["p50_wait_ms"] < 1.0


def test_report_percentiles(fake):
    clock, _ = fake
    srv = serve.Server(budget_bytes=1 << 40, chunk=1, clock=clock, marks=_Marks(), depth=0)
    for k in range(10):
        srv.submit(k, _named(str(k)), k + 1)
    srv.run()
    rep = srv.report()
    lat = sorted(r.done - r.arrival for r in srv.finished)
    assert rep["p50_ms"] == pytest.approx(np.percentile(np.array(lat) * 1e3, 50))
    assert rep["p99_ms"] >= rep["p50_ms"]
    assert rep["particle_steps"] == sum(64 * (k + 1) for k in range(10))


def test_estimate_grows_with_the_scene():
    small, large = scenes.hopper(n=2000, seed=1), scenes.hopper(n=20000, seed=1)
    for mode in (engine.MODE_MIXED, engine.MODE_FP64):
        a, b = serve.estimate_device_bytes(small, mode), serve.estimate_device_bytes(large, mode)
        assert 0 < a < b


def test_poisson_arrivals():
    t = serve.poisson_arrivals(20000, rate=50.0, seed=3)
    assert np.all(np.diff(t) > 0)
    assert abs(t[-1] / 20000 - 1 / 50.0) < 1e-3


def test_hopper_batch_ranges():
    b = scenes.hopper_batch(count=256, seed=1)
    ns = np.array([d["n"] for d in b])
    assert len(b) == 256 and ns.min() >= 2000 and ns.max() <= 200000
    assert all(6.0 <= d["orifice"] <= 12.0 and 0.2 <= d["fric"] <= 0.6 for d in b)


def test_hopper_geometry():
    sc = scenes.hopper(n=3000, seed=2)
    tri = sc.vlist.reshape(-1, 3, 3)
    assert tri.shape[0] == 4096
    # facet normals point at the axis, and no sphere starts inside the wall
    nrm = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
    cen = tri.mean(axis=1)
    cen[:, 2] = 0.0
    assert np.all(np.einsum("ij,ij->i", nrm, -cen) > 0)
    u = nrm / np.linalg.norm(nrm, axis=1, keepdims=True)
    d = np.einsum("tj,ij->it", u, sc.pos[:, :3]) - np.einsum("tj,tj->t", u, tri[:, 0])[None, :]
    # the faceted cone is convex: the smallest signed distance to the facet
    # planes is the gap to the wall
    gap = d.min(axis=1) - sc.pos[:, 3]
    assert gap.min() > 0
    from scipy.spatial import cKDTree
    pr = cKDTree(sc.pos[:, :3]).query_pairs(0.008, output_type="ndarray")
    dist = np.linalg.norm(sc.pos[pr[:, 0], :3] - sc.pos[pr[:, 1], :3], axis=1)
    assert np.all(dist >= sc.pos[pr[:, 0], 3] + sc.pos[pr[:, 1], 3])


def test_resident_scenes_step_as_a_batch(fake):
    """Ticks where every resident scene takes the same step count go through
    one batch per resident set (made again when the set changes); uneven
    ticks fall back to step_many; every batch is closed before its scenes."""
    clock, calls = fake
    srv = serve.Server(budget_bytes=1 << 40, chunk=4, clock=clock, marks=_Marks(), depth=0, batch=True)
    srv.submit("a", _named("a"), 12)
    srv.submit("b", _named("b"), 6)
    srv.submit("c", _named("c"), 8, arrival=0.0015)
    done = srv.run()
    assert {r.rid: r.result["steps"] for r in done} == {"a": 12, "b": 6, "c": 8}
    rep = srv.report()
    assert 0 < rep["batched_ticks"] < rep["ticks"]
    assert len(_FakeScene.batches) >= 2 and all(b.closed for b in _FakeScene.batches)
    assert _FakeScene.live == 0
    # the batches held the resident sets of their ticks
    assert {tuple(h.sc.name for h in b.handles) for b in _FakeScene.batches} == {("a", "b"), ("a", "c")}


def test_batching_off_steps_side_by_side(fake):
    clock, calls = fake
    srv = serve.Server(budget_bytes=1 << 40, chunk=4, clock=clock, marks=_Marks(), depth=0)
    srv.submit("a", _named("a"), 8)
    srv.submit("b", _named("b"), 8)
    srv.run()
    assert srv.report()["batched_ticks"] == 0 and not _FakeScene.batches


def test_failed_requests_leave_the_others_alone(fake):
    """A scene the library refuses fails at admission and one whose state
    blows up is reported non-finite; the other requests run to completion."""
    clock, calls = fake
    srv = serve.Server(budget_bytes=1 << 40, chunk=4, clock=clock, marks=_Marks(), depth=0)
    bad, nan, good = _named("bad"), _named("nan"), _named("good")
    bad.refuse = True
    nan.blow_up = True
    srv.submit("bad", bad, 8)
    srv.submit("nan", nan, 8)
    srv.submit("good", good, 8)
    done = srv.run()
    assert {r.rid for r in done} == {"nan", "good"}
    assert [r.rid for r in srv.failed] == ["bad"] and srv.failed[0].error.startswith("admission")
    errs = {r.rid: r.error for r in done}
    assert errs["nan"] == "non-finite state" and errs["good"] is None
    rep = srv.report()
    assert rep["failed_admission"] == 1 and rep["non_finite"] == 1 and rep["requests"] == 2
    assert _FakeScene.live == 0


def test_cohorts_batch_per_admission_wave(fake):
    """Requests admitted together form one cohort stepped as one batch; a
    member that finishes keeps its result (taken in stream order) while it
    rides along, and the batch is made once for the cohort's life."""
    clock, calls = fake
    srv = serve.Server(budget_bytes=1 << 40, chunk=4, clock=clock, marks=_Marks(), depth=0, cohorts=True)
    srv.submit("a", _named("a"), 12)
    srv.submit("b", _named("b"), 6)
    done = srv.run()
    assert {r.rid: r.result["steps"] for r in done} == {"a": 12, "b": 6}
    # ticks of 4, 2 (b ends), 4, 2 (a ends), all through the cohort's batch
    assert [c[0][1] for c in calls] == [4, 2, 4, 2]
    assert all(len(c) == 2 for c in calls)
    rep = srv.report()
    assert rep["batches_made"] == 1 and rep["batched_ticks"] == 4
    assert all(b.closed for b in _FakeScene.batches) and _FakeScene.live == 0 and srv.used == 0


def test_cohorts_waves_and_merging(fake):
    """Late arrivals form cohorts of their own; past max_cohorts the live
    members are merged into one cohort (one new batch)."""
    clock, calls = fake
    srv = serve.Server(budget_bytes=1 << 40, chunk=2, clock=clock, marks=_Marks(), depth=0, cohorts=True,
                       max_cohorts=2)
    for k, t in enumerate((0.0, 0.0, 0.0025, 0.0025, 0.0045, 0.0045)):
        srv.submit(f"r{k}", _named(f"r{k}"), 12, arrival=t)
    done = srv.run()
    assert sorted(r.result["steps"] for r in done) == [12] * 6
    # three waves of two; the third wave pushes the count past 2 and merges
    assert any(len(b.handles) > 2 for b in _FakeScene.batches)
    assert all(b.closed for b in _FakeScene.batches) and _FakeScene.live == 0


def test_cohort_members_free_their_memory_when_needed(fake):
    """A finished member held in a cohort's batch gives its memory back when
    the next request needs it."""
    clock, calls = fake
    one = serve.estimate_device_bytes(_named("a"))
    srv = serve.Server(budget_bytes=int(2.5 * one), chunk=2, clock=clock, marks=_Marks(), depth=0, cohorts=True)
    srv.submit("a", _named("a"), 20)
    srv.submit("b", _named("b"), 2)
    srv.submit("c", _named("c"), 4, arrival=0.0015)
    done = srv.run()
    assert {r.rid: r.result["steps"] for r in done} == {"a": 20, "b": 2, "c": 4}
    assert srv.peak_used <= int(2.5 * one) and _FakeScene.live == 0
