"""Batches (xd_batch_*, engine.Batch): scenes advanced together by shared
launches give, scene by scene, the same bits as each scene stepped alone --
particle state, re-binnings and the body reactions -- across calls of any
length, with re-binnings inside the calls, and after a scene's walls move
(the batch captures itself again)."""
import numpy as np
import pytest

from metakonga_gb300 import engine, scenes

from .cases import packed_scene, small_drum, small_hopper

pytestmark = pytest.mark.gpu


def _scenes():
    rng = np.random.Generator(np.random.MT19937(41))
    out = [small_hopper(n=1500, seed=5), scenes.hopper(n=900, seed=8), scenes.hopper(n=3000, seed=9),
           packed_scene(n_side=6), small_drum(n=400, seed=6)]
    for sc in out:
        # fast enough that every scene re-bins within the calls
        sc.vel[:] += rng.normal(0.0, 1.5, sc.vel.shape)
    return out


def _run(split, batched, moved=None, timed=False, tuning=None):
    scs = _scenes()
    ds = [engine.DeviceScene(sc, mode=engine.MODE_MIXED, tuning=tuning) for sc in scs]
    b = engine.Batch(ds) if batched else None
    if timed:
        b.set_timing(True)
    for c, k in enumerate(split):
        if moved is not None and c == 1:
            planes = scs[3].planes.copy()
            planes[0]["xw"][2] += 2e-4
            for f in ("w2", "w3", "w4"):
                planes[0][f][2] += 2e-4
            ds[3].set_planes(planes)
        if batched:
            b.step(k, check=True)
        else:
            for d in ds:
                d.step(k, check=True)
    out = [(d.download(), d.rebuilds()[0], d.get_bodies() if d.ntri else None) for d in ds]
    if timed:
        kt = b.kernel_times()
        steps = sum(split)
        assert kt["advance"][1] == steps - len(split) and kt["contact"][1] == steps
        assert kt["advance"][0] > 0 and kt["contact"][0] > 0
        # the scenes have walls: the cooperative pair pass (the default) is
        # followed by a wall pass every step
        assert kt["walls"][1] == steps and kt["walls"][0] > 0
    if b:
        b.close()
    for d in ds:
        d.close()
    return out


@pytest.mark.parametrize("moved,timed", [(None, False), (True, False), (None, True)])
def test_batch_equals_each_scene_alone(cuda, moved, timed):
    """timed: the batch's direct launches with kernel events (the same
    kernels as its step graphs)."""
    alone = _run((5, 27, 16), False, moved)
    batch = _run((5, 27, 16), True, moved, timed)
    assert all(r > 1 for _, r, _ in alone), [r for _, r, _ in alone]
    for (a, ra, ba), (b, rb, bb) in zip(alone, batch):
        assert ra == rb
        for k in ("pos", "vel", "omega", "acc"):
            assert np.array_equal(a[k], b[k]), k
        if ba is not None:
            assert ba.tobytes() == bb.tobytes()


def test_batch_equals_each_scene_alone_per_particle_pass(cuda):
    """The per-particle pair pass (contact_mode 0), batched and alone."""
    t = {"contact_mode": 0}
    alone = _run((5, 27, 16), False, tuning=t)
    batch = _run((5, 27, 16), True, tuning=t)
    for (a, ra, ba), (b, rb, bb) in zip(alone, batch):
        assert ra == rb
        for k in ("pos", "vel", "omega", "acc"):
            assert np.array_equal(a[k], b[k]), k
        if ba is not None:
            assert ba.tobytes() == bb.tobytes()


def test_batch_refuses_scenes_changed_after_creation(cuda):
    """A scene given history, kinematic bodies or an emitter after the batch
    was made: the batch's next step fails instead of ignoring the change."""
    for change in ("history", "kinematic", "emitter"):
        sc = small_drum(n=200, seed=3)
        ds = [engine.DeviceScene(sc, mode=engine.MODE_MIXED), engine.DeviceScene(packed_scene(n_side=4),
                                                                               mode=engine.MODE_MIXED)]
        b = engine.Batch(ds)
        b.step(2, check=True)
        if change == "history":
            ds[0].set_tangential_history(4)
        elif change == "kinematic":
            ds[0].set_kinematic_bodies(True)
        else:
            ds[0].set_emitter(10, [50, 50], active=100)
        with pytest.raises(Exception):
            b.step(2, check=True)
        b.close()
        for d in ds:
            d.close()


def test_batch_refuses_history_and_plain_scenes(cuda):
    sc = packed_scene(n_side=4)
    d1 = engine.DeviceScene(sc, mode=engine.MODE_MIXED)
    d2 = engine.DeviceScene(sc, mode=engine.MODE_FP64)
    d1.set_tangential_history(4)
    for group in ([d1], [d2]):
        with pytest.raises(Exception):
            engine.Batch(group)
    d1.close()
    d2.close()


def test_async_copies_round_trip(cuda):
    """xd_scene_upload_async / xd_scene_download_async: queued on the stream,
    the same data as the waiting copies once the stream is synchronised."""
    import torch

    from metakonga_gb300._lib import call
    sc = small_hopper(n=1500, seed=5)
    d = engine.DeviceScene(sc, mode=engine.MODE_MIXED)
    d.step(3, check=True)
    ref = d.download()
    keys = ("pos", "vel", "acc", "omega", "alpha")
    host = {k: torch.from_numpy(np.ascontiguousarray(ref[k])).pin_memory() for k in keys}
    for k in ("force", "moment", "mass", "inertia"):
        host[k] = torch.from_numpy(np.ascontiguousarray(getattr(sc, k))).pin_memory()
    out = {k: torch.empty_like(host[k]).pin_memory() for k in keys}
    stream = torch.cuda.Stream()
    call("xd_scene_upload_async", d.handle, *[host[k].data_ptr() for k in
                                              ("pos", "vel", "acc", "omega", "alpha", "force", "moment",
                                               "mass", "inertia")], stream.cuda_stream)
    call("xd_scene_download_async", d.handle, *[out[k].data_ptr() for k in keys], None, None, stream.cuda_stream)
    stream.synchronize()
    for k in keys:
        assert np.array_equal(out[k].numpy(), ref[k]), k
    d.close()


def test_state_copies_from_one_block(cuda):
    """Arrays kept back to back in the library's staging order (pos, vel, acc,
    omega, alpha, mass, inertia) go as one copy each way; the state is the
    same as with separate arrays."""
    import torch

    from metakonga_gb300._lib import call
    sc = small_hopper(n=1500, seed=5)
    d = engine.DeviceScene(sc, mode=engine.MODE_MIXED)
    d.step(4, check=True)
    ref = d.download()
    n = sc.np_
    block = torch.empty(18 * n, dtype=torch.float64).pin_memory()
    views, off = {}, 0
    for k, w in (("pos", 4), ("vel", 3), ("acc", 3), ("omega", 3), ("alpha", 3), ("mass", 1), ("inertia", 1)):
        views[k] = block[off:off + w * n]
        src = ref[k] if k in ref else getattr(sc, k)
        views[k].copy_(torch.from_numpy(np.ascontiguousarray(src).reshape(-1)))
        off += w * n
    force = torch.from_numpy(np.ascontiguousarray(sc.force)).pin_memory()
    moment = torch.from_numpy(np.ascontiguousarray(sc.moment)).pin_memory()
    stream = torch.cuda.Stream()
    call("xd_scene_upload_async", d.handle, views["pos"].data_ptr(), views["vel"].data_ptr(), views["acc"].data_ptr(),
         views["omega"].data_ptr(), views["alpha"].data_ptr(), force.data_ptr(), moment.data_ptr(),
         views["mass"].data_ptr(), views["inertia"].data_ptr(), stream.cuda_stream)
    out = torch.zeros(16 * n, dtype=torch.float64).pin_memory()
    o = {}
    off = 0
    for k, w in (("pos", 4), ("vel", 3), ("acc", 3), ("omega", 3), ("alpha", 3)):
        o[k] = out[off:off + w * n]
        off += w * n
    call("xd_scene_download_async", d.handle, *[o[k].data_ptr() for k in ("pos", "vel", "acc", "omega", "alpha")],
         None, None, stream.cuda_stream)
    stream.synchronize()
    for k in o:
        assert np.array_equal(o[k].numpy(), np.ascontiguousarray(ref[k]).reshape(-1)), k
    d.close()
