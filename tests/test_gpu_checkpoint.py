"""Checkpoint and resume on the GPU: the FP64 form continues bit for bit."""
import numpy as np
import pytest

from metakonga_gb300 import engine, results

from .cases import packed_scene

pytestmark = pytest.mark.gpu


def test_fp64_resume_is_bit_exact(cuda, tmp_path):
    sc = packed_scene(n_side=8)
    a = engine.DeviceScene(sc, mode=engine.MODE_FP64)
    a.step(30)
    straight = a.download()
    a.close()

    b = engine.DeviceScene(packed_scene(n_side=8), mode=engine.MODE_FP64)
    b.step(12)
    path = str(tmp_path / "state.ckpt")
    results.write_checkpoint(path, 12 * 1e-5, b.download(), sc.mass, sc.inertia)
    b.close()
    c, ct = results.resume(packed_scene(n_side=8), path, engine.MODE_FP64)
    c.step(18)
    resumed = c.download()
    c.close()
    for k in ("pos", "vel", "acc", "omega", "alpha"):
        assert np.array_equal(straight[k], resumed[k]), k


def test_mixed_resume_tracks_the_straight_run(cuda, tmp_path):
    """The mixed form re-bins after a resume, so pairs may be summed in another
    order; the state stays within FP32 rounding of the uninterrupted run."""
    sc = packed_scene(n_side=8)
    a = engine.DeviceScene(sc, mode=engine.MODE_MIXED)
    a.step(30)
    straight = a.download()
    a.close()
    b = engine.DeviceScene(packed_scene(n_side=8), mode=engine.MODE_MIXED)
    b.step(12)
    path = str(tmp_path / "state.ckpt")
    results.write_checkpoint(path, 0.0, b.download(), sc.mass, sc.inertia)
    b.close()
    c, _ = results.resume(packed_scene(n_side=8), path, engine.MODE_MIXED)
    c.step(18)
    resumed = c.download()
    c.close()
    assert np.abs(straight["pos"] - resumed["pos"]).max() < 1e-10
    vscale = np.abs(straight["vel"]).max()
    assert np.abs(straight["vel"] - resumed["vel"]).max() < 1e-4 * vscale
