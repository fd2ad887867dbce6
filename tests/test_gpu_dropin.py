"""Drop-in check of the C++ boundary: a program written against the
reference's own API names (tests/cpp/reference_step.cpp), linked with
libxdem_mphysics.so, runs whole steps that match the oracle."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from .cases import packed_scene

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
PKG = os.path.join(ROOT, "metakonga_gb300")


def _cuda_root():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return os.path.dirname(os.path.dirname(nvcc))


def test_reference_api_program_matches_oracle(cuda, oracle, tmp_path):
    exe = tmp_path / "reference_step"
    cr = _cuda_root()
    subprocess.run(["g++", "-O2", "-std=c++17", os.path.join(HERE, "cpp", "reference_step.cpp"),
                    "-I", os.path.join(ROOT, "include"), "-I", os.path.join(cr, "include"),
                    "-L", PKG, "-lxdem_mphysics", "-lxdem", "-L", os.path.join(cr, "lib64"),
                    "-lcudart", "-Wl,-rpath," + PKG, "-Wl,-rpath," + os.path.join(cr, "lib64"),
                    "-o", str(exe)], check=True)
    sc = packed_scene(n_side=9)
    nsteps = 6
    p = sc.params.copy()
    p["np"] = sc.np_
    with open(tmp_path / "in.bin", "wb") as f:
        f.write(np.array([sc.np_, sc.planes.shape[0], nsteps], np.uint32).tobytes())
        f.write(p.tobytes())
        f.write(sc.cp_pp.tobytes())
        for i in range(sc.planes.shape[0]):
            f.write(sc.planes[i].tobytes())
            f.write(sc.cp_planes[i].tobytes())
        for k in ("pos", "vel", "acc", "omega", "alpha", "force", "moment", "mass", "inertia"):
            f.write(np.ascontiguousarray(getattr(sc, k)).tobytes())
    r = subprocess.run([str(exe), str(tmp_path / "in.bin"), str(tmp_path / "out.bin")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    buf = open(tmp_path / "out.bin", "rb").read()
    n = sc.np_
    off = 4
    out = {}
    for k, w in (("pos", 4), ("vel", 3), ("acc", 3), ("omega", 3), ("alpha", 3)):
        out[k] = np.frombuffer(buf, np.float64, n * w, off).reshape(n, w)
        off += 8 * n * w
    sorted_ids = np.frombuffer(buf, np.uint32, n, off)
    ref = sc.copy()
    work = oracle.run(ref, nsteps)
    assert np.array_equal(sorted_ids, work["sorted"])
    assert np.abs(out["pos"] - ref.pos).max() <= 1e-13 * np.abs(ref.pos).max()
    assert np.abs(out["vel"] - ref.vel).max() <= 1e-9 * np.abs(ref.vel).max()
