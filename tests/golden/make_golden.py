"""Generate the golden fixtures from the reference's own kernels.

    make -C oracle ref && python tests/golden/make_golden.py

The reference publishes no tests or golden vectors, so the fixtures are made
by running the reference's FP64 kernels (include/mphysics_cuda_impl.cuh,
compiled as host code into oracle/_ref/libxdref.so by oracle/Makefile) on
seeded inputs.  Each .npz holds the inputs, the number of steps, and the
reference's outputs: the full state after the steps, the sorted grid arrays
and the occupied cells' ranges (cell, start, end).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.pyoracle import RefKernels  # noqa: E402
from tests.cases import packed_scene, small_drum  # noqa: E402

STATE = ("pos", "vel", "acc", "omega", "alpha", "force", "moment", "mass", "inertia")


def _save(name, sc, steps, ref):
    init = sc.copy()
    out = sc.copy()
    grid = None
    for _ in range(steps):
        grid = ref.step(out)
    h, ix, cs, ce, so = grid
    occ = np.flatnonzero(cs != 0xFFFFFFFF).astype(np.uint32)
    d = {"steps": np.array(steps)}
    for k in STATE:
        d["in_" + k] = getattr(init, k)
        d["out_" + k] = getattr(out, k)
    d["params"] = init.params.reshape(1).view(np.uint8)
    d["cp_pp"] = init.cp_pp.reshape(1).view(np.uint8)
    d["planes"] = init.planes.view(np.uint8)
    d["cp_planes"] = init.cp_planes.view(np.uint8)
    if init.ntri:
        d["poly"] = init.poly.view(np.uint8)
        d["sphere"] = init.sphere
        d["vlist"] = init.vlist
        d["pmi"] = init.pmi.view(np.uint8)
        d["cp_poly"] = init.cp_poly.view(np.uint8)
        d["out_pmi"] = out.pmi.view(np.uint8)
    d["out_hash"], d["out_sorted"] = h, so
    d["out_cells"] = occ
    d["out_cstart"], d["out_cend"] = cs[occ], ce[occ]
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **d)
    print(f"{path}: {sc.np_} spheres, {sc.ntri} triangles, {steps} steps, {occ.size} cells")


def main():
    ref = RefKernels()
    sc = packed_scene(n_side=6)
    sc.params["grid"] = (32, 32, 32)
    sc.params["ncell"] = 32 ** 3
    _save("packed_216_walls", sc, 3, ref)
    dr = small_drum(n=160)
    dr.params["grid"] = (32, 32, 32)
    dr.params["ncell"] = 32 ** 3
    _save("drum_160_mesh", dr, 3, ref)


if __name__ == "__main__":
    main()
