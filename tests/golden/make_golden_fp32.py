"""Generate the single-precision golden fixtures from the reference's own
float kernels.

    make -C oracle ref && python tests/golden/make_golden_fp32.py

The reference's float kernels (include/mphysics_cuda_impl.cuh:1094-1895,
compiled as host code into oracle/_ref/libxdref.so) run the float step in the
reference's order on seeded inputs converted to single precision
(tests/cases.py:to_single).  Each step records the cell hash and sorted index,
the occupied cells' ranges, the contact force and moment before the velocity
update, and the state after it; the drum case also records the body reaction.
The cube fixture applies the six planes of the packed case's box as one
cube_contact_force call.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.pyoracle import RefKernels  # noqa: E402
from tests.cases import packed_scene, small_drum, to_single  # noqa: E402

STATE = ("pos", "vel", "acc", "omega", "alpha", "force", "moment", "mass", "inertia")
RECORDS = ("params_f", "hash_grid", "cp_pp", "planes", "cp_planes", "poly", "pmi", "cp_poly")


def _bytes(rec):
    """A record array as bytes with zeroed padding (field-wise copy)."""
    rec = np.asarray(rec).reshape(-1)
    out = np.zeros(rec.shape[0], dtype=rec.dtype)
    for name in rec.dtype.names:
        out[name] = rec[name]
    return out.view(np.uint8)


def _step_f(ref, S):
    """One float step in the reference's order (dem_simulation.cpp:447-469)."""
    ref.vv_position_f(S["pos"], S["vel"], S["acc"])
    h, ix, cs, ce, so = ref.detection_f(S["params_f"], S["pos"], S.get("sphere"))
    ref.p2p_f(S["pos"], S["vel"], S["omega"], S["force"], S["moment"], S["mass"], so, cs, ce,
              S["cp_pp"])
    for i in range(S["planes"].shape[0]):
        ref.plane_f(S["planes"][i:i + 1], S["pos"], S["vel"], S["omega"], S["force"], S["moment"],
                    S["mass"], S["cp_planes"][i:i + 1])
    if "poly" in S:
        ref.polygon_f(S["poly"], S["sphere"], S["pmi"], S["pos"], S["vel"], S["omega"], S["force"],
                      S["moment"], S["mass"], so, cs, ce, S["cp_poly"])
    f, m = S["force"].copy(), S["moment"].copy()
    ref.vv_velocity_f(S["vel"], S["acc"], S["omega"], S["alpha"], S["force"], S["moment"],
                      S["mass"], S["inertia"])
    occ = np.flatnonzero(cs != 0xFFFFFFFF).astype(np.uint32)
    return {"hash": h, "sorted": so, "cells": occ, "cstart": cs[occ], "cend": ce[occ],
            "contact_force": f, "contact_moment": m}


def _save(name, S0, steps, ref):
    S = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in S0.items()}
    ref.set_params_f(S["params_f"], S["hash_grid"])
    d = {"steps": np.array(steps)}
    for k in STATE:
        d["in_" + k] = S0[k]
    if "sphere" in S0:
        d["sphere"] = S0["sphere"]
    for k in RECORDS:
        if k in S0:
            d[k] = _bytes(S0[k])
    for t in range(steps):
        out = _step_f(ref, S)
        for k, v in out.items():
            d[f"s{t}_{k}"] = v
        for k in STATE:
            d[f"s{t}_{k}"] = S[k].copy()
        if "pmi" in S:
            d[f"s{t}_pmi"] = _bytes(S["pmi"])
    np.savez_compressed(os.path.join(HERE, name), **d)


def _save_cube(name, S0, ref):
    S = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in S0.items()}
    ref.set_params_f(S["params_f"], S["hash_grid"])
    planes6 = np.ascontiguousarray(S["planes"][:6])
    ref.cube_f(planes6, S["pos"], S["vel"], S["omega"], S["force"], S["moment"], S["mass"],
               S["cp_pp"])
    d = {k: S0[k] for k in ("pos", "vel", "omega", "force", "moment", "mass")}
    d["planes6"] = _bytes(planes6)
    d["cp"] = _bytes(S0["cp_pp"])
    d["params_f"] = _bytes(S0["params_f"])
    d["out_force"], d["out_moment"] = S["force"], S["moment"]
    np.savez_compressed(os.path.join(HERE, name), **d)


def main():
    ref = RefKernels()
    packed = to_single(packed_scene(n_side=8))
    assert packed["planes"].shape[0] == 6
    _save("f32_packed_512_walls.npz", packed, 2, ref)
    _save_cube("f32_cube_512.npz", packed, ref)
    _save("f32_drum_600_mesh.npz", to_single(small_drum()), 1, ref)


if __name__ == "__main__":
    main()
