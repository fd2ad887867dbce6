"""Generate the legacy-interface golden fixtures from the reference's own
legacy kernels.

    make -C oracle ref && python tests/golden/make_golden_legacy.py

The reference's legacy kernels (include/cu_dem_impl.cuh, compiled as host code
into oracle/_ref/libxdref_legacy.so) run on seeded inputs in the legacy layouts
(tests/cases.py:to_legacy):
  legacy_packed_512_cube.npz  two steps of a packed lattice in a box of six
      planes: VV position, hash (sorting), cell ranges, force and moment
      zeroed, particle-particle, cube, VV velocity;
  legacy_drum_600_shape.npz   the small drum's particles against its mesh as
      an indexed shape: mesh placement (cu_update_polygons_position, then
      cu_update_polygons_information) under a rotation, vertices merged into
      the grid after the particles, hash, cell ranges and the shape contact
      (face, then edge or vertex contacts) with its force sum.
"""
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from metakonga_gb300.layouts import LEGACY_MASS_INFO, LEGACY_POLYGON  # noqa: E402
from oracle.pyoracle import LegacyRefKernels  # noqa: E402
from tests.cases import legacy_mesh, legacy_planes, packed_scene, small_drum, to_legacy  # noqa: E402


def _bytes(rec):
    rec = np.asarray(rec).reshape(-1)
    out = np.zeros(rec.shape[0], dtype=rec.dtype)
    for name in rec.dtype.names:
        out[name] = rec[name]
    return out.view(np.uint8)


def packed(ref):
    sc = packed_scene(n_side=8)
    L = to_legacy(sc)
    planes = legacy_planes(sc.planes)
    assert planes.shape[0] == 6
    n = sc.np_
    nc = int(L["params"]["ncell"])
    ref.set_params(L["params"])
    d = {"params": _bytes(L["params"]), "planes": _bytes(planes), "wall": np.array(L["wall"]), "steps": np.array(2)}
    for k in ("pos", "vel", "acc", "omega", "alpha"):
        d["in_" + k] = L[k].copy()
    S = {k: L[k].copy() for k in ("pos", "vel", "acc", "omega", "alpha", "force", "moment")}
    cend = np.zeros(nc, np.uint32)
    line = np.zeros(n, np.bool_)
    for t in range(2):
        ref.vv_position(S["pos"], S["vel"], S["acc"], n)
        h = np.zeros(n, np.uint32)
        ix = np.zeros(n, np.uint32)
        ref.hash_and_index(h, ix, S["pos"], n)
        cs = np.zeros(nc, np.uint32)
        so = np.zeros(n, np.uint32)
        ref.reorder(h, ix, cs, cend, so, n, nc)
        S["force"][:] = 0
        S["moment"][:] = 0
        ref.p2p(S["pos"], S["vel"], S["acc"], S["omega"], S["alpha"], S["force"], S["moment"], so, cs, cend, n)
        d[f"s{t}_p2p_force"] = S["force"].copy()
        d[f"s{t}_p2p_moment"] = S["moment"].copy()
        kn, vn, ks, vs, mu = L["wall"]
        ref.cube(planes, kn, vn, ks, vs, mu, line, S["pos"], S["vel"], S["omega"], S["force"], S["moment"], n)
        d[f"s{t}_force"] = S["force"].copy()
        d[f"s{t}_moment"] = S["moment"].copy()
        ref.vv_velocity(S["vel"], S["acc"], S["omega"], S["alpha"], S["force"], S["moment"], n)
        occ = np.flatnonzero(cs != 0xFFFFFFFF).astype(np.uint32)
        d[f"s{t}_hash"], d[f"s{t}_sorted"] = h, so
        d[f"s{t}_cells"], d[f"s{t}_cstart"], d[f"s{t}_cend"] = occ, cs[occ], cend[occ]
        for k in ("pos", "vel", "acc", "omega", "alpha"):
            d[f"s{t}_{k}"] = S[k].copy()
    np.savez_compressed(os.path.join(HERE, "legacy_packed_512_cube.npz"), **d)


def drum(ref):
    sc = small_drum()
    n = sc.np_
    tri = sc.vlist.reshape(-1, 3, 3)
    verts, indice, id_set, pstart, pend = legacy_mesh(tri)
    nv = verts.shape[0]
    L = to_legacy(sc, nsp=nv, cell_size=2.0 * float(sc.pos[:, 3].max()))
    nc = int(L["params"]["ncell"])
    ref.set_params(L["params"])
    # place the mesh: a small rotation about y and a shift
    th = math.radians(2.0)
    A = np.array([[math.cos(th), 0.0, math.sin(th)], [0.0, 1.0, 0.0], [-math.sin(th), 0.0, math.cos(th)]])
    mpos = np.array([0.0005, -0.0002, 0.0003])
    world = np.zeros((nv, 3))
    ref.update_polygons_position(mpos, np.ascontiguousarray(A.reshape(-1)), verts, world)
    polygons = np.zeros(indice.shape[0], dtype=LEGACY_POLYGON)
    ref.update_polygons_information(polygons, indice, world)
    data = np.zeros((n + nv, 4))
    ref.mergedata(data, L["pos"], n, world, nv)
    h = np.zeros(n + nv, np.uint32)
    ix = np.zeros(n + nv, np.uint32)
    ref.hash_and_index(h, ix, data, n + nv)
    cs = np.zeros(nc, np.uint32)
    ce = np.zeros(nc, np.uint32)
    so = np.zeros(n + nv, np.uint32)
    ref.reorder(h, ix, cs, ce, so, n + nv, nc)
    minfo = np.zeros(1, dtype=LEGACY_MASS_INFO)
    minfo["vel"] = (0.01, -0.02, 0.005)
    line = np.zeros(n, np.bool_)
    force = np.zeros((n, 3))
    moment = np.zeros((n, 3))
    kn, vn, ks, vs, mu = L["wall"]
    total = ref.shape(minfo, polygons, id_set, pstart, pend, kn, vn, ks, vs, mu, line, L["pos"], L["vel"],
                      L["omega"], force, moment, n, so, cs, ce)
    occ = np.flatnonzero(cs != 0xFFFFFFFF).astype(np.uint32)
    d = {"params": _bytes(L["params"]), "wall": np.array(L["wall"]), "verts": verts, "indice": indice,
         "id_set": id_set, "poly_start": pstart, "poly_end": pend, "A": A.reshape(-1), "mpos": mpos,
         "minfo": _bytes(minfo), "pos": L["pos"], "vel": L["vel"], "omega": L["omega"],
         "out_world": world, "out_polygons": _bytes(polygons), "out_data": data, "out_hash": h,
         "out_sorted": so, "out_cells": occ, "out_cstart": cs[occ], "out_cend": ce[occ], "out_force": force,
         "out_moment": moment, "out_line": line, "out_total": total}
    assert line.sum() > 20, "case has few shape contacts"
    np.savez_compressed(os.path.join(HERE, "legacy_drum_600_shape.npz"), **d)


def main():
    ref = LegacyRefKernels()
    packed(ref)
    drum(ref)


if __name__ == "__main__":
    main()
