"""Byte layouts of the structs that cross the reference's DEM boundary.

Each numpy dtype has the exact size and field offsets of the matching C struct
in the reference's include/mphysics_cuda_dec.cuh, so one buffer can be handed
to the CUDA library (libxdem), to a caller that was written against the
reference headers, and to the test oracle.

* ``PARAMS``            device_parameters       (mphysics_cuda_dec.cuh:17-30), 112 B
* ``CONTACT_PROPERTY``  device_contact_property (mphysics_cuda_dec.cuh:78-88), 88 B
* ``PLANE``             device_plane_info       (mphysics_cuda_dec.cuh:43-55), 232 B
* ``POLYGON``           device_polygon_info     (mphysics_cuda_dec.cuh:32-41), 152 B
* ``POLYGON_MASS``      device_polygon_mass_info(mphysics_cuda_dec.cuh:57-65), 160 B
  (``ep`` is a CUDA double4, aligned to 16 bytes)

and their single-precision twins (mphysics_cuda_dec.cuh:165-263):

* ``PARAMS_F``            device_parameters_f        64 B
* ``CONTACT_PROPERTY_F``  device_contact_property_f  44 B
* ``PLANE_F``             device_plane_info_f       116 B
* ``POLYGON_F``           device_polygon_info_f      76 B
* ``POLYGON_MASS_F``      device_polygon_mass_info_f 80 B (``ep`` a float4 at offset 16)
"""
import numpy as np

V3 = ("<f8", (3,))

PARAMS = np.dtype({
    "names": ["rolling", "np", "nsphere", "ncell", "grid", "dt", "half2dt", "cell_size",
              "cohesion", "gravity", "world_origin"],
    "formats": ["u1", "<u4", "<u4", "<u4", ("<u4", (3,)), "<f8", "<f8", "<f8", "<f8", V3, V3],
    "offsets": [0, 4, 8, 12, 16, 32, 40, 48, 56, 64, 88],
    "itemsize": 112,
})

CONTACT_PROPERTY = np.dtype({
    "names": ["Ei", "Ej", "pri", "prj", "Gi", "Gj", "rest", "fric", "rfric", "coh", "sratio"],
    "formats": ["<f8"] * 11,
    "offsets": [8 * i for i in range(11)],
    "itemsize": 88,
})

# device_cylinder_info (mphysics_cuda_dec.cuh:67-76): 176 bytes, ep at 144
CYLINDER = np.dtype({
    "names": ["len", "rbase", "rtop", "pbase", "ptop", "origin", "vel", "omega", "ep"],
    "formats": ["<f8", "<f8", "<f8", ("<f8", 3), ("<f8", 3), ("<f8", 3), ("<f8", 3), ("<f8", 3), ("<f8", 4)],
    "offsets": [0, 8, 16, 24, 48, 72, 96, 120, 144],
    "itemsize": 176,
})

PLANE = np.dtype({
    "names": ["l1", "l2", "u1", "u2", "uw", "xw", "pa", "pb", "w2", "w3", "w4"],
    "formats": ["<f8", "<f8"] + [V3] * 9,
    "offsets": [0, 8] + [16 + 24 * i for i in range(9)],
    "itemsize": 232,
})

POLYGON = np.dtype({
    "names": ["id", "P", "Q", "R", "V", "W", "N"],
    "formats": ["<i4"] + [V3] * 6,
    "offsets": [0] + [8 + 24 * i for i in range(6)],
    "itemsize": 152,
})

POLYGON_MASS = np.dtype({
    "names": ["origin", "ep", "vel", "omega", "force", "moment"],
    "formats": [V3, ("<f8", (4,)), V3, V3, V3, V3],
    "offsets": [0, 32, 64, 88, 112, 136],
    "itemsize": 160,
})

assert PARAMS.itemsize == 112 and CONTACT_PROPERTY.itemsize == 88
assert PLANE.itemsize == 232 and POLYGON.itemsize == 152 and POLYGON_MASS.itemsize == 160

F3 = ("<f4", (3,))

PARAMS_F = np.dtype({
    "names": ["np", "nsphere", "ncell", "grid", "dt", "half2dt", "cell_size", "cohesion",
              "gravity", "world_origin"],
    "formats": ["<u4", "<u4", "<u4", ("<u4", (3,)), "<f4", "<f4", "<f4", "<f4", F3, F3],
    "offsets": [0, 4, 8, 12, 24, 28, 32, 36, 40, 52],
    "itemsize": 64,
})

CONTACT_PROPERTY_F = np.dtype({
    "names": list(CONTACT_PROPERTY.names),
    "formats": ["<f4"] * 11,
    "offsets": [4 * i for i in range(11)],
    "itemsize": 44,
})

PLANE_F = np.dtype({
    "names": list(PLANE.names),
    "formats": ["<f4", "<f4"] + [F3] * 9,
    "offsets": [0, 4] + [8 + 12 * i for i in range(9)],
    "itemsize": 116,
})

POLYGON_F = np.dtype({
    "names": list(POLYGON.names),
    "formats": ["<i4"] + [F3] * 6,
    "offsets": [0] + [4 + 12 * i for i in range(6)],
    "itemsize": 76,
})

POLYGON_MASS_F = np.dtype({
    "names": list(POLYGON_MASS.names),
    "formats": [F3, ("<f4", (4,)), F3, F3, F3, F3],
    "offsets": [0, 16, 32, 44, 56, 68],
    "itemsize": 80,
})


def to_single(rec: np.ndarray, dtype: np.dtype) -> np.ndarray:
    """A double-precision record array converted field by field to its
    single-precision twin (values rounded to nearest float)."""
    out = np.zeros(rec.shape, dtype=dtype)
    for name in dtype.names:
        out[name] = rec[name]
    return out


def make_params(*, np_, ncell, grid, dt, cell_size, world_origin, gravity, rolling=True,
                nsphere=0, cohesion=0.0):
    """Fill a ``device_parameters`` record the way dem_simulation::initialize
    does (dem_simulation.cpp:289-307): half2dt = 0.5*dt*dt."""
    p = np.zeros((), dtype=PARAMS)
    p["rolling"] = 1 if rolling else 0
    p["np"] = np_
    p["nsphere"] = nsphere
    p["ncell"] = ncell
    p["grid"] = grid
    p["dt"] = dt
    p["half2dt"] = 0.5 * dt * dt
    p["cell_size"] = cell_size
    p["cohesion"] = cohesion
    p["gravity"] = gravity
    p["world_origin"] = world_origin
    return p


def make_contact_property(*, E_i, E_j, nu_i, nu_j, G_i=0.0, G_j=0.0, rest, fric, sratio,
                          coh=0.0):
    """``device_contact_property`` as contact::cudaMemoryAlloc builds it
    (contact.cpp:107-116): rolling friction is always 0 there."""
    c = np.zeros((), dtype=CONTACT_PROPERTY)
    c["Ei"], c["Ej"], c["pri"], c["prj"] = E_i, E_j, nu_i, nu_j
    c["Gi"], c["Gj"], c["rest"], c["fric"] = G_i, G_j, rest, fric
    c["rfric"], c["coh"], c["sratio"] = 0.0, coh, sratio
    return c


def define_plane(xw, pa, pc, pb):
    """Four-point plane (xcar plane.cpp:47-76): w2 = pa, w3 = pc, w4 = pb;
    l1 = |pa - xw|, l2 = |pb - xw|, u1, u2 the unit edges, uw = u1 x u2."""
    xw, pa, pc, pb = (np.asarray(v, dtype=np.float64) for v in (xw, pa, pc, pb))
    rec = np.zeros((), dtype=PLANE)
    a = pa - xw
    b = pb - xw
    l1 = float(np.sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]))
    l2 = float(np.sqrt(b[0] * b[0] + b[1] * b[1] + b[2] * b[2]))
    u1 = a / l1
    u2 = b / l2
    uw = np.array([u1[1] * u2[2] - u1[2] * u2[1], u1[2] * u2[0] - u1[0] * u2[2],
                   u1[0] * u2[1] - u1[1] * u2[0]])
    rec["l1"], rec["l2"] = l1, l2
    rec["u1"], rec["u2"], rec["uw"], rec["xw"] = u1, u2, uw, xw
    rec["pa"], rec["pb"] = a, b
    rec["w2"], rec["w3"], rec["w4"] = pa, pc, pb
    return rec


# ---- the legacy interface (cu_dem_dec.cuh:41-87) ----
LEGACY_PARAMS = np.dtype({
    "names": ["np", "nsp", "ncell", "grid", "dt", "half2dt", "cell_size", "gravity", "world_origin",
              "kn", "vn", "ks", "vs", "mu", "cohesive"],
    "formats": ["<u4", "<u4", "<u4", ("<u4", (3,)), "<f8", "<f8", "<f8", V3, V3,
                "<f8", "<f8", "<f8", "<f8", "<f8", "<f8"],
    "offsets": [0, 4, 8, 12, 24, 32, 40, 48, 72, 96, 104, 112, 120, 128, 136],
    "itemsize": 144,
})

LEGACY_PLANE = np.dtype({
    "names": ["l1", "l2", "u1", "u2", "uw", "xw", "pa", "pb"],
    "formats": ["<f8", "<f8"] + [V3] * 6,
    "offsets": [0, 8] + [16 + 24 * i for i in range(6)],
    "itemsize": 160,
})

LEGACY_POLYGON = np.dtype({
    "names": ["P", "Q", "R", "V", "W", "N"],
    "formats": [V3] * 6,
    "offsets": [24 * i for i in range(6)],
    "itemsize": 144,
})

LEGACY_MASS_INFO = np.dtype({"names": ["pos", "vel"], "formats": [V3, V3], "offsets": [0, 24], "itemsize": 48})
