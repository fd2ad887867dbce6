"""Seeded test cases shared by the CPU and GPU tests (small enough for the oracle)."""
import numpy as np

from metakonga_gb300 import scenes
from metakonga_gb300.layouts import CONTACT_PROPERTY


def packed_scene(n_side=12, radius=0.0057, seed=3, vel_sigma=0.05, omega_sigma=5.0):
    """A lattice of pitch 11 mm with r = 5.7 mm: every neighbour pair overlaps
    by up to ~0.4 mm; random velocities and spins so that all force terms are
    exercised.  Walls are the settle box's five planes, placed so that the
    outer spheres touch them."""
    sc = scenes.settle_box(seed=seed, n_side=n_side)
    rng = np.random.Generator(np.random.MT19937(seed + 100))
    sc.pos[:, 3] = radius
    sc.vel[:] = rng.normal(0.0, vel_sigma, sc.vel.shape)
    sc.omega[:] = rng.normal(0.0, omega_sigma, sc.omega.shape)
    m, inertia = scenes.mass_inertia(sc.pos[:, 3])
    sc.mass[:] = m
    sc.inertia[:] = inertia
    sc.force[:] = m[:, None] * np.array(scenes.GRAVITY)
    sc.params["cell_size"] = 2.0 * radius
    # box walls hugging the lattice so that outer particles overlap them
    ext = (n_side - 1) * 0.011 / 2.0
    centre = sc.pos[:, :3].mean(axis=0)
    lo = centre - ext - radius * 0.9
    hi = centre + ext + radius * 0.9
    planes, names = scenes.box_walls(lo, hi, lid=True)
    sc.planes, sc.plane_names = planes, names
    sc.cp_planes = np.array([sc.cp_pp] * len(names), dtype=CONTACT_PROPERTY)
    return sc


def random_positions(n, lo, hi, rmin, rmax, seed):
    rng = np.random.Generator(np.random.MT19937(seed))
    pos = np.empty((n, 4))
    pos[:, :3] = rng.uniform(lo, hi, size=(n, 3))
    pos[:, 3] = rng.uniform(rmin, rmax, size=n)
    return pos


def small_drum(n=600, seed=5):
    """A drum of radius 0.1 m with a coarse mesh; particles dropped next to the
    wall so that many touch triangles (faces, edges and vertices)."""
    sc = scenes.drum(n=n, seed=seed, radius=0.1, length=0.08, n_theta=48, n_z=4, n_ring=6,
                     rmin=0.004, rmax=0.006, fill_height=0.08)
    rng = np.random.Generator(np.random.MT19937(seed + 7))
    # push particles outwards so that they overlap the cylinder wall
    xz = sc.pos[:, [0, 2]]
    r = np.linalg.norm(xz, axis=1)
    target = 0.1 - sc.pos[:, 3] * rng.uniform(0.6, 1.05, size=n)
    outer = r > 0.05
    scale = np.where(outer, target / np.maximum(r, 1e-9), 1.0)
    sc.pos[:, 0] *= scale
    sc.pos[:, 2] *= scale
    sc.vel[:] = rng.normal(0.0, 0.05, sc.vel.shape)
    sc.omega[:] = rng.normal(0.0, 5.0, sc.omega.shape)
    sc.pmi["vel"] = (0.01, -0.02, 0.005)
    return sc


def small_hopper(n=1500, seed=5):
    """A small hopper (4,096 triangles, r_top ~0.1 m) whose outer spheres are
    pushed into the cone wall: each sphere within two diameters of the wall
    is moved out radially until its gap to the smooth cone is -r U[0, 0.4]
    .. +0.05 r, so that faces, edges and vertices of the facets are touched."""
    sc = scenes.hopper(n=n, seed=seed, orifice=7.0, fric=0.3)
    rng = np.random.Generator(np.random.MT19937(seed + 11))
    tri = sc.vlist.reshape(-1, 3, 3)
    r_o = np.hypot(tri[:, :, 0], tri[:, :, 1]).min()
    slope = np.tan(np.radians(60.0))
    sin_a = np.sin(np.radians(60.0))
    rho = np.hypot(sc.pos[:, 0], sc.pos[:, 1])
    r_z = r_o + sc.pos[:, 2] / slope
    room = (r_z - rho) * sin_a
    r = sc.pos[:, 3]
    outer = (room < 4.0 * r) & (rho > 1e-6)
    target = r * rng.uniform(0.6, 1.05, size=sc.np_)
    new_rho = r_z - target / sin_a
    scale = np.where(outer, new_rho / np.maximum(rho, 1e-9), 1.0)
    sc.pos[:, 0] *= scale
    sc.pos[:, 1] *= scale
    sc.vel[:] = rng.normal(0.0, 0.05, sc.vel.shape)
    sc.omega[:] = rng.normal(0.0, 5.0, sc.omega.shape)
    return sc


def to_single(sc):
    """The single-precision form of a scene, as the reference's float path
    holds it: float32 state rows, float records (``layouts.*_F``), the float
    parameter block (dem_simulation.cpp:410-426: dt and the other values cast
    to float, half2dt = float(0.5 * dt_f * dt_f) evaluated in double) and the
    FP64 block whose grid size the float cell hash reads."""
    from metakonga_gb300.layouts import (CONTACT_PROPERTY_F, PARAMS_F, PLANE_F, POLYGON_F,
                                         POLYGON_MASS_F, to_single as rec_single)
    p = sc.params
    pf = np.zeros((), dtype=PARAMS_F)
    pf["np"] = sc.np_
    pf["nsphere"] = 0
    pf["ncell"] = p["ncell"]
    pf["grid"] = p["grid"]
    dt_f = np.float32(p["dt"])
    pf["dt"] = dt_f
    pf["half2dt"] = np.float32(0.5 * np.float64(dt_f) * np.float64(dt_f))
    pf["cell_size"] = np.float32(p["cell_size"])
    pf["cohesion"] = 0.0
    pf["gravity"] = np.asarray(p["gravity"], np.float32)
    pf["world_origin"] = np.asarray(p["world_origin"], np.float32)
    hash_grid = p.copy()
    hash_grid["np"] = sc.np_
    out = {"params_f": pf, "hash_grid": hash_grid}
    for k in ("pos", "vel", "acc", "omega", "alpha", "mass", "inertia"):
        out[k] = np.ascontiguousarray(getattr(sc, k), dtype=np.float32)
    out["force"] = (out["mass"][:, None] * pf["gravity"][None, :]).astype(np.float32)
    out["moment"] = np.zeros_like(out["vel"])
    out["cp_pp"] = rec_single(sc.cp_pp.reshape(1), CONTACT_PROPERTY_F)
    out["planes"] = rec_single(sc.planes, PLANE_F)
    out["cp_planes"] = rec_single(sc.cp_planes, CONTACT_PROPERTY_F)
    if sc.ntri:
        out["poly"] = rec_single(sc.poly, POLYGON_F)
        out["sphere"] = np.ascontiguousarray(sc.sphere, dtype=np.float32)
        out["pmi"] = rec_single(sc.pmi, POLYGON_MASS_F)
        out["cp_poly"] = rec_single(sc.cp_poly, CONTACT_PROPERTY_F)
    return out


def legacy_constants(r_eq, m_eq, fric=scenes.FRICTION):
    """The legacy interface's global contact constants (kn, vn, ks, vs, mu)
    for one equivalent radius and mass, from the DHS definitions."""
    import math
    E, nu, e = scenes.E_YOUNG, scenes.POISSON, scenes.RESTITUTION
    eeq = (E * E) / (E * (1 - nu * nu) + E * (1 - nu * nu))
    beta = math.pi / math.log(e)
    kn = (4.0 / 3.0) * eeq * math.sqrt(r_eq)
    vn = math.sqrt((4.0 * m_eq * kn) / (1.0 + beta * beta))
    return kn, vn, kn * scenes.STIFFNESS_RATIO, vn * scenes.STIFFNESS_RATIO, fric


def to_legacy(sc, nsp=0, cell_size=None):
    """A scene in the legacy layouts (cu_dem_dec.cuh): double4 pos, vel, acc
    (mass in .w), omega, alpha (inertia in .w); double3 force and moment;
    the parameter block with the particle-particle constants of the mean
    radius."""
    from metakonga_gb300.layouts import LEGACY_PARAMS
    n = sc.np_
    out = {"pos": np.ascontiguousarray(sc.pos, dtype=np.float64)}
    for k, w in (("vel", None), ("acc", "mass"), ("omega", None), ("alpha", "inertia")):
        a = np.zeros((n, 4))
        a[:, :3] = getattr(sc, k)
        if w:
            a[:, 3] = getattr(sc, w)
        out[k] = a
    out["force"] = np.zeros((n, 3))
    out["moment"] = np.zeros((n, 3))
    r = float(sc.pos[:, 3].mean())
    m = float(sc.mass.mean())
    kn, vn, ks, vs, mu = legacy_constants(r / 2, m / 2)
    p = np.zeros((), dtype=LEGACY_PARAMS)
    p["np"], p["nsp"], p["ncell"] = n, nsp, sc.params["ncell"]
    p["grid"] = sc.params["grid"]
    p["dt"] = sc.params["dt"]
    p["half2dt"] = sc.params["half2dt"]
    p["cell_size"] = cell_size if cell_size is not None else sc.params["cell_size"]
    p["gravity"] = sc.params["gravity"]
    p["world_origin"] = sc.params["world_origin"]
    p["kn"], p["vn"], p["ks"], p["vs"], p["mu"] = kn, vn, ks, vs, mu
    p["cohesive"] = 0.0
    out["params"] = p
    out["wall"] = legacy_constants(r, m)
    return out


def legacy_planes(planes):
    """Legacy plane records (no w2..w4) of live PLANE records."""
    from metakonga_gb300.layouts import LEGACY_PLANE
    out = np.zeros(planes.shape[0], dtype=LEGACY_PLANE)
    for k in LEGACY_PLANE.names:
        out[k] = planes[k]
    return out


def legacy_mesh(tri):
    """Indexed mesh of triangles (T, 3, 3): vertices (V, 3), indice (T, 3)
    and the polygons of each vertex as id_set / poly_start / poly_end."""
    v = tri.reshape(-1, 3)
    key = np.round(v, 12)
    verts, inv = np.unique(key, axis=0, return_inverse=True)
    inv = inv.reshape(-1)
    indice = inv.reshape(-1, 3).astype(np.uint32)
    pairs = sorted((int(indice[t, c]), t) for t in range(indice.shape[0]) for c in range(3))
    id_set = np.array([t for _, t in pairs], np.uint32)
    counts = np.bincount([vv for vv, _ in pairs], minlength=verts.shape[0])
    poly_end = np.cumsum(counts).astype(np.uint32)
    poly_start = (poly_end - counts).astype(np.uint32)
    return verts.astype(np.float64), indice, id_set, poly_start, poly_end


def emitter_column(n=6, radius=0.005, pitch=0.05, dt=1.0e-5):
    """n spheres 50 mm apart along x at one height: no contacts, no walls."""
    from metakonga_gb300.layouts import PLANE
    pos = np.zeros((n, 4))
    pos[:, 0] = pitch * np.arange(n) - 0.4
    pos[:, 2] = 0.3
    pos[:, 3] = radius
    return scenes.Scene(name="column", seed=0, dt=dt, steps=0, params=scenes._reference_grid(radius, n, dt),
                        pos=pos, **scenes._state(pos), cp_pp=scenes._default_property(),
                        planes=np.zeros(0, dtype=PLANE), plane_names=[],
                        cp_planes=np.zeros(0, dtype=CONTACT_PROPERTY))


EMITTER_MODEL = """MODEL_NAME hopper_fill
GRAVITY 0 -9.80665 0
UNIT 0
SINGLE 0

DEM_MODEL_DATA
INTEGRATOR 0
SORT 0

PARTICLES_DATA
CREATE_SHAPE plane
NAME emitter
MATERIAL_TYPE 7
DIMENSION 0.1 6 0.1
STARTPOINT 0 0.03 0
DIRECTION 0 -1 0
SPACE 0
RADIUS 0.004 0.004
MAKING 1 726 0 0.005 0 none
MATERIAL 1e7 2500 0.3 0
END_DATA

GEOMETRY_OBJECTS_DATA
OBJECT plane
NAME floor
MATERIAL_TYPE 7
GEOMETRY_USE 0
POINT_A 0 0 0
POINT_B 0 0 0.1
POINT_C 0.1 0 0.1
POINT_D 0.1 0 0
MATERIAL 1e7 0.3 2500 0
OBJECT plane
NAME wall_x0
MATERIAL_TYPE 0
GEOMETRY_USE 0
POINT_A 0 0 0
POINT_B 0 0.2 0
POINT_C 0 0.2 0.1
POINT_D 0 0 0.1
MATERIAL 0 0 0 0
OBJECT plane
NAME wall_x1
MATERIAL_TYPE 0
GEOMETRY_USE 0
POINT_A 0.1 0 0
POINT_B 0.1 0 0.1
POINT_C 0.1 0.2 0.1
POINT_D 0.1 0.2 0
MATERIAL 0 0 0 0
OBJECT plane
NAME wall_z0
MATERIAL_TYPE 0
GEOMETRY_USE 0
POINT_A 0 0 0
POINT_B 0.1 0 0
POINT_C 0.1 0.2 0
POINT_D 0 0.2 0
MATERIAL 0 0 0 0
OBJECT plane
NAME wall_z1
MATERIAL_TYPE 0
GEOMETRY_USE 0
POINT_A 0 0 0.1
POINT_B 0 0.2 0.1
POINT_C 0.1 0.2 0.1
POINT_D 0.1 0 0.1
MATERIAL 0 0 0 0
END_DATA

CONTACT_ELEMENTS_DATA
NAME pp
METHOD 1
OBJECT0 particles
OBJECT1 particles
RESTITUTION 0.7
RATIO 0.8
FRICTION 0.3
COHESION 0
NAME p_floor
METHOD 1
OBJECT0 particles
OBJECT1 floor
RESTITUTION 0.6
RATIO 0.8
FRICTION 0.4
COHESION 0
NAME p_wall0
METHOD 1
OBJECT0 particles
OBJECT1 wall_x0
RESTITUTION 0.6
RATIO 0.8
FRICTION 0.4
COHESION 0
NAME p_wall1
METHOD 1
OBJECT0 wall_x1
OBJECT1 particles
RESTITUTION 0.6
RATIO 0.8
FRICTION 0.4
COHESION 0
NAME p_wall2
METHOD 1
OBJECT0 particles
OBJECT1 wall_z0
RESTITUTION 0.6
RATIO 0.8
FRICTION 0.4
COHESION 0
NAME p_wall3
METHOD 1
OBJECT0 particles
OBJECT1 wall_z1
RESTITUTION 0.6
RATIO 0.8
FRICTION 0.4
COHESION 0
END_DATA
"""


def emitter_box(layers=6, drop_speed=2.0):
    """The plane emitter of EMITTER_MODEL: 6 layers of 11 x 11 spheres
    (r = 4 mm) staged at y = 30 mm above the floor of a 0.1 m box with steel
    side walls, one layer every 500 steps (0.005 s at dt = 1e-5), each
    leaving downwards at drop_speed.  Returns the scene and its emitter."""
    from metakonga_gb300 import model_file
    text = EMITTER_MODEL.replace("DIMENSION 0.1 6 0.1", f"DIMENSION 0.1 {layers} 0.1")
    built = model_file.build_scene(model_file.read_model(text), dt=1.0e-5, seed=17)
    sc = built.scene
    sc.vel[:, 1] = -drop_speed
    return sc, built.emitter
