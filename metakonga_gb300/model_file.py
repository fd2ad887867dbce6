"""The reference's model text files: reader, writer and scene builder.

A model file (modelManager::OpenModel, xcar/modelManager.cpp:53-106) is a
whitespace-separated token stream of sections:

    MODEL_NAME <name>  GRAVITY gx gy gz  UNIT u  SINGLE s
    DEM_MODEL_DATA  INTEGRATOR i  SORT s                        (dem_model.cpp:38-46)
    PARTICLES_DATA  CREATE_SHAPE cube|plane|circle ... END_DATA (particleManager.cpp:42-130)
    GEOMETRY_OBJECTS_DATA  OBJECT cube|plane|polygon ... END_DATA
                                                 (xcar/geometryObjects.cpp:26-99)
    CONTACT_ELEMENTS_DATA  NAME ... END_DATA                    (contactManager.cpp:40-63)

Each value follows a keyword token that the reader skips, as the reference's
``qts >> ch >> value`` does; the polygon object's FILE is the rest of its
line.  ``read_model`` returns a ``ModelSpec``; ``write_model`` writes one in
the reference's Save layout (particleManager.cpp:30-40 and the creators'
logs, contactManager.cpp:28-37 and :319-328, geometryObjects.cpp:139-205);
``build_scene`` makes the ``Scene`` and the emitter that
``engine.DeviceScene.set_emitter`` takes, the way dem_simulation::initialize
does (dem_simulation.cpp:204-322).

Out of scope (the DEM contact step only): MULTIBODY_MODEL_DATA is skipped,
plane-polygon contact pairs (contact_plane_polygonObject, an MBD coupling)
are reported in ``Built.ignored``, and polygon shapes other than STL ASCII
(the MilkShape importer) are refused.
"""
from __future__ import annotations

import dataclasses
import os

import numpy as np

from . import creators
from .layouts import (CONTACT_PROPERTY, PLANE, POLYGON_MASS, define_plane, make_contact_property,
                      make_params)
from .scenes import Scene, _mesh_arrays, mass_inertia

USER_INPUT = 7

# material constants by material_type (xcar/types.h:20-55, getMaterialConstant
# :309-323): (youngs, density, poisson, shear)
MATERIALS = {
    0: (2e11, 7850.0, 0.3, 0.0),        # steel
    1: (35e6, 1900.0, 0.45, 0.0),       # medium clay
    2: (1.1e9, 950.0, 0.42, 0.0),       # polyethylene
    3: (6.8e10, 2180.0, 0.19, 0.0),     # glass
    4: (3.2e9, 1185.0, 0.37, 0.0),      # acrylic
    5: (70.0e9, 2700.0, 0.34, 0.0),     # aluminium
    6: (4.0e7, 2600.0, 0.3, 0.0),       # sand
}


def material(mtype: int, youngs: float, density: float, poisson: float, shear: float):
    """object::setMaterial (xcar/object.cpp:86-106): the given values for
    USER_INPUT, the table's otherwise.  Returns (youngs, density, poisson, shear)."""
    if int(mtype) == USER_INPUT:
        return (float(youngs), float(density), float(poisson), float(shear))
    if int(mtype) not in MATERIALS:
        raise ValueError(f"unknown material type {mtype}")
    return MATERIALS[int(mtype)]


@dataclasses.dataclass
class ModelSpec:
    name: str = "model"
    gravity: tuple = (0.0, -9.80665, 0.0)
    unit: int = 0
    single: int = 0
    integrator: int = 0
    sort: int = 0
    shapes: list = dataclasses.field(default_factory=list)     # particle creators, in file order
    objects: dict = dataclasses.field(default_factory=dict)    # name -> geometry object
    contacts: list = dataclasses.field(default_factory=list)   # contact pairs, in file order


class _Tokens:
    def __init__(self, text: str):
        self.text = text
        self.i = 0

    def word(self) -> str:
        t, n, i = self.text, len(self.text), self.i
        while i < n and t[i].isspace():
            i += 1
        j = i
        while j < n and not t[j].isspace():
            j += 1
        self.i = j
        if i == j:
            raise ValueError("model file ends inside a section")
        return t[i:j]

    def num(self, kind=float):
        w = self.word()
        return int(w) if kind is int else float(w)

    def rest_of_line(self) -> str:
        j = self.text.find("\n", self.i)
        j = len(self.text) if j < 0 else j
        line = self.text[self.i:j]
        self.i = j
        return line[1:] if line.startswith(" ") else line   # QString::remove(0, 1)

    def at_end(self) -> bool:
        return self.text[self.i:].strip() == ""


def _read_particles(tk: _Tokens, spec: ModelSpec) -> None:
    ch = ""
    while ch != "END_DATA":
        ch = tk.word()
        if ch == "CREATE_SHAPE":
            ch = tk.word()
        if ch == "cube":
            s = {"kind": "cube"}
            tk.word(); s["name"] = tk.word()
            tk.word(); s["type"] = tk.num(int)
            tk.word(); s["dim"] = tuple(tk.num() for _ in range(3))
            tk.word(); s["start"] = tuple(tk.num() for _ in range(3))
            tk.word(); s["spacing"] = tk.num()
            tk.word(); s["radius"] = (tk.num(), tk.num())
            tk.word(); s["material"] = tuple(tk.num() for _ in range(4))   # youngs density poisson shear
            spec.shapes.append(s)
        elif ch in ("plane", "circle"):
            s = {"kind": ch}
            tk.word(); s["name"] = tk.word()
            tk.word(); s["type"] = tk.num(int)
            if ch == "plane":
                tk.word(); s["dim"] = (tk.num(), tk.num(int), tk.num())          # dx ny dz
            else:
                tk.word(); s["diameter"] = tk.num()
                tk.word(); s["ny"] = tk.num(int)
            tk.word(); s["start"] = tuple(tk.num() for _ in range(3))
            tk.word(); s["direction"] = tuple(tk.num() for _ in range(3))
            tk.word(); s["spacing"] = tk.num()
            tk.word(); s["radius"] = (tk.num(), tk.num())
            tk.word()
            s["making"] = {"realtime": tk.num(int), "np": tk.num(int), "per_np": tk.num(int),
                           "per_time": tk.num(), "one_by_one": tk.num(int), "file": tk.word()}
            tk.word(); s["material"] = tuple(tk.num() for _ in range(4))
            spec.shapes.append(s)


def _read_objects(tk: _Tokens, spec: ModelSpec) -> None:
    ch = ""
    while ch != "END_DATA":
        ch = tk.word()
        if ch == "OBJECT":
            ch = tk.word()
        if ch == "cube":
            o = {"kind": "cube"}
            tk.word(); name = tk.word()
            tk.word(); o["type"] = tk.num(int)
            tk.word(); o["use"] = tk.num(int)
            tk.word(); o["start"] = tuple(tk.num() for _ in range(3))
            tk.word(); o["end"] = tuple(tk.num() for _ in range(3))
            tk.word(); o["material"] = tuple(tk.num() for _ in range(4))   # youngs poisson density shear
            spec.objects[name] = o
        elif ch == "plane":
            o = {"kind": "plane"}
            tk.word(); name = tk.word()
            tk.word(); o["type"] = tk.num(int)
            tk.word(); o["use"] = tk.num(int)
            o["points"] = []
            for _ in range(4):
                tk.word()
                o["points"].append(tuple(tk.num() for _ in range(3)))
            tk.word(); o["material"] = tuple(tk.num() for _ in range(4))
            spec.objects[name] = o
        elif ch == "polygon":
            o = {"kind": "polygon"}
            tk.word(); name = tk.word()
            tk.word(); o["file"] = tk.rest_of_line().strip()
            tk.word(); o["cm"] = tuple(tk.num() for _ in range(3))
            tk.word(); o["type"] = tk.num(int)
            tk.word(); o["use"] = tk.num(int)
            tk.word(); o["shape_type"] = tk.num(int)
            tk.word(); o["material"] = tuple(tk.num() for _ in range(4))
            tk.word(); o["tool"] = (tk.word(), tk.word(), tk.num())
            spec.objects[name] = o


def _read_contacts(tk: _Tokens, spec: ModelSpec) -> None:
    ch = tk.word()
    while ch != "END_DATA":
        c = {"name": tk.word()}
        tk.word(); c["method"] = tk.num(int)
        tk.word(); c["obj0"] = tk.word()
        tk.word(); c["obj1"] = tk.word()
        tk.word(); c["rest"] = tk.num()
        tk.word(); c["ratio"] = tk.num()
        tk.word(); c["fric"] = tk.num()
        tk.word(); c["coh"] = tk.num()
        spec.contacts.append(c)
        ch = tk.word()


def read_model(text: str) -> ModelSpec:
    """Parses a model file's text (modelManager::OpenModel order)."""
    tk = _Tokens(text)
    spec = ModelSpec()
    while not tk.at_end():
        ch = tk.word()
        if ch == "MODEL_NAME":
            spec.name = tk.word()
            tk.word(); spec.gravity = tuple(tk.num() for _ in range(3))
            tk.word(); spec.unit = tk.num(int)
            tk.word(); spec.single = tk.num(int)
        elif ch == "DEM_MODEL_DATA":
            tk.word(); spec.integrator = tk.num(int)
            tk.word(); spec.sort = tk.num(int)
        elif ch == "PARTICLES_DATA":
            _read_particles(tk, spec)
        elif ch == "GEOMETRY_OBJECTS_DATA":
            _read_objects(tk, spec)
        elif ch == "CONTACT_ELEMENTS_DATA":
            _read_contacts(tk, spec)
        elif ch == "MULTIBODY_MODEL_DATA":
            # out of scope: skip to its END_DATA
            while tk.word() != "END_DATA":
                pass
    return spec


def _g(x) -> str:
    return repr(float(x)) if isinstance(x, float) else str(x)


def write_model(spec: ModelSpec) -> str:
    """The model in the reference's Save layout; sections' entries in name
    order, as its QMap-held logs are written."""
    L = [f"MODEL_NAME {spec.name}",
         "GRAVITY " + " ".join(_g(float(v)) for v in spec.gravity),
         f"UNIT {spec.unit}", f"SINGLE {spec.single}", "",
         "DEM_MODEL_DATA", f"INTEGRATOR {spec.integrator}", f"SORT {spec.sort}", "", "PARTICLES_DATA"]
    for s in sorted(spec.shapes, key=lambda s: s["name"]):
        v3 = lambda t: " ".join(_g(float(x)) for x in t)
        L += [f"CREATE_SHAPE {s['kind']}", f"NAME {s['name']}", f"MATERIAL_TYPE {s['type']}"]
        if s["kind"] == "cube":
            L += ["DIMENSION " + v3(s["dim"]), "STARTPOINT " + v3(s["start"])]
        elif s["kind"] == "plane":
            dx, ny, dz = s["dim"]
            L += [f"DIMENSION {_g(float(dx))} {int(ny)} {_g(float(dz))}", "STARTPOINT " + v3(s["start"]),
                  "DIRECTION " + v3(s["direction"])]
        else:
            L += [f"DIAMETER {_g(float(s['diameter']))}", f"NUM_HEIGHT {int(s['ny'])}",
                  "STARTPOINT " + v3(s["start"]), "DIRECTION " + v3(s["direction"])]
        L += [f"SPACE {_g(float(s['spacing']))}", "RADIUS " + v3(s["radius"])]
        if s["kind"] != "cube":
            m = s["making"]
            L.append(f"MAKING {m['realtime']} {m['np']} {m['per_np']} {_g(float(m['per_time']))} "
                     f"{m['one_by_one']} {m['file']}")
        L.append("MATERIAL " + v3(s["material"]))
    L += ["END_DATA", "", "GEOMETRY_OBJECTS_DATA"]
    for name in sorted(spec.objects):
        o = spec.objects[name]
        v3 = lambda t: " ".join(_g(float(x)) for x in t)
        if o["kind"] == "cube":
            L += ["OBJECT cube", f"NAME {name}", f"MATERIAL_TYPE {o['type']}", f"GEOMETRY_USE {o['use']}",
                  "START_POINT " + v3(o["start"]), "END_POINT " + v3(o["end"]), "MATERIAL " + v3(o["material"])]
        elif o["kind"] == "plane":
            L += ["OBJECT plane", f"NAME {name}", f"MATERIAL_TYPE {o['type']}", f"GEOMETRY_USE {o['use']}"]
            L += [f"POINT_{k} " + v3(p) for k, p in zip("ABCD", o["points"])]
            L.append("MATERIAL " + v3(o["material"]))
        else:
            t = o["tool"]
            L += ["OBJECT polygon", f"NAME {name}", f"FILE {o['file']}", "CM " + v3(o["cm"]),
                  f"MATERIAL_TYPE {o['type']}", f"GEOMETRY_USE {o['use']}",
                  f"IMPORT_SHAPE_TYPE {o['shape_type']}", "MATERIAL " + v3(o["material"]),
                  f"TOOL {t[0]} {t[1]} {_g(float(t[2]))}"]
    L += ["END_DATA", "", "CONTACT_ELEMENTS_DATA"]
    for c in sorted(spec.contacts, key=lambda c: c["name"]):
        L += [f"NAME {c['name']}", f"METHOD {c['method']}", f"OBJECT0 {c['obj0']}", f"OBJECT1 {c['obj1']}",
              f"RESTITUTION {_g(float(c['rest']))}", f"RATIO {_g(float(c['ratio']))}",
              f"FRICTION {_g(float(c['fric']))}", f"COHESION {_g(float(c['coh']))}"]
    L += ["END_DATA", ""]
    return "\n".join(L)


def read_stl_ascii(path: str) -> np.ndarray:
    """Triangles (T, 3, 3) of an ASCII STL file, scaled by 0.001 (millimetres
    to metres), as vpolygon::_loadSTLASCII reads them (vpolygon.cpp:188-262)."""
    with open(path) as f:
        words = f.read().split()
    tri = []
    i = 0
    while i < len(words):
        if words[i] == "vertex":
            tri.append([float(words[i + 1]), float(words[i + 2]), float(words[i + 3])])
            i += 4
        else:
            i += 1
    if not tri or len(tri) % 3:
        raise ValueError(f"{path}: not an ASCII STL of whole facets")
    return 0.001 * np.asarray(tri, dtype=np.float64).reshape(-1, 3, 3)


@dataclasses.dataclass
class Built:
    scene: Scene
    emitter: dict            # {"period", "groups", "active"} or None: every particle from the start
    ignored: list            # contact pairs outside the DEM contact step
    particle_material: tuple  # (youngs, density, poisson, shear)


def _cube_planes(start, end):
    """cube::define (xcar/cube.cpp:55-75): six three-point planes from the
    minimum corner; a three-point plane leaves w2..w4 at zero (plane.cpp:78-93)."""
    mn = np.asarray(start, dtype=np.float64)
    mx = np.asarray(end, dtype=np.float64)
    size = np.array([np.linalg.norm(mx - np.array([mn[0], mx[1], mx[2]])),
                     np.linalg.norm(mx - np.array([mx[0], mn[1], mx[2]])),
                     np.linalg.norm(mx - np.array([mx[0], mx[1], mn[2]]))])
    X, Y, Z = (np.array([size[0], 0, 0]), np.array([0, size[1], 0]), np.array([0, 0, size[2]]))
    three = [(mn, mn + Z, mn + X), (mn, mn + Y, mn + Z), (mn + X, mn + X + Z, mn + X + Y),
             (mn, mn + X, mn + Y), (mn + Z, mn + Y + Z, mn + X + Z), (mn + Y, mn + X + Y, mn + Y + Z)]
    out = np.zeros(6, dtype=PLANE)
    for k, (xw, pa, pb) in enumerate(three):
        rec = define_plane(xw, pa, pb, pb)
        rec["w2"], rec["w3"], rec["w4"] = 0.0, 0.0, 0.0
        out[k] = rec
    return out


def build_scene(spec: ModelSpec, dt: float, seed: int = 0, base_dir: str = ".", steps: int = 0) -> Built:
    """The scene a model describes: particles from its creators, walls and
    meshes from the objects its contact pairs name, the reference's grid
    (origin (-1, -1, -1), 128^3 cells of twice the largest particle or
    triangle radius, dem_simulation.cpp:254-262), mass and inertia from the
    particles' density (dem_simulation.cpp:240-250), force = m g."""
    rng = np.random.Generator(np.random.MT19937(seed))
    pos_parts, groups = [], []
    pmat = None
    realtime, one_by_one, per_np, per_time = False, False, 0, 0.0
    for s in spec.shapes:
        rmin, rmax = s["radius"]
        if s["kind"] == "cube":
            c = creators.cube_particles(*s["dim"], *s["start"], rmin, rmax, rng)
        elif s["kind"] == "plane":
            dx, ny, dz = s["dim"]
            c = creators.plane_particles(dx, ny, dz, *s["start"], rmin, rmax, rng)
        else:
            c = creators.circle_particles(s["diameter"], s["ny"], *s["start"], rmin, rmax, rng)
        pos_parts.append(c.pos)
        groups += c.groups
        pmat = material(s["type"], *s["material"])   # the last creator's (setMaterial per creator)
        if s["kind"] != "cube":
            m = s["making"]
            realtime, one_by_one, per_time = bool(m["realtime"]), bool(m["one_by_one"]), float(m["per_time"])
            if one_by_one:
                if s["kind"] == "plane":
                    raise ValueError("plane creator with one-by-one emission: the reference divides by "
                                     "its zero y layer count (particleManager.cpp:395-396)")
                per_np = int(m["per_np"])
    if pmat is None:
        raise ValueError("model has no particles")
    pos = np.concatenate(pos_parts) if pos_parts else np.zeros((0, 4))
    n = pos.shape[0]

    planes, cp_planes, plane_names, bodies, ignored = [], [], [], [], []
    cp_pp = None
    ymod, _, nu, shear = pmat
    for c in sorted(spec.contacts, key=lambda c: c["name"]):   # QMap order (contactManager.cpp:167-174)
        names = (c["obj0"], c["obj1"])
        if "particles" not in names:
            ignored.append(c["name"])
            continue
        other = names[1] if names[0] == "particles" else names[0]
        if other == "particles":
            mo = (ymod, nu, shear)
        else:
            o = spec.objects[other]
            e, p, d, sh = o["material"]          # youngs poisson density shear
            oy, _, op, osh = material(o["type"], e, d, p, sh)
            mo = (oy, op, osh)
        first = names[0] == "particles"
        a = (ymod, nu, shear) if first else mo
        b = mo if first else (ymod, nu, shear)
        cp = make_contact_property(E_i=a[0], E_j=b[0], nu_i=a[1], nu_j=b[1], G_i=a[2], G_j=b[2],
                                   rest=c["rest"], fric=c["fric"], sratio=c["ratio"], coh=c["coh"])
        if other == "particles":
            cp_pp = cp
            continue
        o = spec.objects[other]
        if o["kind"] == "plane":
            pa, pb, pc, pd = o["points"]
            planes.append(np.asarray(define_plane(pa, pb, pc, pd)).reshape(1))
            cp_planes.append(cp)
            plane_names.append(c["name"])
        elif o["kind"] == "cube":
            planes.append(_cube_planes(o["start"], o["end"]))
            cp_planes += [cp] * 6
            plane_names += [f"{c['name']}[{k}]" for k in range(6)]
        else:
            if o["shape_type"] != 2:
                raise ValueError(f"polygon object {other}: only STL ASCII shapes are read")
            if o["tool"][0] == "poly_refinement" and o["tool"][2]:
                raise ValueError(f"polygon object {other}: mesh refinement is not supported")
            path = o["file"] if os.path.isabs(o["file"]) else os.path.join(base_dir, o["file"])
            bodies.append((read_stl_ascii(path), np.asarray(o["cm"], dtype=np.float64), cp))

    plane_arr = np.concatenate(planes) if planes else np.zeros(0, dtype=PLANE)
    poly = sphere = vlist = pmi = cp_poly = None
    maxr = float(pos[:, 3].max()) if n else 0.0
    ntri = 0
    if bodies:
        polys, spheres, vlists = [], [], []
        pmi = np.zeros(len(bodies), dtype=POLYGON_MASS)
        for b, (tri, cm, _) in enumerate(bodies):
            p, sp, _world = _mesh_arrays(tri, body=b)
            polys.append(p)
            spheres.append(sp)
            vlists.append((tri - cm).reshape(-1, 9))   # body frame (polygonObject.cpp:119-159)
            pmi[b]["origin"] = cm
            pmi[b]["ep"] = (1.0, 0.0, 0.0, 0.0)
        poly, sphere, vlist = np.concatenate(polys), np.concatenate(spheres), np.concatenate(vlists)
        cp_poly = np.array([cp for _, _, cp in bodies], dtype=CONTACT_PROPERTY)
        ntri = poly.shape[0]
        maxr = max(maxr, float(sphere[:, 3].max()))
    params = make_params(np_=n, ncell=128 ** 3, grid=(128, 128, 128), dt=dt, cell_size=2.0 * maxr,
                         world_origin=(-1.0, -1.0, -1.0), gravity=spec.gravity, rolling=True, nsphere=ntri)
    m, inertia = mass_inertia(pos[:, 3], density=pmat[1])
    force = m[:, None] * np.asarray(spec.gravity, dtype=np.float64)[None, :]
    z3 = lambda: np.zeros((n, 3))
    if cp_pp is None:
        cp_pp = make_contact_property(E_i=ymod, E_j=ymod, nu_i=nu, nu_j=nu, rest=0.0, fric=0.0, sratio=0.0)
        ignored.append("(no particle-particle pair: contact constants zero)")
    sc = Scene(name=spec.name, seed=seed, dt=dt, steps=steps, params=params, pos=np.ascontiguousarray(pos),
               vel=z3(), acc=z3(), omega=z3(), alpha=z3(), force=np.ascontiguousarray(force), moment=z3(),
               mass=m, inertia=inertia, cp_pp=cp_pp, planes=plane_arr, plane_names=plane_names,
               cp_planes=np.array(cp_planes, dtype=CONTACT_PROPERTY), poly=poly, sphere=sphere,
               vlist=vlist, pmi=pmi, cp_poly=cp_poly)
    emitter = None
    if realtime:
        # dem_simulation.cpp:210-222: steps between creations
        period = int((1.0 / per_np) / dt) if one_by_one else int((per_time + 1e-9) / dt)
        if period:
            emitter = {"period": period, "groups": None if one_by_one else list(groups), "active": 0}
    return Built(scene=sc, emitter=emitter, ignored=ignored, particle_material=pmat)
