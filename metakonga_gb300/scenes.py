"""Seeded synthetic DEM scenes in the reference's boundary layouts.

The reference reads particle sets and walls from its model files
(particleManager.cpp:42-130, contactManager.cpp:29-63); those files are not
available, so the workloads are generated here with the shapes, sizes and
material constants of the benchmark scenes:

* ``settle_box``   8,000 monodisperse spheres (r = 5 mm) on a jittered
                   20x20x20 lattice of pitch 11 mm, centred in a 0.3x0.3x0.5 m
                   box of 5 plane walls, dt = 1e-5 s.
* ``polydisperse_box``  N spheres (default 1,000,000) with r ~ U[2, 4] mm,
                   rejection-sampled without overlap in a 1x1x2 m box of plane
                   walls, dt = 5e-6 s.
* ``drum``         spheres inside a closed, tessellated cylinder that rotates
                   about its axis (particle-triangle contacts).
* ``lattice_box``  the polydisperse settle's box and density with the
                   spheres on a jittered lattice (fast, for request streams).
* ``hopper``       spheres in a 60-degree conical hopper of 4,096 triangles
                   above a plane floor, r ~ U[2, 4] mm, orifice of 6-12
                   particle diameters; ``hopper_batch`` draws the batch of
                   independent hoppers (log-uniform particle counts).

Every scene carries the state arrays the reference's dem_simulation allocates
(dem_simulation.cpp:174-199, 232-251): pos (x, y, z, r) as double4, vel, acc,
omega, alpha, force (= m g), moment as packed double3, mass and inertia, plus
the grid parameters the reference hard-codes (dem_simulation.cpp:259-262:
origin (-1, -1, -1), 128^3 cells, cell size = 2 x the largest radius).
Random numbers come from numpy's MT19937 with the seed recorded on the scene.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

from .layouts import (CONTACT_PROPERTY, PLANE, POLYGON, POLYGON_MASS, define_plane,
                      make_contact_property, make_params)

# material constants of the benchmark scenes (Hertz-Mindlin, DHS model)
E_YOUNG = 1.0e7
POISSON = 0.3
RESTITUTION = 0.7
FRICTION = 0.3
STIFFNESS_RATIO = 0.8          # contactPairDialog.cpp:8 default
DENSITY = 2500.0
GRAVITY = (0.0, 0.0, -9.81)


@dataclasses.dataclass
class Scene:
    name: str
    seed: int
    dt: float
    steps: int
    params: np.ndarray            # layouts.PARAMS record
    pos: np.ndarray               # (N, 4) float64
    vel: np.ndarray               # (N, 3)
    acc: np.ndarray
    omega: np.ndarray
    alpha: np.ndarray
    force: np.ndarray
    moment: np.ndarray
    mass: np.ndarray              # (N,)
    inertia: np.ndarray
    cp_pp: np.ndarray             # CONTACT_PROPERTY record
    planes: np.ndarray            # PLANE array, in contact-name order
    plane_names: list
    cp_planes: np.ndarray         # CONTACT_PROPERTY per plane
    poly: np.ndarray = None       # POLYGON array (T,)
    sphere: np.ndarray = None     # (T, 4) circumcentre + radius
    vlist: np.ndarray = None      # (T, 9) body-frame vertices
    pmi: np.ndarray = None        # POLYGON_MASS per polygon body
    cp_poly: np.ndarray = None    # CONTACT_PROPERTY per polygon body

    @property
    def np_(self) -> int:
        return int(self.pos.shape[0])

    @property
    def ntri(self) -> int:
        return 0 if self.poly is None else int(self.poly.shape[0])

    @property
    def ncell(self) -> int:
        return int(self.params["ncell"])

    def copy(self) -> "Scene":
        kw = {}
        for f in dataclasses.fields(self):
            v = getattr(self, f.name)
            kw[f.name] = v.copy() if isinstance(v, np.ndarray) else (list(v) if isinstance(v, list) else v)
        return Scene(**kw)


def _rng(seed: int) -> np.random.Generator:
    return np.random.Generator(np.random.MT19937(seed))


def mass_inertia(radius: np.ndarray, density: float = DENSITY):
    """m = rho * 4/3 * pi * r^3, I = 2/5 * m * r^2 (dem_simulation.cpp:244-245)."""
    m = density * (4.0 / 3.0) * math.pi * np.power(radius, 3.0)
    inertia = (2.0 / 5.0) * m * np.power(radius, 2.0)
    return m, inertia


def _state(pos: np.ndarray, gravity=GRAVITY):
    n = pos.shape[0]
    z3 = lambda: np.zeros((n, 3), dtype=np.float64)
    m, inertia = mass_inertia(pos[:, 3])
    force = np.empty((n, 3), dtype=np.float64)
    for a in range(3):
        force[:, a] = m * gravity[a]
    return dict(vel=z3(), acc=z3(), omega=z3(), alpha=z3(), force=force, moment=z3(),
                mass=m, inertia=inertia)


def _reference_grid(max_radius: float, np_: int, dt: float, nsphere: int = 0, grid=(128, 128, 128),
                    origin=(-1.0, -1.0, -1.0)):
    ncell = grid[0] * grid[1] * grid[2]
    return make_params(np_=np_, ncell=ncell, grid=grid, dt=dt, cell_size=max_radius * 2.0,
                       world_origin=origin, gravity=GRAVITY, rolling=True, nsphere=nsphere)


def _default_property(fric=FRICTION):
    return make_contact_property(E_i=E_YOUNG, E_j=E_YOUNG, nu_i=POISSON, nu_j=POISSON,
                                 rest=RESTITUTION, fric=fric, sratio=STIFFNESS_RATIO)


def box_walls(lo, hi, lid: bool = False):
    """Axis-aligned box of finite four-point planes (floor, 4 sides[, lid]),
    returned in contact-name order (the reference iterates contacts in
    QMap key order, contactManager.cpp:167-174)."""
    x0, y0, z0 = lo
    x1, y1, z1 = hi
    walls = {
        "wall_floor": define_plane((x0, y0, z0), (x1, y0, z0), (x1, y1, z0), (x0, y1, z0)),
        "wall_xm": define_plane((x0, y0, z0), (x0, y1, z0), (x0, y1, z1), (x0, y0, z1)),
        "wall_xp": define_plane((x1, y0, z0), (x1, y0, z1), (x1, y1, z1), (x1, y1, z0)),
        "wall_ym": define_plane((x0, y0, z0), (x0, y0, z1), (x1, y0, z1), (x1, y0, z0)),
        "wall_yp": define_plane((x0, y1, z0), (x1, y1, z0), (x1, y1, z1), (x0, y1, z1)),
    }
    if lid:
        walls["wall_lid"] = define_plane((x0, y0, z1), (x0, y1, z1), (x1, y1, z1), (x1, y0, z1))
    names = sorted(walls)
    arr = np.zeros(len(names), dtype=PLANE)
    for i, n in enumerate(names):
        arr[i] = walls[n]
    return arr, names


def settle_box(seed: int = 2024, n_side: int = 20, pitch: float = 0.011, radius: float = 0.005,
               jitter: float = 0.0005, box=(0.3, 0.3, 0.5), steps: int = 10_000,
               dt: float = 1.0e-5) -> Scene:
    """Monodisperse lattice settle in a box of 5 plane walls (the 8,000-sphere
    CPU-path benchmark scene)."""
    rng = _rng(seed)
    idx = np.arange(n_side, dtype=np.float64)
    gx, gy, gz = np.meshgrid(idx, idx, idx, indexing="ij")
    centre_off = (n_side - 1) * pitch / 2.0
    lo = np.array([-box[0] / 2, -box[1] / 2, 0.0])
    hi = np.array([box[0] / 2, box[1] / 2, box[2]])
    centre = (lo + hi) / 2.0
    n = n_side ** 3
    pos = np.empty((n, 4), dtype=np.float64)
    pos[:, 0] = (gx.ravel() * pitch - centre_off) + centre[0]
    pos[:, 1] = (gy.ravel() * pitch - centre_off) + centre[1]
    pos[:, 2] = (gz.ravel() * pitch - centre_off) + centre[2]
    pos[:, :3] += rng.uniform(-jitter, jitter, size=(n, 3))
    pos[:, 3] = radius
    planes, names = box_walls(lo, hi)
    cp = _default_property()
    return Scene(name="settle_box", seed=seed, dt=dt, steps=steps,
                 params=_reference_grid(radius, n, dt), pos=pos, **_state(pos), cp_pp=cp,
                 planes=planes, plane_names=names,
                 cp_planes=np.array([cp] * len(names), dtype=CONTACT_PROPERTY))


def _reject_overlaps(p: np.ndarray, r: np.ndarray, rmax: float) -> np.ndarray:
    """Greedy rejection: drop the later sphere of every overlapping pair."""
    from scipy.spatial import cKDTree
    tree = cKDTree(p)
    pairs = tree.query_pairs(2.0 * rmax, output_type="ndarray")
    keep = np.ones(p.shape[0], dtype=bool)
    if pairs.size:
        d = np.linalg.norm(p[pairs[:, 0]] - p[pairs[:, 1]], axis=1)
        bad = pairs[d < r[pairs[:, 0]] + r[pairs[:, 1]]]
        bad = bad[np.argsort(bad.max(axis=1), kind="stable")]
        for i, j in bad:
            if keep[i] and keep[j]:
                keep[max(i, j)] = False
    return keep


def polydisperse_box(n: int = 1_000_000, seed: int = 7, rmin: float = 0.002, rmax: float = 0.004,
                     box=(1.0, 1.0, 2.0), steps: int = 20_000, dt: float = 5.0e-6,
                     grid=(128, 128, 128)) -> Scene:
    """Polydisperse spheres, r ~ U[rmin, rmax], rejection-sampled without
    overlap in a box of plane walls (the 1,000,000-sphere settle scene).
    Smaller n keeps the same density by shrinking the box's x/y extent."""
    rng = _rng(seed)
    scale = (n / 1_000_000) ** 0.5
    bx, by, bz = box[0] * scale, box[1] * scale, box[2]
    lo = np.array([-bx / 2, -by / 2, 0.0])
    hi = np.array([bx / 2, by / 2, bz])
    pts = np.empty((0, 3))
    rad = np.empty((0,))
    rounds = 0
    while pts.shape[0] < n:
        rounds += 1
        if rounds > 200:
            raise ValueError("polydisperse_box: too dense for rejection sampling")
        m = int((n - pts.shape[0]) * 1.15) + 64
        r_new = rng.uniform(rmin, rmax, size=m)
        p_new = rng.uniform(0.0, 1.0, size=(m, 3)) * (hi - lo - 2 * r_new[:, None]) + lo + r_new[:, None]
        allp = np.concatenate([pts, p_new])
        allr = np.concatenate([rad, r_new])
        keep = _reject_overlaps(allp, allr, rmax)
        keep[: pts.shape[0]] = True
        pts, rad = allp[keep], allr[keep]
    pts, rad = pts[:n], rad[:n]
    pos = np.empty((n, 4), dtype=np.float64)
    pos[:, :3] = pts
    pos[:, 3] = rad
    planes, names = box_walls(lo, hi)
    cp = _default_property()
    return Scene(name="polydisperse_box", seed=seed, dt=dt, steps=steps,
                 params=_reference_grid(rmax, n, dt, grid=grid), pos=pos, **_state(pos),
                 cp_pp=cp, planes=planes, plane_names=names,
                 cp_planes=np.array([cp] * len(names), dtype=CONTACT_PROPERTY))


def lattice_box(n: int = 100_000, seed: int = 7, rmin: float = 0.002, rmax: float = 0.004,
                box=(1.0, 1.0, 2.0), steps: int = 20_000, dt: float = 5.0e-6) -> Scene:
    """The polydisperse settle's geometry and density (the box's x/y extent
    scaled by sqrt(n / 1e6) as in ``polydisperse_box``), with the spheres on
    a jittered cubic lattice instead of rejection-sampled: n random sites of
    a lattice that fills the box, r ~ U[rmin, rmax], each moved by at most
    pitch / 2 - r so that none overlap.  Generation is O(n) numpy (for the
    served request stream, which makes many such scenes)."""
    rng = _rng(seed)
    scale = (n / 1_000_000) ** 0.5
    ext = np.array([box[0] * scale, box[1] * scale, box[2]])
    lo = np.array([-ext[0] / 2, -ext[1] / 2, 0.0])
    pitch = (float(np.prod(ext)) / n) ** (1.0 / 3.0)
    while True:
        # sites at least pitch / 2 from every wall
        k = np.floor(ext / pitch).astype(int)
        if pitch < 2.04 * rmax:
            raise ValueError("lattice_box: box too small for n spheres")
        if int(np.prod(k)) >= n:
            break
        pitch *= 0.98
    start = lo + 0.5 * (ext - (k - 1) * pitch)
    pick = np.sort(rng.choice(int(np.prod(k)), size=n, replace=False))
    ix, iy, iz = np.unravel_index(pick, tuple(k))
    pts = start + np.stack([ix, iy, iz], axis=1) * pitch
    rad = rng.uniform(rmin, rmax, size=n)
    amp = np.minimum(0.5 * pitch - rad, rmax) / math.sqrt(3.0)
    pts = pts + rng.uniform(-1.0, 1.0, size=(n, 3)) * amp[:, None]
    pos = np.empty((n, 4), dtype=np.float64)
    pos[:, :3] = pts
    pos[:, 3] = rad
    planes, names = box_walls(lo, lo + ext)
    cp = _default_property()
    return Scene(name="lattice_box", seed=seed, dt=dt, steps=steps,
                 params=_reference_grid(rmax, n, dt), pos=pos, **_state(pos),
                 cp_pp=cp, planes=planes, plane_names=names,
                 cp_planes=np.array([cp] * len(names), dtype=CONTACT_PROPERTY))


def served_requests(count: int = 32, seed: int = 4, n_min: int = 1_000, n_max: int = 500_000,
                    steps_min: int = 1_000, steps_max: int = 20_000):
    """A request stream's scene parameters: geometry a settle box
    (``lattice_box``) or a hopper (``hopper``, orifice U[6, 12], friction
    U[0.2, 0.6]) with equal odds, particle count log-uniform in
    [n_min, n_max], step count uniform in [steps_min, steps_max].  Returns
    a list of dicts (kind, kwargs, steps)."""
    rng = _rng(seed)
    out = []
    for k in range(count):
        n = int(math.exp(rng.uniform(math.log(n_min), math.log(n_max))))
        steps = int(rng.integers(steps_min, steps_max + 1))
        if rng.uniform() < 0.5:
            out.append(dict(kind="box", kwargs=dict(n=n, seed=seed * 7919 + k), steps=steps))
        else:
            out.append(dict(kind="hopper", kwargs=dict(n=n, seed=seed * 7919 + k,
                                                       orifice=float(rng.uniform(6.0, 12.0)),
                                                       fric=float(rng.uniform(0.2, 0.6))),
                            steps=steps))
    return out


def make_request_scene(req) -> Scene:
    """The scene of one ``served_requests`` entry."""
    return lattice_box(**req["kwargs"]) if req["kind"] == "box" else hopper(**req["kwargs"])


def circumcentre(P, Q, R):
    """numeric::utility::calculate_center_of_triangle, as restated by the
    mesh-update kernel (mphysics_cuda_impl.cuh:1930-1951)."""
    V = Q - P
    W = R - P
    N = np.cross(V, W)
    N = N / np.linalg.norm(N, axis=-1, keepdims=True)
    M1 = 0.5 * (Q + P)
    M2 = 0.5 * (R + P)
    D1 = np.cross(N, V)
    D2 = np.cross(N, W)
    det_xy = D1[..., 0] * D2[..., 1] - D1[..., 1] * D2[..., 0]
    det_xz = D1[..., 0] * D2[..., 2] - D1[..., 2] * D2[..., 0]
    det_yz = D1[..., 1] * D2[..., 2] - D1[..., 2] * D2[..., 1]
    with np.errstate(divide="ignore", invalid="ignore"):
        t_xy = (D2[..., 0] * (M1[..., 1] - M2[..., 1])) / det_xy - (D2[..., 1] * (M1[..., 0] - M2[..., 0])) / det_xy
        t_xz = (D2[..., 0] * (M1[..., 2] - M2[..., 2])) / det_xz - (D2[..., 2] * (M1[..., 0] - M2[..., 0])) / det_xz
        t_yz = (D2[..., 1] * (M1[..., 2] - M2[..., 2])) / det_yz - (D2[..., 2] * (M1[..., 1] - M2[..., 1])) / det_yz
    t = np.where(np.abs(det_xy) > 1e-13, t_xy, np.where(np.abs(det_xz) > 1e-13, t_xz,
                 np.where(np.abs(det_yz) > 1e-13, t_yz, 0.0)))
    return M1 + t[..., None] * D1


def cylinder_mesh(radius: float, length: float, n_theta: int, n_z: int, n_ring: int):
    """Closed cylinder about the y axis, centred at the origin, wound so that
    (Q - P) x (R - P) points into the cylinder (the side the particles are
    on: the polygon contact pushes along that normal,
    mphysics_cuda_impl.cuh:985-987).  Side: n_theta x n_z quads; each cap:
    n_ring concentric rings with 6k vertices on ring k (6 n_ring^2 triangles)."""
    tris = []
    th = np.linspace(0.0, 2 * np.pi, n_theta + 1)[:-1]
    ys = np.linspace(-length / 2, length / 2, n_z + 1)
    for j in range(n_z):
        for i in range(n_theta):
            t0, t1 = th[i], th[(i + 1) % n_theta]
            a = np.array([radius * np.cos(t0), ys[j], radius * np.sin(t0)])
            b = np.array([radius * np.cos(t1), ys[j], radius * np.sin(t1)])
            c = np.array([radius * np.cos(t1), ys[j + 1], radius * np.sin(t1)])
            d = np.array([radius * np.cos(t0), ys[j + 1], radius * np.sin(t0)])
            tris.append((a, b, c))
            tris.append((a, c, d))

    def ring(k):
        if k == 0:
            return [np.zeros(2)]
        rr = radius * k / n_ring
        m = 6 * k
        ang = np.arange(m) * 2 * np.pi / m
        return [np.array([rr * np.cos(a), rr * np.sin(a)]) for a in ang]

    cap = []
    for k in range(n_ring):
        inner, outer = ring(k), ring(k + 1)
        if k == 0:
            for i in range(6):
                cap.append((inner[0], outer[i], outer[(i + 1) % 6]))
            continue
        ni, no = len(inner), len(outer)
        i = o = 0
        while i < ni or o < no:
            # advance along whichever polygon lags in angle
            ai = (i / ni) if i < ni else 2.0
            ao = (o / no) if o < no else 2.0
            if ao <= ai:
                cap.append((inner[i % ni], outer[o % no], outer[(o + 1) % no]))
                o += 1
            else:
                cap.append((inner[i % ni], outer[o % no], inner[(i + 1) % ni]))
                i += 1
    for (p, q, r) in cap:
        for y, flip in ((-length / 2, False), (length / 2, True)):
            P = np.array([p[0], y, p[1]])
            Q = np.array([q[0], y, q[1]])
            R = np.array([r[0], y, r[1]])
            tris.append((P, R, Q) if flip else (P, Q, R))
    tri = np.array(tris, dtype=np.float64)           # (T, 3, 3)
    # orient every triangle so that its normal points towards the axis / inside
    n = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
    cen = tri.mean(axis=1)
    inward = -cen.copy()
    side = np.abs(cen[:, 1]) < length / 2 - 1e-9
    inward[side, 1] = 0.0
    inward[~side] = 0.0
    inward[~side, 1] = -np.sign(cen[~side, 1])
    flip = np.einsum("ij,ij->i", n, inward) < 0
    tri[flip] = tri[flip][:, [0, 2, 1]]
    return tri


def drum(n: int = 4000, seed: int = 11, rmin: float = 0.003, rmax: float = 0.005,
         radius: float = 0.5, length: float = 0.4, omega: float = 1.0, n_theta: int = 242,
         n_z: int = 20, n_ring: int = 30, wall_friction: float = 0.5, steps: int = 50_000,
         dt: float = 5.0e-6, fill_height: float = None) -> Scene:
    """Spheres in a rotating closed drum of triangles (particle-polygon
    contacts).  The default mesh has 242 x 20 x 2 side triangles and two caps
    of 6 x 30^2, i.e. 20,480 triangles.  Spheres are rejection-sampled in the
    lower part of the drum; the drum spins about its (y) axis at ``omega``."""
    rng = _rng(seed)
    tri = cylinder_mesh(radius, length, n_theta, n_z, n_ring)
    T = tri.shape[0]
    cen = circumcentre(tri[:, 0], tri[:, 1], tri[:, 2])
    trad = np.linalg.norm(cen - tri[:, 0], axis=1)
    # sample particles in a slab at the bottom of the drum
    inner = radius - rmax - 0.002
    pts = np.empty((0, 3))
    rad = np.empty((0,))
    fh = fill_height if fill_height is not None else inner
    rounds = 0
    while pts.shape[0] < n:
        rounds += 1
        if rounds > 200:
            raise ValueError("drum: too dense for rejection sampling; raise fill_height")
        m = int((n - pts.shape[0]) * 1.3) + 64
        r_new = rng.uniform(rmin, rmax, size=m)
        x = rng.uniform(-inner, inner, size=m)
        z = rng.uniform(-inner, -inner + 2 * fh, size=m)
        y = rng.uniform(-length / 2 + rmax + 0.002, length / 2 - rmax - 0.002, size=m)
        ok = (x * x + z * z) < (inner * inner)
        p_new = np.stack([x, y, z], axis=1)[ok]
        r_new = r_new[ok]
        allp = np.concatenate([pts, p_new])
        allr = np.concatenate([rad, r_new])
        keep = _reject_overlaps(allp, allr, rmax)
        keep[: pts.shape[0]] = True
        pts, rad = allp[keep], allr[keep]
    pts, rad = pts[:n], rad[:n]
    pos = np.empty((n, 4), dtype=np.float64)
    pos[:, :3] = pts
    pos[:, 3] = rad
    poly = np.zeros(T, dtype=POLYGON)
    poly["id"] = 0
    poly["P"], poly["Q"], poly["R"] = tri[:, 0], tri[:, 1], tri[:, 2]
    poly["V"] = tri[:, 1] - tri[:, 0]
    poly["W"] = tri[:, 2] - tri[:, 0]
    poly["N"] = np.cross(poly["V"], poly["W"])
    sphere = np.empty((T, 4))
    sphere[:, :3] = cen
    sphere[:, 3] = trad
    pmi = np.zeros(1, dtype=POLYGON_MASS)
    pmi["ep"] = (1.0, 0.0, 0.0, 0.0)
    pmi["omega"] = (0.0, omega, 0.0)
    cp_wall = _default_property(fric=wall_friction)
    maxr = max(rmax, float(trad.max()))
    cp = _default_property()
    empty_planes, names = np.zeros(0, dtype=PLANE), []
    return Scene(name="drum", seed=seed, dt=dt, steps=steps,
                 params=_reference_grid(maxr, n, dt, nsphere=0), pos=pos, **_state(pos),
                 cp_pp=cp, planes=empty_planes, plane_names=names,
                 cp_planes=np.zeros(0, dtype=CONTACT_PROPERTY), poly=poly, sphere=sphere,
                 vlist=tri.reshape(T, 9).copy(), pmi=pmi,
                 cp_poly=np.array([cp_wall], dtype=CONTACT_PROPERTY))


def drum_lattice(n: int = 500_000, seed: int = 13, rmin: float = 0.002, rmax: float = 0.004,
                 radius: float = 0.5, length: float = 0.4, omega: float = 1.0, n_theta: int = 242,
                 n_z: int = 20, n_ring: int = 30, wall_friction: float = 0.5, dt: float = 5.0e-6,
                 steps: int = 50_000, slab: float = None) -> Scene:
    """The rotating drum at full size: ``n`` spheres on a jittered FCC lattice
    (nearest neighbours 2.04 r_max apart) filling the drum from the bottom, in
    the closed 20,480-triangle cylinder of ``drum`` turning at ``omega`` about
    its (y) axis.  Radii U[2, 4] mm: 500,000 such spheres settle to about a
    third of the drum's volume (mean sphere volume 1.26e-7 m^3, packing
    ~0.6); spheres of 3-5 mm would need 45 % of the drum as solid.  ``slab``
    fills only the lattice sites within slab / 2 of the drum's mid-plane
    (an axial slab of the bed, in the full mesh)."""
    rng = _rng(seed)
    tri = cylinder_mesh(radius, length, n_theta, n_z, n_ring)
    d = 2.04 * rmax
    a = d * math.sqrt(2.0)
    margin = rmax + 0.002
    rin, half = radius - margin, length / 2 - margin
    ks = np.arange(-int(rin / a) - 1, int(rin / a) + 2)
    ky = np.arange(-int(half / a) - 1, int(half / a) + 2)
    base = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    gx, gy, gz = np.meshgrid(ks, ky, ks, indexing="ij")
    cells = np.stack([gx.ravel(), gy.ravel(), gz.ravel()], axis=1).astype(np.float64)
    pts = (cells[:, None, :] + base[None, :, :]).reshape(-1, 3) * a
    ok = (pts[:, 0] ** 2 + pts[:, 2] ** 2 < rin * rin) & (np.abs(pts[:, 1]) < (half if slab is None else slab / 2))
    pts = pts[ok]
    if pts.shape[0] < n:
        raise ValueError(f"drum_lattice: {pts.shape[0]} lattice sites, {n} requested")
    order = np.lexsort((pts[:, 0], pts[:, 1], pts[:, 2]))     # from the bottom up
    pts = pts[order[:n]]
    pos = np.empty((n, 4), dtype=np.float64)
    pos[:, :3] = pts + rng.uniform(-0.01 * d, 0.01 * d, size=(n, 3))
    pos[:, 3] = rng.uniform(rmin, rmax, size=n)
    poly, sphere, vlist = _mesh_arrays(tri)
    pmi = np.zeros(1, dtype=POLYGON_MASS)
    pmi["ep"] = (1.0, 0.0, 0.0, 0.0)
    pmi["omega"] = (0.0, omega, 0.0)
    maxr = max(rmax, float(sphere[:, 3].max()))
    return Scene(name="drum_lattice", seed=seed, dt=dt, steps=steps,
                 params=_reference_grid(maxr, n, dt, nsphere=0), pos=pos, **_state(pos),
                 cp_pp=_default_property(), planes=np.zeros(0, dtype=PLANE), plane_names=[],
                 cp_planes=np.zeros(0, dtype=CONTACT_PROPERTY), poly=poly, sphere=sphere,
                 vlist=vlist, pmi=pmi,
                 cp_poly=np.array([_default_property(fric=wall_friction)], dtype=CONTACT_PROPERTY))


def euler_parameters_about_y(angle: float):
    """Euler parameters (e0, e1, e2, e3) of a rotation by ``angle`` about y."""
    return (math.cos(angle / 2), 0.0, math.sin(angle / 2), 0.0)


def cone_mesh(r_bottom: float, r_top: float, z_bottom: float, height: float, n_theta: int = 64,
              n_z: int = 32) -> np.ndarray:
    """Open cone frustum about the z axis from radius r_bottom at z_bottom to
    r_top at z_bottom + height: n_theta x n_z quads, two triangles each
    (64 x 32 x 2 = 4,096 by default), (T, 3, 3).  Every triangle is wound so
    that (Q - P) x (R - P) points towards the axis, the side the particles
    are on."""
    th = np.linspace(0.0, 2 * np.pi, n_theta + 1)[:-1]
    ct, st_ = np.cos(th), np.sin(th)
    tris = np.empty((n_z, n_theta, 2, 3, 3))
    for j in range(n_z):
        z0 = z_bottom + height * j / n_z
        z1 = z_bottom + height * (j + 1) / n_z
        r0 = r_bottom + (r_top - r_bottom) * j / n_z
        r1 = r_bottom + (r_top - r_bottom) * (j + 1) / n_z
        i1 = (np.arange(n_theta) + 1) % n_theta
        a = np.stack([r0 * ct, r0 * st_, np.full(n_theta, z0)], axis=1)
        b = np.stack([r0 * ct[i1], r0 * st_[i1], np.full(n_theta, z0)], axis=1)
        c = np.stack([r1 * ct[i1], r1 * st_[i1], np.full(n_theta, z1)], axis=1)
        d = np.stack([r1 * ct, r1 * st_, np.full(n_theta, z1)], axis=1)
        tris[j, :, 0] = np.stack([a, b, c], axis=1)
        tris[j, :, 1] = np.stack([a, c, d], axis=1)
    tri = tris.reshape(-1, 3, 3)
    n = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
    inward = -tri.mean(axis=1)
    inward[:, 2] = 0.0
    flip = np.einsum("ij,ij->i", n, inward) < 0
    tri[flip] = tri[flip][:, [0, 2, 1]]
    return tri


def _mesh_arrays(tri: np.ndarray, body: int = 0):
    """POLYGON records, circumspheres and body-frame vertex list of a mesh."""
    T = tri.shape[0]
    cen = circumcentre(tri[:, 0], tri[:, 1], tri[:, 2])
    trad = np.linalg.norm(cen - tri[:, 0], axis=1)
    poly = np.zeros(T, dtype=POLYGON)
    poly["id"] = body
    poly["P"], poly["Q"], poly["R"] = tri[:, 0], tri[:, 1], tri[:, 2]
    poly["V"] = tri[:, 1] - tri[:, 0]
    poly["W"] = tri[:, 2] - tri[:, 0]
    poly["N"] = np.cross(poly["V"], poly["W"])
    sphere = np.empty((T, 4))
    sphere[:, :3] = cen
    sphere[:, 3] = trad
    return poly, sphere, tri.reshape(T, 9).copy()


def hopper(n: int = 20_000, seed: int = 3, orifice: float = 8.0, fric: float = 0.4,
           rmin: float = 0.002, rmax: float = 0.004, wall_angle_deg: float = 60.0,
           n_theta: int = 64, n_z: int = 32, steps: int = 10_000, dt: float = 5.0e-6,
           packing: float = 0.25, gate: bool = False) -> Scene:
    """Hopper discharge: n spheres, r ~ U[rmin, rmax], on a jittered cubic
    lattice (no overlaps) inside a conical hopper whose wall rises at
    ``wall_angle_deg`` from the horizontal; the orifice (at z = 0) is
    ``orifice`` mean particle diameters wide and open, with a plane floor
    below it.  The cone is a fixed polygon body of n_theta x n_z x 2
    triangles; its top radius is chosen so that the spheres (the lattice
    pitch gives the packing fraction, at most ``packing``) fill the lower 60%
    of its volume.  Particle-particle friction is ``fric``, as is the wall's.
    ``gate`` adds a second plane that closes the orifice (z = 0), so that the
    spheres can fill and settle into a bed before the discharge;
    ``open_gate`` gives the planes with it moved out of the way."""
    rng = _rng(seed)
    d_mean = rmin + rmax
    r_o = 0.5 * orifice * d_mean
    slope = math.tan(math.radians(wall_angle_deg))
    mean_vol = math.pi * (rmax ** 4 - rmin ** 4) / (3.0 * (rmax - rmin))
    # jittered cubic lattice: pitch >= 2 rmax, so that no two spheres overlap
    pitch = max(2.04 * rmax, (mean_vol / packing) ** (1.0 / 3.0))
    sin_a = math.sin(math.radians(wall_angle_deg))
    margin = 0.05 * rmin

    def usable(rt):
        h = (rt - r_o) * slope
        return math.pi * h / 3.0 * (r_o * r_o + r_o * rt + rt * rt)

    def radius_holding(vol):
        lo_r, hi_r = r_o, 1.0
        while usable(hi_r) < vol:
            hi_r *= 2.0
        for _ in range(60):
            mid = 0.5 * (lo_r + hi_r)
            if usable(mid) >= vol:
                hi_r = mid
            else:
                lo_r = mid
        return hi_r

    def sites(r_fill):
        """Lattice sites of the cone below radius r_fill whose ball of
        radius pitch / 2 stays off the wall and above the orifice plane."""
        z_fill = (r_fill - r_o) * slope
        k = int(math.ceil(r_fill / pitch))
        g = np.arange(-k, k + 1) * pitch
        zs = np.arange(0.5 * pitch + margin, z_fill, pitch)
        X, Y, Z = np.meshgrid(g, g, zs, indexing="ij")
        p = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
        # the facets lie inside the smooth cone by up to r (1 - cos(pi / n_theta))
        inner = (r_o + p[:, 2] / slope) * math.cos(math.pi / n_theta)
        room = (inner - np.hypot(p[:, 0], p[:, 1])) * sin_a
        return p[room > 0.5 * pitch + margin]

    r_fill = radius_holding(n * pitch ** 3)
    cand = sites(r_fill)
    while cand.shape[0] < n:
        r_fill *= 1.03
        cand = sites(r_fill)
    r_top = max(radius_holding(usable(r_fill) / 0.6), r_fill + 2.0 * pitch)
    height = (r_top - r_o) * slope
    tri = cone_mesh(r_o, r_top, 0.0, height, n_theta, n_z)
    poly, sphere, vlist = _mesh_arrays(tri)
    # the lowest n sites (ties in lattice order), each with a random radius and
    # a jitter that keeps every pair apart: |shift| <= pitch / 2 - r
    order = np.argsort(cand[:, 2], kind="stable")[:n]
    pts = cand[np.sort(order)]
    rad = rng.uniform(rmin, rmax, size=n)
    amp = (0.5 * pitch - rad) / math.sqrt(3.0)
    pts = pts + rng.uniform(-1.0, 1.0, size=(n, 3)) * amp[:, None]
    pos = np.empty((n, 4), dtype=np.float64)
    pos[:, :3] = pts
    pos[:, 3] = rad
    pmi = np.zeros(1, dtype=POLYGON_MASS)
    pmi["ep"] = (1.0, 0.0, 0.0, 0.0)
    cp = _default_property(fric=fric)
    zf = -max(0.1, 10.0 * d_mean)
    w = r_top + 0.1
    floor = define_plane((-w, -w, zf), (w, -w, zf), (w, w, zf), (-w, w, zf))
    walls, names = [floor], ["floor"]
    if gate:
        g = r_o + 2.0 * rmax
        walls.append(define_plane((-g, -g, 0.0), (g, -g, 0.0), (g, g, 0.0), (-g, g, 0.0)))
        names.append("gate")
    planes = np.array(walls, dtype=PLANE)
    maxr = max(rmax, float(sphere[:, 3].max()))
    return Scene(name="hopper", seed=seed, dt=dt, steps=steps,
                 params=_reference_grid(maxr, n, dt), pos=pos, **_state(pos),
                 cp_pp=cp, planes=planes, plane_names=names,
                 cp_planes=np.array([cp] * len(names), dtype=CONTACT_PROPERTY), poly=poly,
                 sphere=sphere, vlist=vlist, pmi=pmi, cp_poly=np.array([cp], dtype=CONTACT_PROPERTY))


def open_gate(sc: Scene) -> np.ndarray:
    """The planes of a gated ``hopper`` with the gate moved 2 cm below the
    floor, where no sphere reaches it (the orifice open)."""
    planes = sc.planes.copy()
    k = sc.plane_names.index("gate")
    floor = planes[sc.plane_names.index("floor")]
    drop = np.array([0.0, 0.0, float(floor["xw"][2]) - 0.02])
    g = planes[k]
    planes[k] = define_plane(g["xw"] + drop, g["w2"] + drop, g["w3"] + drop, g["w4"] + drop)
    return planes


def hopper_batch(count: int = 256, seed: int = 1, n_min: int = 2_000, n_max: int = 200_000):
    """Parameters of a batch of independent hoppers: particle count
    log-uniform in [n_min, n_max], orifice U[6, 12] diameters, friction
    U[0.2, 0.6], one seed each.  Returns a list of keyword dicts for
    ``hopper``."""
    rng = _rng(seed)
    ns = np.exp(rng.uniform(math.log(n_min), math.log(n_max), size=count)).astype(np.int64)
    orif = rng.uniform(6.0, 12.0, size=count)
    mu = rng.uniform(0.2, 0.6, size=count)
    return [dict(n=int(ns[k]), seed=seed * 100_003 + k, orifice=float(orif[k]), fric=float(mu[k]))
            for k in range(count)]
