"""Model text files (metakonga_gb300.model_file) and the particle creators
(metakonga_gb300.creators): layouts against the reference's formulas worked
by hand, the reader against the writer, and the scene a model builds."""
import math

import numpy as np
import pytest

from metakonga_gb300 import creators, model_file
from metakonga_gb300.layouts import define_plane

from .cases import EMITTER_MODEL


def _rng():
    return np.random.Generator(np.random.MT19937(3))


def test_cube_creator_lattice():
    # 0.1 m cube, r = 4 mm: floor(0.1 / 0.008) - 1 = 11 per axis, gaps of
    # (0.1 - 11 * 0.008) / 12 = 1 mm, jitter below r * 1 mm = 4e-6 m
    c = creators.cube_particles(0.1, 0.1, 0.1, 0.0, 0.0, 0.0, 0.004, 0.004, _rng())
    assert c.pos.shape == (1331, 4) and c.groups == []
    lattice = 0.004 + 0.001 + np.arange(11) * 0.009
    # x fastest, then y, then z
    ix = np.arange(1331) % 11
    iz = np.arange(1331) // 121
    dx = c.pos[:, 0] - lattice[ix]
    dz = c.pos[:, 2] - lattice[iz]
    assert (dx >= 0).all() and (dx < 0.004 * 0.001 + 1e-15).all()
    assert (dz >= 0).all() and (dz < 0.004 * 0.001 + 1e-15).all()
    assert (c.pos[:, 3] == 0.004).all()
    # a polydisperse cube makes no particle in the reference
    assert creators.cube_particles(0.1, 0.1, 0.1, 0, 0, 0, 0.003, 0.004, _rng()).pos.shape == (0, 4)


def test_plane_creator_layers_and_groups():
    c = creators.plane_particles(0.1, 3, 0.05, 0.2, 0.5, -0.1, 0.004, 0.004, _rng())
    nx, nz = 11, 5          # floor(0.1 / 0.008) - 1, floor(0.05 / 0.008) - 1
    assert c.groups == [nx * nz] * 3 and c.pos.shape == (3 * nx * nz, 4)
    assert (c.pos[:, 1] == 0.5).all()                   # every layer at ly
    sx = (0.1 - 0.008 * nx) / (nx + 1)
    x0 = 0.2 + sx + (np.arange(3 * nx * nz) % nx) * (0.008 + sx)
    assert ((c.pos[:, 0] - x0) >= 0).all() and ((c.pos[:, 0] - x0) <= 100 * 0.004 * sx).all()
    poly = creators.plane_particles(0.1, 2, 0.1, 0, 0, 0, 0.002, 0.004, _rng())
    assert poly.pos[:, 3].min() >= 0.002 and poly.pos[:, 3].max() < 0.004


def test_circle_creator_rings():
    c = creators.circle_particles(0.1, 2, 0.0, 1.0, 0.0, 0.005, 0.005, _rng())
    # R = 0.05, d = 0.01: nr = 4 rings, space = (0.05 - 0.045) / 5 = 1 mm,
    # ring i: radius 0.011 i, floor(2 pi i) particles = 6, 12, 18, 25
    assert c.groups == [61, 61]
    assert c.pos.shape[0] == creators.circle_count(0.1, 2, 0.005) == 124
    layer = c.pos[:62]
    rad = np.hypot(layer[:, 0], layer[:, 2])
    assert rad[0] == 0.0
    np.testing.assert_allclose(np.sort(np.unique(np.round(rad[1:], 12))), 0.011 * np.arange(1, 5), rtol=1e-12)
    assert (c.pos[:, 1] == 1.0).all()


def test_reader_writer_round_trip():
    spec = model_file.read_model(EMITTER_MODEL)
    assert spec.name == "hopper_fill" and spec.gravity == (0.0, -9.80665, 0.0)
    assert [s["kind"] for s in spec.shapes] == ["plane"]
    s = spec.shapes[0]
    assert s["dim"] == (0.1, 6, 0.1) and s["making"]["per_time"] == 0.005 and s["making"]["realtime"] == 1
    assert sorted(spec.objects) == ["floor", "wall_x0", "wall_x1", "wall_z0", "wall_z1"]
    assert [c["name"] for c in spec.contacts] == ["pp", "p_floor", "p_wall0", "p_wall1", "p_wall2", "p_wall3"]
    again = model_file.read_model(model_file.write_model(spec))
    assert again.shapes == spec.shapes and again.objects == spec.objects
    assert sorted(again.contacts, key=lambda c: c["name"]) == sorted(spec.contacts, key=lambda c: c["name"])


def test_build_scene_walls_contacts_and_emitter():
    built = model_file.build_scene(model_file.read_model(EMITTER_MODEL), dt=1e-5, seed=1)
    sc = built.scene
    assert sc.np_ == 726
    assert built.emitter == {"period": 500, "groups": [121] * 6, "active": 0}
    # walls in contact-name order (p_floor < p_wall0 < ...), floor normal up
    assert sc.plane_names == ["p_floor", "p_wall0", "p_wall1", "p_wall2", "p_wall3"]
    ref = define_plane((0, 0, 0), (0, 0, 0.1), (0.1, 0, 0.1), (0.1, 0, 0))
    assert sc.planes[0].tobytes() == np.asarray(ref).tobytes()
    # steel walls (the table's 2e11): E_i is OBJECT0's, E_j OBJECT1's
    assert sc.cp_planes["Ej"][1] == 2e11 and sc.cp_planes["Ei"][2] == 2e11   # p_wall1 lists the wall first
    assert sc.cp_planes["rest"][0] == 0.6 and sc.cp_pp["rest"] == 0.7 and sc.cp_pp["sratio"] == 0.8
    # reference grid: 2 r_max cells from (-1, -1, -1), mass from the density
    assert sc.params["cell_size"] == 0.008 and tuple(sc.params["world_origin"]) == (-1.0, -1.0, -1.0)
    np.testing.assert_allclose(sc.mass[0], 2500.0 * (4.0 / 3.0) * math.pi * 0.004 ** 3.0, rtol=1e-15)
    np.testing.assert_array_equal(sc.force[:, 1], sc.mass * -9.80665)


def test_build_scene_cube_and_stl_polygon(tmp_path):
    stl = tmp_path / "tri.stl"
    # one square of two facets in millimetres
    stl.write_text("solid s\n"
                   " facet normal 0 0 1\n  outer loop\n   vertex 0 0 0\n   vertex 100 0 0\n   vertex 100 100 0\n"
                   "  endloop\n endfacet\n"
                   " facet normal 0 0 1\n  outer loop\n   vertex 0 0 0\n   vertex 100 100 0\n   vertex 0 100 0\n"
                   "  endloop\n endfacet\nendsolid s\n")
    text = f"""MODEL_NAME m
GRAVITY 0 0 -9.81
UNIT 0
SINGLE 0
PARTICLES_DATA
CREATE_SHAPE cube
NAME c
MATERIAL_TYPE 6
DIMENSION 0.05 0.05 0.05
STARTPOINT 0.01 0.01 0.01
SPACE 0
RADIUS 0.005 0.005
MATERIAL 0 0 0 0
END_DATA
GEOMETRY_OBJECTS_DATA
OBJECT cube
NAME box
MATERIAL_TYPE 7
GEOMETRY_USE 0
START_POINT 0 0 0
END_POINT 0.1 0.2 0.3
MATERIAL 5e6 0.25 1000 0
OBJECT polygon
NAME plate
FILE {stl}
CM 0.05 0.05 0
MATERIAL_TYPE 0
GEOMETRY_USE 0
IMPORT_SHAPE_TYPE 2
MATERIAL 0 0 0 0
TOOL none none 0
END_DATA
CONTACT_ELEMENTS_DATA
NAME a_box
METHOD 1
OBJECT0 particles
OBJECT1 box
RESTITUTION 0.5
RATIO 0.7
FRICTION 0.2
COHESION 0
NAME b_plate
METHOD 1
OBJECT0 particles
OBJECT1 plate
RESTITUTION 0.4
RATIO 0.8
FRICTION 0.5
COHESION 0
END_DATA
"""
    built = model_file.build_scene(model_file.read_model(text), dt=1e-5)
    sc = built.scene
    assert built.emitter is None
    assert sc.np_ == 64                          # floor(0.05 / 0.01) - 1 = 4 per axis
    # sand density (the table's)
    np.testing.assert_allclose(sc.mass[0], 2600.0 * (4.0 / 3.0) * math.pi * 0.005 ** 3.0, rtol=1e-15)
    # the cube's six three-point planes: sizes 0.1, 0.2, 0.3, corner info zero
    assert sc.planes.shape == (6,) and sc.plane_names[0] == "a_box[0]"
    assert sorted(np.round(np.concatenate([sc.planes["l1"], sc.planes["l2"]]), 12).tolist()) == \
        sorted([0.3, 0.1, 0.2, 0.3, 0.3, 0.2, 0.1, 0.2, 0.2, 0.1, 0.1, 0.3])
    assert (sc.planes["w2"] == 0).all() and (sc.planes["w4"] == 0).all()
    assert sc.cp_planes["Ej"][0] == 5e6 and sc.cp_planes["prj"][0] == 0.25
    # STL in millimetres -> metres; body frame relative to CM; steel table
    assert sc.ntri == 2 and sc.pmi.shape == (1,)
    np.testing.assert_array_equal(sc.poly["R"][0], (0.1, 0.1, 0.0))
    np.testing.assert_allclose(sc.vlist[0, 3:6], (0.05, -0.05, 0.0), rtol=0, atol=1e-17)
    assert tuple(sc.pmi["origin"][0]) == (0.05, 0.05, 0.0) and sc.cp_poly["Ej"][0] == 2e11
    assert sc.params["nsphere"] == 2


def test_refusals():
    spec = model_file.read_model(EMITTER_MODEL.replace("MAKING 1 726 0 0.005 0 none", "MAKING 1 726 3 0.005 1 none"))
    with pytest.raises(ValueError, match="divides"):
        model_file.build_scene(spec, dt=1e-5)
    with pytest.raises(ValueError, match="material type"):
        model_file.material(42, 0, 0, 0, 0)
