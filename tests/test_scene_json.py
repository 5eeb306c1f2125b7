"""CPU tests of the scene-file loader (the reference's JSON scene layout, Simulator::loadScene in
src/intf/simulator.cpp:250-594): defaults, value types, rotations, skipped and unsupported bodies,
and the ignore-collision flag as the oracle's broadphase sees it.  The reference's sample scenes
are read only where the reference tree is present."""
import json
from pathlib import Path

import numpy as np
import pytest

import build_ref
import orc
from pe_gb300 import scene as sc
from pe_gb300.scene_json import UnsupportedScene, load_scene_json

_REF = build_ref.reference_dir()
SAMPLES = (_REF / "SampleScenes") if _REF is not None else Path("reference-sample-scenes-not-present")


def write(tmp_path, doc):
    p = tmp_path / "scene.json"
    p.write_text(json.dumps(doc))
    return p


def test_defaults_of_a_bare_box(tmp_path):
    s, ignored = load_scene_json(write(tmp_path, {"RigidBodies": [{"type": "box"}]}))
    assert s.n_bodies == 1 and ignored == []
    assert s.shape_type[0] == sc.BOX
    np.testing.assert_array_equal(s.shape_param[0], [1, 1, 1])
    assert (s.mass[0], s.friction[0], s.restitution[0], s.lin_damp[0], s.ang_damp[0]) == (1.0, 0.5, 0.5, 0.0, 0.0)
    np.testing.assert_array_equal(s.origin[0], [0, 0, 0])
    np.testing.assert_array_equal(s.basis[0], np.eye(3))
    assert s.gravity == (0.0, -9.8, 0.0)
    assert s.dt == pytest.approx(1 / 60) and s.iterations == 10


def test_configuration_and_integer_numbers(tmp_path):
    doc = {"Configuration": {"gravity": [0, -10, 1]},
           "RigidBodies": [{"type": "box", "mass": 3, "position": [1, 2, 3], "scale": [2, 4, 6], "friction": 1}]}
    s, _ = load_scene_json(write(tmp_path, doc))
    assert s.gravity == (0.0, -10.0, 1.0)
    assert s.mass[0] == 3.0 and s.friction[0] == 1.0
    np.testing.assert_array_equal(s.origin[0], [1, 2, 3])
    np.testing.assert_array_equal(s.shape_param[0], [2, 4, 6])


def test_kinematic_bodies_keep_zero_velocity_and_damping(tmp_path):
    body = {"type": "box", "linear_velocity": [1, 2, 3], "angular_velocity": [4, 5, 6], "linear_damping": 0.3,
            "angular_damping": 0.7}
    s, _ = load_scene_json(write(tmp_path, {"RigidBodies": [dict(body, kinematic=True), dict(body, kinematic=False)]}))
    assert s.body_flags[0] & sc.KINEMATIC and not s.body_flags[1] & sc.KINEMATIC
    np.testing.assert_array_equal(s.lin_vel[0], 0)
    np.testing.assert_array_equal(s.ang_vel[0], 0)
    assert (s.lin_damp[0], s.ang_damp[0]) == (0.0, 0.0)
    np.testing.assert_array_equal(s.lin_vel[1], [1, 2, 3])
    np.testing.assert_array_equal(s.ang_vel[1], [4, 5, 6])
    assert (s.lin_damp[1], s.ang_damp[1]) == (0.3, 0.7)


def test_rotations_row_major_matrix_and_quaternion(tmp_path):
    m = [0, -1, 0, 1, 0, 0, 0, 0, 1]
    h = np.sqrt(0.5)
    doc = {"RigidBodies": [{"type": "box", "rotation": m}, {"type": "box", "rotation": [h, 0, 0, h]}]}
    s, _ = load_scene_json(write(tmp_path, doc))
    np.testing.assert_array_equal(s.basis[0], np.array(m, float).reshape(3, 3))
    # (w, x, y, z) = 90 degrees about z
    np.testing.assert_allclose(s.basis[1], [[0, -1, 0], [1, 0, 0], [0, 0, 1]], atol=1e-15)
    np.testing.assert_array_equal(s.basis[1], sc.quat_to_basis(np.array([h, 0, 0, h])))


def test_sphere_and_cylinder_sizes(tmp_path):
    doc = {"RigidBodies": [{"type": "sphere", "scale": [1.2]}, {"type": "sphere"}, {"type": "cylinder", "scale": [0.3, 2]},
                           {"type": "cylinder"}]}
    s, _ = load_scene_json(write(tmp_path, doc))
    assert list(s.shape_type[s.body_shape]) == [sc.SPHERE, sc.SPHERE, sc.CYLINDER, sc.CYLINDER]
    p = s.shape_param[s.body_shape]
    assert p[0][0] == 1.2 and p[1][0] == 1.0
    assert tuple(p[2][:2]) == (0.3, 2.0) and tuple(p[3][:2]) == (0.5, 1.0)


@pytest.mark.parametrize("body", [
    {"type": "box", "scale": [1, 2]},                 # wrong length
    {"type": "sphere", "scale": [1, 2]},
    {"type": "box", "mass": "heavy"},                 # wrong type
    {"type": "box", "mass": True},                    # a boolean is not a number
    {"type": "box", "kinematic": 1},                  # a number is not a boolean
    {"type": "box", "position": [0, "a", 0]},         # non-numeric element
    {"type": "box", "rotation": [1, 0, 0]},           # neither matrix nor quaternion
    {"type": "box", "linear_velocity": 3},            # not an array
    {"type": 7},                                       # type must be a string
    {"type": "box", "tag": 5},
])
def test_malformed_values_raise(tmp_path, body):
    with pytest.raises(ValueError):
        load_scene_json(write(tmp_path, {"RigidBodies": [body]}))


def test_unknown_or_missing_types_are_skipped(tmp_path):
    doc = {"RigidBodies": [{"type": "box"}, {"type": "capsule"}, {"mass": 2}, {"type": "sphere"}]}
    s, ignored = load_scene_json(write(tmp_path, doc))
    assert s.n_bodies == 2
    assert list(s.shape_type[s.body_shape]) == [sc.BOX, sc.SPHERE]
    assert any("capsule" in x for x in ignored) and any("no type" in x for x in ignored)


TETRA = """# a tetrahedron
v 0 0 0
v 1 0 0
vt 0.5 0.5
v 0 1 0
v 0 0 1
vn 0 0 1
f 1/1/1 3/1/1 2/1/1
f 1//1 2//1 4//1
f 1 4 3
f 2 3 4
"""


@pytest.mark.parametrize("kind", ["convex", "concave"])
def test_mesh_bodies_read_obj_files(tmp_path, kind):
    """Mesh::loadFromObj: "v" lines (every coordinate times scale[0]), "f" corners before the first
    '/', 1-based; a path is tried relative to the scene file as well."""
    (tmp_path / "tet.obj").write_text(TETRA)
    doc = {"RigidBodies": [{"type": kind, "mesh": "tet.obj", "scale": [2, 5, 7], "position": [0, 3, 0]}]}
    s, ignored = load_scene_json(write(tmp_path, doc))
    assert ignored == [] and s.n_bodies == 1
    assert s.shape_type[s.body_shape[0]] == (sc.HULL if kind == "convex" else sc.CONCAVE)
    np.testing.assert_array_equal(s.hull_verts, [[0, 0, 0], [2, 0, 0], [0, 2, 0], [0, 0, 2]])
    assert s.hull_vcnt[s.body_shape[0]] == 4 and s.hull_fcnt[s.body_shape[0]] == 4
    np.testing.assert_array_equal(s.hull_face_idx[:6], [0, 2, 1, 0, 1, 3])


def test_obj_coordinates_in_float_precision(tmp_path):
    """For a 32-bit world the product is formed in float, as the reference's float build does."""
    (tmp_path / "m.obj").write_text("v 0.1 0.2 0.3\nv 1 0 0\nv 0 1 0\nf 1 2 3\n")
    s, _ = load_scene_json(write(tmp_path, {"RigidBodies": [{"type": "convex", "mesh": "m.obj", "scale": [0.7, 1, 1]}]}),
                           real_bits=32)
    assert s.hull_verts[0, 0] == float(np.float32(np.float32("0.1") * np.float32(0.7)))


@pytest.mark.parametrize("kind", ["convex", "concave"])
def test_mesh_bodies_without_file_are_skipped(tmp_path, kind):
    doc = {"RigidBodies": [{"type": "box"}, {"type": kind, "mesh": "missing.obj"}, {"type": kind}]}
    s, ignored = load_scene_json(write(tmp_path, doc))
    assert s.n_bodies == 1
    assert any("mesh file not found" in x for x in ignored) and any("mesh path not specified" in x for x in ignored)


def test_compound_bodies(tmp_path):
    """Sub-shapes in file order with their mass ratios (default 1), positions and rotations; the
    body origin moves by the rotated centroid so that init()'s relocation keeps every child in
    place."""
    rz = [0, -1, 0, 1, 0, 0, 0, 0, 1]
    doc = {"RigidBodies": [{"type": "compound", "position": [1, 2, 3], "rotation": rz, "mass": 2.0, "shapes": [
        {"type": "box", "scale": [1, 2, 3], "mass_ratio": 0.5},
        {"type": "sphere", "scale": [0.5], "position": [2, 0, 0]},
        {"type": "cylinder", "scale": [0.2, 1], "position": [0, 1, 0], "rotation": [1, 0, 0, 0], "mass_ratio": 0.5}]}]}
    s, ignored = load_scene_json(write(tmp_path, doc))
    assert ignored == [] and s.n_bodies == 1
    c = s.body_shape[0]
    assert s.shape_type[c] == sc.COMPOUND and s.cmp_cnt[c] == 3
    kids = s.child_shape[s.cmp_beg[c]:s.cmp_beg[c] + 3]
    assert list(s.shape_type[kids]) == [sc.BOX, sc.SPHERE, sc.CYLINDER]
    np.testing.assert_array_equal(s.child_ratio, [0.5, 1.0, 0.5])
    np.testing.assert_array_equal(s.child_origin, [[0, 0, 0], [2, 0, 0], [0, 1, 0]])
    centroid = np.array([2.0, 0.5, 0.0]) / 2.0
    np.testing.assert_allclose(s.origin[0], np.array([1, 2, 3]) + np.array(rz, float).reshape(3, 3) @ centroid)
    # a body written back and read again keeps its children
    p = tmp_path / "s.pescene"
    s.write(p)
    t = sc.Scene.read(p)
    np.testing.assert_array_equal(t.child_shape, s.child_shape)
    np.testing.assert_array_equal(t.child_basis, s.child_basis)


@pytest.mark.parametrize("sub, err", [({"type": "convex", "mesh": "a.obj", "scale": [1, 1, 1]}, UnsupportedScene),
                                      ({"type": "convex", "mesh": "a.obj"}, ValueError), ({"type": "convex"}, ValueError),
                                      ({"type": "compound"}, ValueError), ({"type": "concave"}, ValueError),
                                      ({"type": "capsule"}, ValueError), ({"scale": [1, 1, 1]}, ValueError),
                                      ({"type": "box", "mass_ratio": 0.0}, ValueError),
                                      ({"type": "box", "position": [0, 0]}, ValueError)])
def test_invalid_compound_sub_shapes(tmp_path, sub, err):
    with pytest.raises(err):
        load_scene_json(write(tmp_path, {"RigidBodies": [{"type": "compound", "shapes": [{"type": "box"}, sub]}]}))


def test_compound_without_sub_shapes_is_skipped(tmp_path):
    s, ignored = load_scene_json(write(tmp_path, {"RigidBodies": [{"type": "compound"}, {"type": "box"}]}))
    assert s.n_bodies == 1 and any("compound without sub-shapes" in x for x in ignored)


def test_unmodelled_features_are_reported(tmp_path):
    doc = {"Configuration": {"sleep_time_threshold": 1.0},
           "RigidBodies": [{"type": "box", "fracturable": True, "tag": "wheel", "lifetime": 5.0},
                           {"type": "box", "lifetime": -1}],
           "DamageSources": [{"type": "sphere"}]}
    s, ignored = load_scene_json(write(tmp_path, doc))
    assert s.n_bodies == 2
    text = " | ".join(ignored)
    for word in ("sleep_time_threshold", "fracturable", "wheel", "lifetime 5", "DamageSources"):
        assert word in text
    assert "body 1" not in text   # a negative lifetime means forever


def test_ignore_collision_bodies_make_no_pairs_in_the_oracle(tmp_path):
    """Three overlapping unit boxes; the middle one ignores collisions -> only the outer pair."""
    bodies = [{"type": "box", "position": [0, 0.6 * i, 0], "ignore_collision": i == 1} for i in range(3)]
    bodies[2]["position"] = [0, 0.9, 0]
    s, _ = load_scene_json(write(tmp_path, {"RigidBodies": bodies}))
    assert list(s.body_flags) == [0, sc.IGNORE_COLLISION, 0]
    for bits in (32, 64):
        w = orc.OracleWorld(s, bits)
        w.integrate()
        assert w.broadphase() == 1
        assert sorted(w.pairs()[0]) == [0, 2]


def test_scene_file_round_trip_keeps_flags(tmp_path):
    doc = {"RigidBodies": [{"type": "box", "kinematic": True, "ignore_collision": True}, {"type": "sphere"}]}
    s, _ = load_scene_json(write(tmp_path, doc), real_bits=32)
    p = tmp_path / "s.pescene"
    s.write(p)
    t = sc.Scene.read(p, real_bits=32)
    assert list(t.body_flags) == [sc.KINEMATIC | sc.IGNORE_COLLISION, 0]
    assert t.dt == s.dt and t.gravity == s.gravity


@pytest.mark.skipif(not SAMPLES.is_dir(), reason="reference sample scenes not present")
def test_reference_sample_scenes():
    s, ignored = load_scene_json(SAMPLES / "bomb_crash_tower_smaller.json")
    assert s.n_bodies == 17 and s.body_flags[0] & sc.KINEMATIC
    assert s.shape_type[s.body_shape[-1]] == sc.SPHERE and s.mass[-1] == 50.0
    np.testing.assert_array_equal(s.lin_vel[-1], [0, 0, -70])
    s, _ = load_scene_json(SAMPLES / "bomb_crash_tower.json")
    assert s.n_bodies == 2022 and (s.shape_type[s.body_shape] == sc.BOX).sum() == 2021
    s, ignored = load_scene_json(SAMPLES / "urban_combat_layout.json")
    assert s.n_bodies == 401 and any("fracturable" in x for x in ignored)
    s, _ = load_scene_json(SAMPLES / "compound_smaller.json")
    assert s.n_bodies == 3 and s.n_children == 7
    s, _ = load_scene_json(SAMPLES / "compound.json")
    assert s.n_bodies == 14 and (s.shape_type[s.body_shape] == sc.COMPOUND).sum() == 10
    s, ignored = load_scene_json(SAMPLES / "standford_bunny_smaller.json")   # its OBJ file is not shipped
    assert s.n_bodies == 5 and any("mesh file not found" in x for x in ignored)
