"""Scene files in the reference's JSON layout (Simulator::loadScene, src/intf/simulator.cpp:250-594).

``load_scene_json(path)`` reads the ``Configuration`` block (gravity) and the ``RigidBodies`` list
into a ``Scene`` for the GPU world, following the reference loader's rules:

* a value is used only when its key is present and not null; numbers may be integers or floats;
  an array of the wrong length or a value of the wrong type is an error
  (simulator.cpp:27-66, jsonNodeExists / jsonArrayExists);
* ``kinematic`` bodies keep zero velocities: damping and velocities are read for dynamic bodies only
  (:348-354);
* ``rotation`` is a row-major 3x3 matrix (9 numbers) or a quaternion (w, x, y, z) (:362-375);
* ``type``: ``box`` size = ``scale`` (3 numbers, default 1, 1, 1), ``sphere`` radius = ``scale[0]``
  (1 number, default 1), ``cylinder`` radius, height = ``scale`` (2 numbers, default 0.5, 1)
  (:379-395);
* RigidBody defaults where a key is absent: mass 1, friction 0.5, restitution 0.5, no damping
  (rigidbody.cpp:87-103).

* a body without a ``type``, or with a type the loader does not know, is skipped (:535-545).

* ``compound`` bodies take their children from ``shapes`` (:438-531).  The reference loader never
  calls ``CompoundShape::init()``, which leaves the compound's inertia uninitialised; here every
  consumer runs ``init()`` (children relocated to their mass-ratio centroid, inertia from the
  children) and the loader moves the body origin by the rotated centroid, so each child stays
  where the file places it.

* ``convex`` / ``concave`` bodies (and convex compound sub-shapes) read the OBJ file named by
  ``mesh`` (Mesh::loadFromObj, every coordinate scaled by ``scale[0]`` as the reference does); a
  path that does not exist relative to the working directory is tried relative to the scene
  file, and a body whose file is missing is skipped, as the reference skips it (:412-416).

What the rigid-body step here does not model is reported rather than silently dropped:
fracturable bodies step as plain
rigid bodies and ``DamageSources`` are not applied (no fracture solver), and sleep thresholds,
finite lifetimes and tags are ignored (sleeping, lifetimes and the "wheel" tag are not on the
path).  These, and the skipped bodies, are listed in ``ignored``.

The time step is not part of the file: the reference simulator uses 1 / target frame rate (60 by
default, simulator.cpp:1043), and the sequential-impulse solver 10 iterations
(sequential_impulse_solver.cpp:8).
"""
from __future__ import annotations

import json
from numbers import Number
from pathlib import Path

import numpy as np

from .scene import BOX, CONCAVE, CYLINDER, HULL, SPHERE, SceneBuilder, quat_to_basis


class UnsupportedScene(ValueError):
    pass


def _present(node, key):
    return isinstance(node, dict) and key in node and node[key] is not None


def _number(node, key):
    if not _present(node, key):
        return None
    v = node[key]
    if isinstance(v, bool) or not isinstance(v, Number):
        raise ValueError(f"node {key} should be a number")
    return float(v)


def _boolean(node, key):
    if not _present(node, key):
        return None
    v = node[key]
    if not isinstance(v, bool):
        raise ValueError(f"node {key} should be a boolean")
    return v


def _string(node, key):
    if not _present(node, key):
        return None
    v = node[key]
    if not isinstance(v, str):
        raise ValueError(f"node {key} should be a string")
    return v


def _list(node, key):
    if not _present(node, key):
        return None
    if not isinstance(node[key], list):
        raise ValueError(f"node {key} should be an array")
    return node[key]


def _array(node, key, size):
    if not _present(node, key):
        return None
    v = node[key]
    if not isinstance(v, list):
        raise ValueError(f"node {key} should be an array")
    if size and len(v) != size:
        raise ValueError(f"node {key} should have {size} elements")
    for x in v:
        if isinstance(x, bool) or not isinstance(x, Number):
            raise ValueError(f"node {key} should have numeric elements")
    return [float(x) for x in v]


def _atoi(tok):
    """C atoi: optional sign and leading digits, 0 when there are none."""
    tok = tok.lstrip()
    k = 1 if tok[:1] in ("+", "-") else 0
    while k < len(tok) and tok[k].isdigit():
        k += 1
    digits = tok[:k]
    return int(digits) if digits not in ("", "+", "-") else 0


def load_obj(path, scale_x=1.0, real_bits=64):
    """Mesh::loadFromObj (common/mesh.cpp:36-67): "v" lines give vertices, every coordinate
    multiplied by the first scale component (the reference scales y and z by size.x() too), in the
    world's precision; "f" lines give faces from the index before the first '/' of each corner,
    1-based.  Returns (vertices [n,3], faces)."""
    verts, faces = [], []
    f32 = real_bits == 32
    sx = np.float32(scale_x) if f32 else float(scale_x)
    for line in Path(path).read_text().splitlines():
        parts = line[:1023].split()
        if not parts:
            continue
        if parts[0] == "v":
            xyz = parts[1:4]
            if f32:
                verts.append([float(np.float32(np.float32(v) * sx)) for v in xyz])
            else:
                verts.append([float(v) * sx for v in xyz])
        elif parts[0] == "f":
            faces.append([_atoi(t.split("/")[0]) - 1 for t in parts[1:]])
    for f in faces:
        if len(f) < 3:
            raise ValueError(f"{path}: invalid mesh face: less than 3 vertices")
    return np.array(verts, np.float64).reshape(-1, 3), faces


def _mesh_path(node, base):
    p = _string(node, "mesh")
    if p is None:
        return None
    q = Path(p)
    if not q.exists() and not q.is_absolute() and base is not None and (base / q).exists():
        q = base / q   # relative to the scene file when not found relative to the working directory
    return q


def _rotation(node, where):
    rot = _array(node, "rotation", 0)
    if rot is None:
        return np.eye(3)
    if len(rot) >= 9:
        return np.array(rot[:9]).reshape(3, 3)
    if len(rot) >= 4:
        return quat_to_basis(np.array(rot[:4]))
    raise ValueError(f"{where}: invalid rotation data")


def _primitive(sb, node, kind):
    """box / sphere / cylinder shape of a body or compound sub-shape (simulator.cpp:379-395, :472-490)."""
    if kind == "box":
        return sb.shape(BOX, _array(node, "scale", 3) or [1.0, 1.0, 1.0])
    if kind == "sphere":
        r = _array(node, "scale", 1)
        return sb.shape(SPHERE, (r[0] if r else 1.0,))
    return sb.shape(CYLINDER, _array(node, "scale", 2) or [0.5, 1.0])


def _compound(sb, rb, idx, base=None, real_bits=64):
    """CompoundShape from the "shapes" list (simulator.cpp:438-531): per sub-shape a mass ratio
    (default 1), a position (3 numbers), a rotation and a box / sphere / cylinder type with the
    body rules for "scale".  The reference deletes the body and goes on iterating its sub-shapes
    when a sub-shape is invalid (a use after free); here such a file is an error."""
    kids = _list(rb, "shapes")
    if kids is None:
        return None
    children = []
    for k, node in enumerate(kids):
        where = f"body {idx} sub-shape {k}"
        if not isinstance(node, dict):
            raise ValueError("node shapes should have elements of type object")
        ratio = _number(node, "mass_ratio")
        pos = _array(node, "position", 3) or [0.0, 0.0, 0.0]
        rot = _rotation(node, where)
        sub = _string(node, "type")
        if sub == "convex":   # simulator.cpp:492-503: the scale is read unchecked
            mp = _mesh_path(node, base)
            if mp is None:
                raise ValueError(f"{where}: convex sub-shape mesh path not specified")
            sc = _array(node, "scale", 3)
            if sc is None:
                raise ValueError(f"{where}: convex sub-shape needs a scale")
            if not mp.exists():
                raise UnsupportedScene(f"{where}: mesh file not found: {mp}")
            shape = sb.shape(HULL, hull=load_obj(mp, sc[0], real_bits))
        elif sub in ("compound", "concave"):
            raise ValueError(f"{where}: compound sub-shapes cannot be compound or concave")
        elif sub not in ("box", "sphere", "cylinder"):
            raise ValueError(f"{where}: invalid compound sub-shape type {sub!r}")
        else:
            shape = _primitive(sb, node, sub)
        children.append((shape, pos, rot, 1.0 if ratio is None else ratio))
    if not children:
        raise ValueError(f"body {idx}: a compound needs at least one sub-shape")
    return sb.compound(children)


def load_scene_json(path, real_bits: int = 64, dt: float = 1.0 / 60.0, iterations: int = 10):
    """Returns (Scene, ignored): the scene and the list of file features the step does not model."""
    data = json.loads(Path(path).read_text())
    base = Path(path).resolve().parent
    gravity = (0.0, -9.8, 0.0)
    ignored = []
    if not isinstance(data, dict):
        raise ValueError("a scene file holds one JSON object")
    cfg = data.get("Configuration")
    if _present(data, "Configuration"):
        if not isinstance(cfg, dict):
            raise ValueError("node Configuration should be an object")
        g = _array(cfg, "gravity", 3)
        if g is not None:
            gravity = tuple(g)
        for k in ("sleep_linear_velocity2_threshold", "sleep_angular_velocity2_threshold", "sleep_time_threshold"):
            v = _number(cfg, k)
            if v:
                ignored.append(f"{k}={v:g} (no sleeping)")
    sb = SceneBuilder(dt=dt, gravity=gravity, iterations=iterations)
    bodies = _list(data, "RigidBodies") or []
    if _list(data, "DamageSources"):
        ignored.append("DamageSources (no fracture solver)")
    for idx, rb in enumerate(bodies):
        if not isinstance(rb, dict):
            raise ValueError("node RigidBodies should have elements of type object")
        kind = _string(rb, "type")
        if _boolean(rb, "fracturable"):
            ignored.append(f"body {idx}: fracturable (stepped as a rigid body)")
        _string(rb, "name")
        tag = _string(rb, "tag")
        if tag:
            ignored.append(f"body {idx}: tag '{tag}'")
        life = _number(rb, "lifetime")   # negative means forever (simulator.cpp:356-360)
        if life is not None and 0 <= life < 1e100:
            ignored.append(f"body {idx}: lifetime {life:g}")
        kinematic = bool(_boolean(rb, "kinematic"))
        ignore_collision = bool(_boolean(rb, "ignore_collision"))
        ld = ad = 0.0
        v = w = (0.0, 0.0, 0.0)
        if not kinematic:
            ld = _number(rb, "linear_damping") or 0.0
            ad = _number(rb, "angular_damping") or 0.0
            v = _array(rb, "linear_velocity", 3) or v
            w = _array(rb, "angular_velocity", 3) or w
        pos = _array(rb, "position", 0) or [0.0, 0.0, 0.0]
        if len(pos) < 3:
            raise ValueError(f"body {idx}: node position should have at least 3 elements")
        basis = _rotation(rb, f"body {idx}")
        mass = _number(rb, "mass")
        fr = _number(rb, "friction")
        re = _number(rb, "restitution")
        if kind not in ("box", "sphere", "cylinder", "compound", "convex", "concave"):
            # the reference logs the body and goes on without it (simulator.cpp:535-545)
            ignored.append(f"body {idx}: type {kind!r} (body skipped)" if kind else f"body {idx}: no type (body skipped)")
            continue
        origin = np.array(pos[:3])
        if kind in ("convex", "concave"):   # simulator.cpp:407-437: an OBJ mesh scaled by scale[0]
            mp = _mesh_path(rb, base)
            if mp is None:
                ignored.append(f"body {idx}: mesh path not specified (body skipped)")
                continue
            if not mp.exists():
                ignored.append(f"body {idx}: mesh file not found: {mp} (body skipped)")
                continue
            sc = _array(rb, "scale", 3) or [1.0, 1.0, 1.0]
            shape = sb.shape(HULL if kind == "convex" else CONCAVE, hull=load_obj(mp, sc[0], real_bits))
        elif kind == "compound":
            shape = _compound(sb, rb, idx, base, real_bits)
            if shape is None:
                ignored.append(f"body {idx}: compound without sub-shapes (body skipped)")
                continue
            # init() relocates the children to their centroid; the body origin moves with them so
            # that every child stays where the file puts it
            origin = origin + basis @ sb.compound_centroid(shape)
        else:
            shape = _primitive(sb, rb, kind)
        sb.body(shape, origin, basis, mass=1.0 if mass is None else mass, v=v, w=w,
                friction=0.5 if fr is None else fr, restitution=0.5 if re is None else re, kinematic=kinematic,
                lin_damp=ld, ang_damp=ad, ignore_collision=ignore_collision)
    return sb.build(real_bits), ignored
