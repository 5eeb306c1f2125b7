"""Scene description, the ``.pescene`` file format, and seeded synthetic scene generators.

A scene is what a caller hands to ``pe_intf::World`` before stepping it
(src/intf/world.h:68 addRigidBody, :24-25 gravity/dt, solver iteration
src/rigid/constraint/constraint_solver/constraint_solver.h:72): a list of collision
shapes and a list of rigid bodies referencing them.  Shape type codes follow the
reference's ``ShapeType`` enum order (src/rigid/shape/shape.h:7-9):
0 box (full size), 1 sphere (radius), 2 cylinder (radius, height), 3 convex mesh.

Body fields mirror the reference's RigidBody setters (src/rigid/object/rigidbody.h):
mass, friction, restitution, linear/angular damping, kinematic flag, transform
(origin + row-major 3x3 basis) and linear/angular velocity.

All reals are stored as float64.  A scene meant for the single-precision build is
generated with every real rounded to float32 first, so that loading it into a
``float`` world is exact.

Generators (all seeded, all synthetic; no dataset is involved):
  * ``tower``      - boxes stacked in a grid on a static ground box, hit by a sphere.
  * ``random_cube``- bodies of mixed shapes scattered uniformly in a cube (one-step stress).
  * ``pile``       - a jittered pile of mixed shapes (incl. convex hulls) dropped on a ground box.
  * ``pair_zoo``   - many isolated body pairs of one shape pairing, for narrowphase coverage.
"""
from __future__ import annotations

import dataclasses
import struct
from pathlib import Path

import numpy as np

BOX, SPHERE, CYLINDER, HULL = 0, 1, 2, 3
CONCAVE = 4    # ShapeType::ST_ConcaveMesh: a triangle mesh (static terrain), shares the hull tables
COMPOUND = 5   # ShapeType::ST_Compound
JOINT_BALL, JOINT_HINGE, JOINT_SLIDER = 0, 1, 2   # ConstraintType::CT_{BALL,HINGE,SLIDER}_JOINT
KINEMATIC = 1
IGNORE_COLLISION = 2   # RigidBody::setIgnoreCollision: the body takes part in no pair

MAGIC = b"PESCENE1"
MAGIC_COMPOUND = b"PESCENE2"   # the same layout followed by the compound-children tables


@dataclasses.dataclass
class Scene:
    dt: float = 0.01
    gravity: tuple = (0.0, -9.8, 0.0)
    iterations: int = 10
    real_bits: int = 64
    # shapes
    shape_type: np.ndarray = None      # int32 [S]
    shape_param: np.ndarray = None     # float64 [S,3]
    hull_vbeg: np.ndarray = None       # int32 [S]
    hull_vcnt: np.ndarray = None
    hull_fbeg: np.ndarray = None
    hull_fcnt: np.ndarray = None
    hull_verts: np.ndarray = None      # float64 [HV,3]
    hull_face_off: np.ndarray = None   # int32 [HF+1]
    hull_face_idx: np.ndarray = None   # int32 [HI]
    # bodies
    body_shape: np.ndarray = None      # int32 [N]
    body_flags: np.ndarray = None      # int32 [N]
    mass: np.ndarray = None            # float64 [N]
    friction: np.ndarray = None
    restitution: np.ndarray = None
    lin_damp: np.ndarray = None
    ang_damp: np.ndarray = None
    origin: np.ndarray = None          # float64 [N,3]
    basis: np.ndarray = None           # float64 [N,3,3]
    lin_vel: np.ndarray = None         # float64 [N,3]
    ang_vel: np.ndarray = None         # float64 [N,3]
    # compound shapes (CompoundShape::addShape arguments, before init() relocates them): shape s of
    # type COMPOUND owns children [cmp_beg[s], cmp_beg[s] + cmp_cnt[s]); a child names a
    # non-compound shape of the same table and its local transform and mass ratio
    cmp_beg: np.ndarray = None         # int32 [S]
    cmp_cnt: np.ndarray = None         # int32 [S]
    child_shape: np.ndarray = None     # int32 [C]
    child_origin: np.ndarray = None    # float64 [C,3]
    child_basis: np.ndarray = None     # float64 [C,3,3]
    child_ratio: np.ndarray = None     # float64 [C]

    # joints (World::addConstraint of Ball/Hinge/SliderJointConstraint, in order): type JOINT_*,
    # bodies (a, b), flags (bit 0 use_limits, bit 1 use_motor) and 15 reals: anchor_a, anchor_b,
    # axis_a, axis_b (3 each), min_angle, max_angle, target_speed
    joint_type: np.ndarray = None      # int32 [J]
    joint_body: np.ndarray = None      # int32 [J,2]
    joint_flag: np.ndarray = None      # int32 [J]
    joint_real: np.ndarray = None      # float64 [J,15]
    # RigidBody::addIgnoreCollisionId: body pairs that never collide
    ignore_pairs: np.ndarray = None    # int32 [K,2]

    def __post_init__(self):
        if self.child_shape is None:
            self.child_shape = np.zeros(0, np.int32)
            self.child_origin = np.zeros((0, 3))
            self.child_basis = np.zeros((0, 3, 3))
            self.child_ratio = np.zeros(0)
        if self.joint_type is None:
            self.joint_type = np.zeros(0, np.int32)
            self.joint_body = np.zeros((0, 2), np.int32)
            self.joint_flag = np.zeros(0, np.int32)
            self.joint_real = np.zeros((0, 15))
        if self.ignore_pairs is None:
            self.ignore_pairs = np.zeros((0, 2), np.int32)

    @property
    def n_joints(self) -> int:
        return int(self.joint_type.shape[0])

    @property
    def n_children(self) -> int:
        return int(self.child_shape.shape[0])

    def compound_tables(self):
        """(cmp_beg, cmp_cnt) per shape, zeros where the scene has no compound shapes."""
        S = self.n_shapes
        if self.cmp_beg is None:
            return np.zeros(S, np.int32), np.zeros(S, np.int32)
        return self.cmp_beg, self.cmp_cnt

    @property
    def n_bodies(self) -> int:
        return int(self.body_shape.shape[0])

    @property
    def n_shapes(self) -> int:
        return int(self.shape_type.shape[0])

    def rounded(self, real_bits: int) -> "Scene":
        """Copy with every real rounded to the given precision (exact load into that build)."""
        s = dataclasses.replace(self)
        s.real_bits = real_bits
        if real_bits == 32:
            r = lambda a: np.asarray(a, np.float64).astype(np.float32).astype(np.float64)
            s.dt = float(np.float32(self.dt))
            s.gravity = tuple(float(np.float32(g)) for g in self.gravity)
            for f in ("shape_param", "hull_verts", "mass", "friction", "restitution", "lin_damp",
                      "ang_damp", "origin", "basis", "lin_vel", "ang_vel", "child_origin", "child_basis", "child_ratio",
                      "joint_real"):
                setattr(s, f, r(getattr(self, f)))
        return s

    # ------------------------------------------------------------------ file format
    def write(self, path) -> None:
        """Write the little-endian ``.pescene`` layout read by every consumer of a scene."""
        S, N = self.n_shapes, self.n_bodies
        compound = (self.n_children > 0 or bool((self.shape_type == COMPOUND).any()) or self.n_joints > 0
                    or len(self.ignore_pairs) > 0)
        with open(path, "wb") as f:
            f.write(MAGIC_COMPOUND if compound else MAGIC)
            f.write(struct.pack("<6i", S, N, len(self.hull_verts), len(self.hull_face_off) - 1,
                                len(self.hull_face_idx), int(self.iterations)))
            f.write(struct.pack("<4d", float(self.dt), *map(float, self.gravity)))
            for a, t in ((self.shape_type, "<i4"), (self.shape_param, "<f8"), (self.hull_vbeg, "<i4"),
                         (self.hull_vcnt, "<i4"), (self.hull_fbeg, "<i4"), (self.hull_fcnt, "<i4"),
                         (self.hull_verts, "<f8"), (self.hull_face_off, "<i4"), (self.hull_face_idx, "<i4"),
                         (self.body_shape, "<i4"), (self.body_flags, "<i4"), (self.mass, "<f8"),
                         (self.friction, "<f8"), (self.restitution, "<f8"), (self.lin_damp, "<f8"),
                         (self.ang_damp, "<f8"), (self.origin, "<f8"), (self.basis, "<f8"),
                         (self.lin_vel, "<f8"), (self.ang_vel, "<f8")):
                f.write(np.ascontiguousarray(a, dtype=t).tobytes())
            if compound:
                cb, cc = self.compound_tables()
                f.write(struct.pack("<i", self.n_children))
                for a, t in ((cb, "<i4"), (cc, "<i4"), (self.child_shape, "<i4"), (self.child_origin, "<f8"),
                             (self.child_basis, "<f8"), (self.child_ratio, "<f8")):
                    f.write(np.ascontiguousarray(a, dtype=t).tobytes())
                # tagged sections: 1 joints, 2 ignored body pairs
                if self.n_joints:
                    f.write(struct.pack("<2i", 1, self.n_joints))
                    for a, t in ((self.joint_type, "<i4"), (self.joint_body, "<i4"), (self.joint_flag, "<i4"),
                                 (self.joint_real, "<f8")):
                        f.write(np.ascontiguousarray(a, dtype=t).tobytes())
                if len(self.ignore_pairs):
                    f.write(struct.pack("<2i", 2, len(self.ignore_pairs)))
                    f.write(np.ascontiguousarray(self.ignore_pairs, dtype="<i4").tobytes())

    @staticmethod
    def read(path, real_bits: int = 64) -> "Scene":
        b = Path(path).read_bytes()
        if b[:8] not in (MAGIC, MAGIC_COMPOUND):
            raise ValueError("not a .pescene file")
        S, N, HV, HF, HI, iters = struct.unpack_from("<6i", b, 8)
        dt, gx, gy, gz = struct.unpack_from("<4d", b, 32)
        off = 64
        s = Scene(dt=dt, gravity=(gx, gy, gz), iterations=iters, real_bits=real_bits)

        def take(n, t, shape=None):
            nonlocal off
            a = np.frombuffer(b, dtype=t, count=n, offset=off).copy()
            off += a.nbytes
            return a.reshape(shape) if shape else a

        s.shape_type = take(S, "<i4")
        s.shape_param = take(S * 3, "<f8", (S, 3))
        s.hull_vbeg, s.hull_vcnt, s.hull_fbeg, s.hull_fcnt = (take(S, "<i4") for _ in range(4))
        s.hull_verts = take(HV * 3, "<f8", (HV, 3))
        s.hull_face_off = take(HF + 1, "<i4")
        s.hull_face_idx = take(HI, "<i4")
        s.body_shape = take(N, "<i4")
        s.body_flags = take(N, "<i4")
        s.mass, s.friction, s.restitution, s.lin_damp, s.ang_damp = (take(N, "<f8") for _ in range(5))
        s.origin = take(N * 3, "<f8", (N, 3))
        s.basis = take(N * 9, "<f8", (N, 3, 3))
        s.lin_vel = take(N * 3, "<f8", (N, 3))
        s.ang_vel = take(N * 3, "<f8", (N, 3))
        if b[:8] == MAGIC_COMPOUND:
            C = int(take(1, "<i4")[0])
            s.cmp_beg, s.cmp_cnt = take(S, "<i4"), take(S, "<i4")
            s.child_shape = take(C, "<i4")
            s.child_origin = take(C * 3, "<f8", (C, 3))
            s.child_basis = take(C * 9, "<f8", (C, 3, 3))
            s.child_ratio = take(C, "<f8")
            while off < len(b):
                tag, n = (int(x) for x in take(2, "<i4"))
                if tag == 1:
                    s.joint_type = take(n, "<i4")
                    s.joint_body = take(2 * n, "<i4", (n, 2))
                    s.joint_flag = take(n, "<i4")
                    s.joint_real = take(15 * n, "<f8", (n, 15))
                elif tag == 2:
                    s.ignore_pairs = take(2 * n, "<i4", (n, 2))
                else:
                    raise ValueError(f"unknown .pescene section {tag}")
        return s


# ---------------------------------------------------------------------- builders
class SceneBuilder:
    """Incremental construction of a Scene (shapes are deduplicated by parameters)."""

    def __init__(self, dt=0.01, gravity=(0.0, -9.8, 0.0), iterations=10):
        self.dt, self.gravity, self.iterations = dt, gravity, iterations
        self.shapes = []          # (type, (p0,p1,p2), hull index or -1)
        self.shape_key = {}
        self.hulls = []           # (verts [V,3], faces list[list[int]])
        self.bodies = []
        self.joints = []
        self.ignores = []

    def shape(self, kind, params=(0.0, 0.0, 0.0), hull=None):
        params = tuple(float(p) for p in params) + (0.0,) * (3 - len(params))
        if kind in (HULL, CONCAVE):
            self.hulls.append(hull)
            self.shapes.append((kind, (0.0, 0.0, 0.0), len(self.hulls) - 1))
            return len(self.shapes) - 1
        key = (kind, params)
        if key not in self.shape_key:
            self.shapes.append((kind, params, -1))
            self.shape_key[key] = len(self.shapes) - 1
        return self.shape_key[key]

    def compound(self, children):
        """A compound shape (CompoundShape::addShape for each child): children are
        (shape, origin, basis or None, mass ratio) with shape a non-compound shape of this builder.
        Every consumer runs CompoundShape::init() on it (children relocated to their mass-ratio
        centroid, local inertia from theirs); compound_centroid gives the relocation vector."""
        if not children:
            raise ValueError("a compound shape needs at least one child")
        kids = []
        for sh, o, b, r in children:
            if self.shapes[sh][0] == COMPOUND:
                raise ValueError("CompoundShape cannot contain another CompoundShape")
            if self.shapes[sh][0] == CONCAVE:
                raise ValueError("CompoundShape cannot contain ConcaveMeshShape")
            if not r >= 1e-5:   # compound_shape.cpp:14-16 (PE_EPS)
                raise ValueError("mass ratio must be greater than 0")
            kids.append((int(sh), np.asarray(o, np.float64), np.eye(3) if b is None else np.asarray(b, np.float64),
                         float(r)))
        self.shapes.append((COMPOUND, (0.0, 0.0, 0.0), kids))
        return len(self.shapes) - 1

    def joint(self, kind, a, b, anchor_a=(0, 0, 0), anchor_b=(0, 0, 0), axis_a=(1, 0, 0), axis_b=(1, 0, 0),
              limits=None, motor_speed=None):
        """World::addConstraint of a ball, hinge or slider joint between bodies a and b (anchors and
        axes in the bodies' frames; hinge limits (min_angle, max_angle) and motor target speed)."""
        flag = (1 if limits is not None else 0) | (2 if motor_speed is not None else 0)
        lo, hi = limits if limits is not None else (0.0, 0.0)
        real = [*anchor_a, *anchor_b, *axis_a, *axis_b, lo, hi, motor_speed or 0.0]
        self.joints.append((int(kind), int(a), int(b), flag, [float(x) for x in real]))
        return len(self.joints) - 1

    def ignore_pair(self, a, b):
        """RigidBody::addIgnoreCollisionId: bodies a and b never form a collision pair."""
        self.ignores.append((int(a), int(b)))

    def compound_centroid(self, shape):
        """The vector CompoundShape::init() returns (compound_shape.cpp:27-33): the mass-ratio
        weighted mean of the children's origins, summed in child order."""
        kids = self.shapes[shape][2]
        c, total = np.zeros(3), 0.0
        for _, o, _, r in kids:
            c = c + o * r
            total += r
        return c / total

    def body(self, shape, origin, basis=None, mass=1.0, v=(0, 0, 0), w=(0, 0, 0), friction=0.5,
             restitution=0.5, kinematic=False, lin_damp=0.0, ang_damp=0.0, ignore_collision=False):
        basis = np.eye(3) if basis is None else np.asarray(basis, np.float64)
        flags = (KINEMATIC if kinematic else 0) | (IGNORE_COLLISION if ignore_collision else 0)
        self.bodies.append((shape, flags, float(mass), float(friction),
                            float(restitution), float(lin_damp), float(ang_damp),
                            np.asarray(origin, np.float64), basis, np.asarray(v, np.float64),
                            np.asarray(w, np.float64)))
        return len(self.bodies) - 1

    def build(self, real_bits=64) -> Scene:
        S = len(self.shapes)
        s = Scene(dt=self.dt, gravity=tuple(self.gravity), iterations=self.iterations, real_bits=64)
        s.shape_type = np.array([t for t, _, _ in self.shapes], np.int32)
        s.shape_param = np.array([p for _, p, _ in self.shapes], np.float64).reshape(S, 3)
        vbeg, vcnt, fbeg, fcnt = (np.zeros(S, np.int32) for _ in range(4))
        verts, face_off, face_idx = [], [0], []
        nv = nf = 0
        cmp_beg, cmp_cnt = np.zeros(S, np.int32), np.zeros(S, np.int32)
        kids = []
        for i, (t, _, h) in enumerate(self.shapes):
            if t == COMPOUND:
                cmp_beg[i], cmp_cnt[i] = len(kids), len(h)
                kids.extend(h)
            if t not in (HULL, CONCAVE):
                continue
            hv, hf = self.hulls[h]
            vbeg[i], vcnt[i], fbeg[i], fcnt[i] = nv, len(hv), nf, len(hf)
            verts.append(np.asarray(hv, np.float64))
            for face in hf:
                face_idx.extend(int(k) for k in face)
                face_off.append(len(face_idx))
            nv += len(hv)
            nf += len(hf)
        s.hull_vbeg, s.hull_vcnt, s.hull_fbeg, s.hull_fcnt = vbeg, vcnt, fbeg, fcnt
        s.hull_verts = np.concatenate(verts) if verts else np.zeros((0, 3))
        s.hull_face_off = np.array(face_off, np.int32)
        s.hull_face_idx = np.array(face_idx, np.int32)
        if kids:
            s.cmp_beg, s.cmp_cnt = cmp_beg, cmp_cnt
            s.child_shape = np.array([k[0] for k in kids], np.int32)
            s.child_origin = np.array([k[1] for k in kids], np.float64).reshape(-1, 3)
            s.child_basis = np.array([k[2] for k in kids], np.float64).reshape(-1, 3, 3)
            s.child_ratio = np.array([k[3] for k in kids], np.float64)
        if self.joints:
            s.joint_type = np.array([j[0] for j in self.joints], np.int32)
            s.joint_body = np.array([[j[1], j[2]] for j in self.joints], np.int32)
            s.joint_flag = np.array([j[3] for j in self.joints], np.int32)
            s.joint_real = np.array([j[4] for j in self.joints], np.float64)
        if self.ignores:
            s.ignore_pairs = np.array(self.ignores, np.int32)
        B = self.bodies
        s.body_shape = np.array([b[0] for b in B], np.int32)
        s.body_flags = np.array([b[1] for b in B], np.int32)
        s.mass, s.friction, s.restitution, s.lin_damp, s.ang_damp = (
            np.array([b[k] for b in B], np.float64) for k in range(2, 7))
        s.origin = np.array([b[7] for b in B]).reshape(-1, 3)
        s.basis = np.array([b[8] for b in B]).reshape(-1, 3, 3)
        s.lin_vel = np.array([b[9] for b in B]).reshape(-1, 3)
        s.ang_vel = np.array([b[10] for b in B]).reshape(-1, 3)
        return s.rounded(real_bits) if real_bits == 32 else s


# ---------------------------------------------------------------------- geometry helpers
def quat_to_basis(q):
    """Row-major rotation matrices from unit quaternions (w, x, y, z), shape [...,4] -> [...,3,3]."""
    q = np.asarray(q, np.float64)
    w, x, y, z = q[..., 0], q[..., 1], q[..., 2], q[..., 3]
    m = np.empty(q.shape[:-1] + (3, 3))
    m[..., 0, 0] = 1 - 2 * (y * y + z * z)
    m[..., 0, 1] = 2 * (x * y - z * w)
    m[..., 0, 2] = 2 * (x * z + y * w)
    m[..., 1, 0] = 2 * (x * y + z * w)
    m[..., 1, 1] = 1 - 2 * (x * x + z * z)
    m[..., 1, 2] = 2 * (y * z - x * w)
    m[..., 2, 0] = 2 * (x * z - y * w)
    m[..., 2, 1] = 2 * (y * z + x * w)
    m[..., 2, 2] = 1 - 2 * (x * x + y * y)
    return m


def random_rotations(rng, n):
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    return quat_to_basis(q)


def random_hull(rng, nverts, scale):
    """Convex hull of ``nverts`` points on the unit sphere scaled by ``scale``.

    Faces are triangles wound counter-clockwise seen from outside, which is the
    winding the reference's per-face normal ((p2-p1)x(p3-p1), common/mesh.cpp:1-10)
    expects for outward normals.
    """
    from scipy.spatial import ConvexHull

    while True:
        p = rng.normal(size=(nverts, 3))
        p /= np.linalg.norm(p, axis=1, keepdims=True)
        p *= scale
        h = ConvexHull(p)
        if len(h.vertices) == nverts:
            break
    remap = {int(v): i for i, v in enumerate(sorted(h.vertices))}
    verts = p[sorted(h.vertices)]
    faces = []
    centre = verts.mean(axis=0)
    for simplex in h.simplices:
        a, b, c = (remap[int(k)] for k in simplex)
        n = np.cross(verts[b] - verts[a], verts[c] - verts[a])
        if np.dot(n, verts[a] - centre) < 0:
            b, c = c, b
        faces.append([a, b, c])
    return verts, faces


def hull_volume(verts, faces):
    v = 0.0
    for f in faces:
        a, b, c = verts[f[0]], verts[f[1]], verts[f[2]]
        v += np.dot(a, np.cross(b, c)) / 6.0
    return v


# ---------------------------------------------------------------------- generators
def tower(nx=10, ny=10, nz=10, half=0.5, gap=0.001, density=1000.0, sphere_r=1.0, sphere_mass=50.0,
          sphere_speed=30.0, dt=1.0 / 60.0, iterations=20, friction=0.5, restitution=0.0,
          real_bits=64, ground=(100.0, 1.0, 100.0)) -> Scene:
    """Boxes stacked as an nx x ny x nz tower with ``gap`` spacing on a static ground box,
    and a sphere fired horizontally (+x) into the tower at mid-height."""
    sb = SceneBuilder(dt=dt, gravity=(0.0, -9.8, 0.0), iterations=iterations)
    g = sb.shape(BOX, ground)
    sb.body(g, (0.0, -ground[1] / 2, 0.0), mass=0.0, friction=friction, restitution=restitution,
            kinematic=True)
    size = 2 * half
    bshape = sb.shape(BOX, (size, size, size))
    m = density * size ** 3
    pitch = size + gap
    x0 = -(nx - 1) * pitch / 2
    z0 = -(nz - 1) * pitch / 2
    for j in range(ny):
        for i in range(nx):
            for k in range(nz):
                sb.body(bshape, (x0 + i * pitch, half + gap + j * pitch, z0 + k * pitch), mass=m,
                        friction=friction, restitution=restitution)
    s = sb.shape(SPHERE, (sphere_r,))
    sb.body(s, (x0 - 10.0, ny * pitch / 2, 0.0), mass=sphere_mass, v=(sphere_speed, 0.0, 0.0),
            friction=friction, restitution=restitution)
    return sb.build(real_bits)


def _random_body(sb, rng, kind, origin, density, basis, v, w, friction=0.5, restitution=0.0, hull_range=(8, 64)):
    if kind == BOX:
        he = rng.uniform(0.2, 1.0, size=3)
        sh = sb.shape(BOX, 2 * he)
        vol = np.prod(2 * he)
    elif kind == SPHERE:
        r = rng.uniform(0.2, 1.0)
        sh = sb.shape(SPHERE, (r,))
        vol = 4.0 / 3.0 * np.pi * r ** 3
    elif kind == CYLINDER:
        r = rng.uniform(0.2, 0.8)
        h = rng.uniform(0.4, 2.0)
        sh = sb.shape(CYLINDER, (r, h))
        vol = np.pi * r * r * h
    else:
        nv = int(rng.integers(hull_range[0], hull_range[1] + 1))
        verts, faces = random_hull(rng, nv, rng.uniform(0.3, 1.0))
        sh = sb.shape(HULL, hull=(verts, faces))
        vol = hull_volume(verts, faces)
    return sb.body(sh, origin, basis, mass=density * vol, v=v, w=w, friction=friction, restitution=restitution)


def random_cube(n=65536, seed=0, extent=100.0, mix=(0.60, 0.25, 0.15, 0.0), density=1000.0,
                vel_sigma=2.0, dt=1.0 / 60.0, iterations=10, real_bits=32) -> Scene:
    """Bodies with mixed shapes, uniform positions in a cube, uniform random rotations and
    N(0, vel_sigma) linear velocities (broad/narrowphase stress)."""
    rng = np.random.default_rng(seed)
    sb = SceneBuilder(dt=dt, iterations=iterations)
    kinds = rng.choice(4, size=n, p=np.asarray(mix) / np.sum(mix))
    pos = rng.uniform(0.0, extent, size=(n, 3))
    rot = random_rotations(rng, n)
    vel = rng.normal(0.0, vel_sigma, size=(n, 3))
    for i in range(n):
        _random_body(sb, rng, int(kinds[i]), pos[i], density, rot[i], vel[i], (0.0, 0.0, 0.0))
    return sb.build(real_bits)


def pile(n, seed=0, mix=(0.5, 0.2, 0.1, 0.2), density=1000.0, drop=(0.0, 5.0), dt=1.0 / 60.0,
         iterations=10, real_bits=32, hull_range=(8, 64)) -> Scene:
    """A jittered pile of mixed shapes (box/sphere/cylinder/convex hull) above a static ground
    box, lowest layer between drop[0] and drop[1] metres above the ground."""
    rng = np.random.default_rng(seed)
    sb = SceneBuilder(dt=dt, iterations=iterations)
    side = max(2, int(np.ceil(np.sqrt(n / 2.0))))
    pitch = 2.2
    ground = (side * pitch + 10.0, 1.0, side * pitch + 10.0)
    g = sb.shape(BOX, ground)
    sb.body(g, (0.0, -0.5, 0.0), mass=0.0, kinematic=True)
    kinds = rng.choice(4, size=n, p=np.asarray(mix) / np.sum(mix))
    rot = random_rotations(rng, n)
    base = rng.uniform(*drop)
    for i in range(n):
        layer, cell = divmod(i, side * side)
        gx, gz = divmod(cell, side)
        org = ((gx - side / 2) * pitch + rng.uniform(-0.1, 0.1), 1.2 + base + layer * pitch,
               (gz - side / 2) * pitch + rng.uniform(-0.1, 0.1))
        _random_body(sb, rng, int(kinds[i]), org, density, rot[i], (0.0, 0.0, 0.0), (0.0, 0.0, 0.0),
                     hull_range=hull_range)
    return sb.build(real_bits)


def pair_zoo(kind_a, kind_b, m=64, seed=0, spacing=20.0, real_bits=64, hull_range=(8, 32)) -> Scene:
    """``m`` isolated body pairs of one shape pairing, each placed in its own cell with random
    rotations and a random offset that mostly overlaps (narrowphase coverage, zero gravity)."""
    rng = np.random.default_rng(seed)
    sb = SceneBuilder(dt=1.0 / 60.0, gravity=(0.0, 0.0, 0.0), iterations=10)
    side = int(np.ceil(m ** (1 / 3)))
    for i in range(m):
        cx, rem = divmod(i, side * side)
        cy, cz = divmod(rem, side)
        c = np.array([cx, cy, cz], np.float64) * spacing
        rot = random_rotations(rng, 2)
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        off = d * rng.uniform(0.3, 1.6)
        for k, (kind, o) in enumerate(((kind_a, c), (kind_b, c + off))):
            _random_body(sb, rng, kind, o, 1000.0, rot[k], (0.0, 0.0, 0.0), (0.0, 0.0, 0.0),
                         friction=0.5, restitution=0.2, hull_range=hull_range)
    return sb.build(real_bits)


def _rot(axis, angle):
    c, s_ = np.cos(angle), np.sin(angle)
    x, y, z = axis
    return np.array([[c + x * x * (1 - c), x * y * (1 - c) - z * s_, x * z * (1 - c) + y * s_],
                     [y * x * (1 - c) + z * s_, c + y * y * (1 - c), y * z * (1 - c) - x * s_],
                     [z * x * (1 - c) - y * s_, z * y * (1 - c) + x * s_, c + z * z * (1 - c)]])


def compound_pile(n=24, seed=0, real_bits=64, dt=1.0 / 60.0, iterations=10, spacing=2.6, drop=(0.5, 3.0),
                  n_primitives=12, friction=0.5, restitution=0.3, hull_children=True) -> Scene:
    """Compound bodies dropped on a static ground box among primitive bodies.  Three compound
    kinds rotate through the ``n`` compounds: the reference's compound demo "jack" (a unit box
    hub, a long cylinder up, short cylinders down and along +-x, +-z, mass ratios 0.3 / 0.2 /
    0.1, examples/compound_demo/main.cpp:48-80), a dumbbell (two spheres on a cylinder bar), and
    a box with a convex-hull cap.  Bodies are placed like the demo: the body origin minus the
    centroid init() returns.  The primitives (box, sphere, cylinder, hull) fall among them so
    that pairs meet compounds on both sides of the pair order."""
    rng = np.random.default_rng(seed)
    sb = SceneBuilder(dt=dt, iterations=iterations)
    g = sb.shape(BOX, (60.0, 1.0, 60.0))
    sb.body(g, (0.0, -0.5, 0.0), mass=0.0, friction=friction, restitution=restitution, kinematic=True)
    hub = sb.shape(BOX, (1.0, 1.0, 1.0))
    long_arm = sb.shape(CYLINDER, (0.2, 2.0))
    arm = sb.shape(CYLINDER, (0.2, 1.0))
    rz, rx = _rot((0, 0, 1), np.pi / 2), _rot((1, 0, 0), np.pi / 2)
    jack = sb.compound([(hub, (0, 0, 0), None, 0.3), (long_arm, (0, 1.5, 0), None, 0.2), (arm, (0, -1, 0), None, 0.1),
                        (arm, (1, 0, 0), rz, 0.1), (arm, (-1, 0, 0), rz, 0.1), (arm, (0, 0, 1), rx, 0.1),
                        (arm, (0, 0, -1), rx, 0.1)])
    ball = sb.shape(SPHERE, (0.45,))
    bar = sb.shape(CYLINDER, (0.12, 1.6))
    dumbbell = sb.compound([(ball, (-0.9, 0, 0), None, 0.4), (ball, (0.9, 0, 0), None, 0.4), (bar, (0, 0, 0), rz, 0.2)])
    kinds = [jack, dumbbell]
    if hull_children:
        hv, hf = random_hull(rng, 12, 0.6)
        cap = sb.shape(HULL, hull=(hv, hf))
        base = sb.shape(BOX, (1.2, 0.6, 1.2))
        kinds.append(sb.compound([(base, (0, 0, 0), None, 0.6), (cap, (0.1, 0.55, -0.05), _rot((0, 1, 0), 0.3), 0.4)]))
    side = int(np.ceil(np.sqrt(n + n_primitives)))
    slots = rng.permutation(side * side)[:n + n_primitives]
    rots = random_rotations(rng, n + n_primitives)
    for i, slot in enumerate(slots):
        cx, cz = divmod(int(slot), side)
        o = np.array([(cx - (side - 1) / 2) * spacing, 2.5 + rng.uniform(*drop) + 1.5 * (i % 3),
                      (cz - (side - 1) / 2) * spacing])
        v = (0.0, rng.uniform(-1.0, 0.0), 0.0)
        w = rng.normal(size=3) * 0.5
        if i < n:
            c = kinds[i % len(kinds)]
            sb.body(c, o - sb.compound_centroid(c), rots[i], mass=float(rng.uniform(1.0, 4.0)), v=v, w=w,
                    friction=friction, restitution=restitution)
        else:
            _random_body(sb, rng, (BOX, SPHERE, CYLINDER, HULL)[i % 4], o, 300.0, rots[i], v, w, friction=friction,
                         restitution=restitution, hull_range=(8, 16))
    return sb.build(real_bits)


def joint_demo(real_bits=64, chain=6, motor_speed=2.0, hinge_limits=True, dt=1.0 / 60.0, iterations=10) -> Scene:
    """The reference's constraints demo (examples/constraints_demo/main.cpp:23-164): a ball-joint
    double pendulum on a kinematic sphere, a hinge with angle limits carrying a second hinged
    stick, and a box slider on a kinematic rail between two kinematic stops, with the demo's
    ignored collision pairs between jointed bodies; plus a motor-driven hinge paddle and a chain
    of ``chain`` boxes hanging by ball joints from a kinematic anchor, released horizontally."""
    sb = SceneBuilder(dt=dt, iterations=iterations)
    pi = np.pi
    I3 = np.eye(3)

    def xf(b, o):
        return (np.asarray(b, np.float64), np.asarray(o, np.float64))

    def mul(t1, t2):
        return (t1[0] @ t2[0], t1[0] @ t2[1] + t1[1])

    def add(kind, params, t, mass=1.0, kinematic=False, restitution=0.5):
        sh = sb.shape(kind, params)
        return sb.body(sh, t[1], t[0], mass=mass, friction=0.5, restitution=restitution, kinematic=kinematic,
                       ang_damp=0.0 if kinematic else 0.8)

    add(BOX, (30, 10, 30), xf(I3, (0, -5, 0)), mass=10000.0, kinematic=True)
    # ball joints
    rb2 = add(SPHERE, (0.5,), xf(I3, (0, 0.5, 0)), kinematic=True)
    rb3 = add(CYLINDER, (0.2, 6), xf(_rot((0, 0, 1), pi / 6), (-3.3 * np.sin(pi / 6), 3.3 * np.cos(pi / 6) + 0.5, 0)))
    sb.ignore_pair(rb2, rb3)
    sb.joint(JOINT_BALL, rb2, rb3, (0, 0, 0), (0, -3.3, 0))
    rb4 = add(SPHERE, (0.4,), xf(I3, (-6.6 * np.sin(pi / 6), 6.6 * np.cos(pi / 6) + 0.5, 0)))
    sb.ignore_pair(rb4, rb3)
    rb5 = add(CYLINDER, (0.2, 6), xf(_rot((0, 0, 1), pi / 2), (-3.3 - 6.6 * np.sin(pi / 6), 6.6 * np.cos(pi / 6) + 0.5, 0)))
    sb.ignore_pair(rb4, rb5)
    sb.joint(JOINT_BALL, rb4, rb5, (0, 0, 0), (0, -3.3, 0))
    sb.joint(JOINT_BALL, rb3, rb4, (0, 3.3, 0), (0, 0, 0))
    # hinge joints
    t = xf(_rot((1, 0, 0), pi / 6), (4, 8, 0))
    rb6 = add(CYLINDER, (0.2, 1), t, kinematic=True)
    rb7 = add(CYLINDER, (0.2, 4), mul(t, xf(_rot((0, 0, -1), pi / 2), (2, 0, 0))))
    sb.ignore_pair(rb6, rb7)
    sb.joint(JOINT_HINGE, rb6, rb7, (0, 0, 0), (0, -2, 0), (0, 1, 0), (-1, 0, 0),
             limits=(-pi / 3, pi / 3) if hinge_limits else None)
    rb8 = add(CYLINDER, (0.2, 2), mul(t, xf(_rot((1, 0, 0), pi / 2), (4, 0, 0.75))))
    sb.ignore_pair(rb7, rb8)
    sb.joint(JOINT_HINGE, rb7, rb8, (0, 2, 0), (0, -0.75, 0), (0, 1, 0), (0, 0, -1))
    # slider
    t0 = xf(_rot((0, 1, 0), -pi / 4), (-1, 6, 0))
    tt = mul(t0, xf(_rot((0, 0, 1), pi / 3), (0, 0, 0)))
    rail = add(BOX, (0.3, 10, 0.3), tt, kinematic=True)
    add(BOX, (1, 0.4, 1), mul(tt, xf(I3, (0, 5.2, 0))), kinematic=True)
    add(BOX, (1, 0.4, 1), mul(tt, xf(I3, (0, -5.2, 0))), kinematic=True)
    slider = add(BOX, (1, 1.2, 1), mul(tt, xf(I3, (0, 4.4, 0))))
    sb.ignore_pair(rail, slider)
    sb.joint(JOINT_SLIDER, rail, slider, (0, 0, 0), (0, 0, 0), (0, 1, 0), (0, 1, 0))
    # motor hinge: a paddle spun about a kinematic post
    post = add(BOX, (0.2, 2, 0.2), xf(I3, (8, 1, -4)), kinematic=True)
    paddle = add(BOX, (2, 0.2, 0.5), xf(I3, (8, 2.3, -4)))
    sb.ignore_pair(post, paddle)
    sb.joint(JOINT_HINGE, post, paddle, (0, 1.3, 0), (0, 0, 0), (0, 1, 0), (0, 1, 0), motor_speed=motor_speed)
    # a chain of boxes hanging from a kinematic anchor by ball joints, released horizontally
    prev = add(SPHERE, (0.2,), xf(I3, (-8, 10, 5)), kinematic=True)
    link = _rot((0, 0, 1), pi / 2)
    for k in range(chain):
        cur = add(BOX, (0.3, 1.0, 0.3), xf(link, (-8 + 0.5 + k * 1.0, 10, 5)))
        sb.ignore_pair(prev, cur)
        sb.joint(JOINT_BALL, prev, cur, (0, 0, 0) if k == 0 else (0, -0.5, 0), (0, 0.5, 0))
        prev = cur
    return sb.build(real_bits)


def chain_field(n_chains=64, links=8, seed=0, spacing=3.0, height=6.0, hinge_limits=True, real_bits=64, dt=1.0 / 60.0,
                iterations=10) -> Scene:
    """``n_chains`` chains of ``links`` boxes, each hanging from a kinematic anchor sphere and
    released horizontally above a static ground box.  Consecutive links are joined by a ball joint,
    a hinge (every third joint, limited to +-60 degrees on odd chains, motor-driven on chains
    divisible by 4) or a slider (every fifth joint); jointed neighbours ignore each other's
    collisions, so the links meet the ground and the other chains only."""
    rng = np.random.default_rng(seed)
    sb = SceneBuilder(dt=dt, iterations=iterations)
    g = sb.shape(BOX, (n_chains ** 0.5 * spacing * 2 + 20, 1.0, n_chains ** 0.5 * spacing * 2 + 20))
    sb.body(g, (0, -0.5, 0), mass=0.0, kinematic=True)
    ball = sb.shape(SPHERE, (0.15,))
    link = sb.shape(BOX, (0.8, 0.25, 0.25))
    side = int(np.ceil(np.sqrt(n_chains)))
    for c in range(n_chains):
        cx, cz = divmod(c, side)
        x0 = (cx - (side - 1) / 2) * spacing + rng.uniform(-0.2, 0.2)
        z0 = (cz - (side - 1) / 2) * spacing + rng.uniform(-0.2, 0.2)
        yaw = _rot((0, 1, 0), rng.uniform(0, 2 * np.pi))
        d = yaw @ np.array([1.0, 0, 0])
        a0 = np.array([x0, height + rng.uniform(0, 1), z0])
        prev = sb.body(ball, a0, kinematic=True, mass=0.0)
        for k in range(links):
            cur = sb.body(link, a0 + d * (0.4 + 0.8 * k), yaw, mass=float(rng.uniform(0.5, 2.0)), ang_damp=0.1,
                          friction=0.5, restitution=0.2)
            sb.ignore_pair(prev, cur)
            anc_a = (0, 0, 0) if k == 0 else (0.4, 0, 0)
            if k > 0 and k % 5 == 0:
                sb.joint(JOINT_SLIDER, prev, cur, anc_a, (-0.4, 0, 0), (1, 0, 0), (1, 0, 0))
            elif k > 0 and k % 3 == 0:
                sb.joint(JOINT_HINGE, prev, cur, anc_a, (-0.4, 0, 0), (0, 0, 1), (0, 0, 1),
                         limits=(-np.pi / 3, np.pi / 3) if c % 2 and hinge_limits else None,
                         motor_speed=1.5 if c % 4 == 0 else None)
            else:
                sb.joint(JOINT_BALL, prev, cur, anc_a, (-0.4, 0, 0))
            prev = cur
    return sb.build(real_bits)


def heightfield(nx, nz, cell=1.0, amp=0.6, seed=0):
    """A terrain triangle mesh over [0, nx*cell] x [0, nz*cell] centred on the origin: heights from
    a few seeded sines, two triangles per cell wound counter-clockwise seen from above (normals up)."""
    rng = np.random.default_rng(seed)
    xs = (np.arange(nx + 1) - nx / 2) * cell
    zs = (np.arange(nz + 1) - nz / 2) * cell
    X, Z = np.meshgrid(xs, zs, indexing="ij")
    H = np.zeros_like(X)
    for _ in range(4):
        kx, kz, ph = rng.uniform(0.1, 0.5), rng.uniform(0.1, 0.5), rng.uniform(0, 2 * np.pi)
        H += amp / 4 * np.sin(kx * X + ph) * np.cos(kz * Z - ph)
    verts = np.stack([X.ravel(), H.ravel(), Z.ravel()], axis=1)
    idx = lambda i, j: i * (nz + 1) + j
    faces = []
    for i in range(nx):
        for j in range(nz):
            faces.append([idx(i, j), idx(i, j + 1), idx(i + 1, j + 1)])
            faces.append([idx(i, j), idx(i + 1, j + 1), idx(i + 1, j)])
    return verts, faces


def terrain_drop(n=40, nx=16, nz=16, seed=0, real_bits=64, dt=1.0 / 60.0, iterations=10, drop=(0.8, 2.5),
                 compounds=True) -> Scene:
    """Bodies of every kind (box, sphere, cylinder, convex hull and, optionally, compound) dropped
    onto a static concave heightfield of nx x nz cells (2 triangles each; 16 x 16 gives 512
    faces, above 4,094 faces the face tree gets leaves of several faces)."""
    rng = np.random.default_rng(seed)
    sb = SceneBuilder(dt=dt, iterations=iterations)
    hv, hf = heightfield(nx, nz, seed=seed)
    t = sb.shape(CONCAVE, hull=(hv, hf))
    sb.body(t, (0.0, 0.0, 0.0), mass=0.0, friction=0.6, restitution=0.2, kinematic=True)
    kinds = [BOX, SPHERE, CYLINDER, HULL]
    if compounds:
        hub = sb.shape(BOX, (0.5, 0.5, 0.5))
        arm = sb.shape(CYLINDER, (0.1, 0.8))
        jack = sb.compound([(hub, (0, 0, 0), None, 0.5), (arm, (0.55, 0, 0), _rot((0, 0, 1), np.pi / 2), 0.25),
                            (arm, (-0.55, 0, 0), _rot((0, 0, 1), np.pi / 2), 0.25)])
    span = min(nx, nz) * 0.8 / 2
    rots = random_rotations(rng, n)
    for i in range(n):
        o = np.array([rng.uniform(-span, span), rng.uniform(*drop) + 0.6, rng.uniform(-span, span)])
        if compounds and i % 5 == 4:
            sb.body(jack, o - sb.compound_centroid(jack), rots[i], mass=float(rng.uniform(0.5, 2.0)), friction=0.6,
                    restitution=0.2)
        else:
            _random_body(sb, rng, kinds[i % 4], o, 300.0, rots[i], (0.0, 0.0, 0.0), (0.0, 0.0, 0.0), friction=0.6,
                         restitution=0.2, hull_range=(8, 16))
    return sb.build(real_bits)


def concat(scenes):
    """Scenes side by side in one Scene (bodies of scene i at [off[i], off[i+1])); shapes are
    concatenated and re-indexed.  Used for batched stepping of independent scenes."""
    first = scenes[0]
    out = Scene(dt=first.dt, gravity=first.gravity, iterations=first.iterations, real_bits=first.real_bits)
    sh_base = vb = fb = ib = 0
    cols = {k: [] for k in ("shape_type", "shape_param", "hull_vbeg", "hull_vcnt", "hull_fbeg", "hull_fcnt", "hull_verts",
                            "hull_face_idx", "body_shape", "body_flags", "mass", "friction", "restitution", "lin_damp",
                            "ang_damp", "origin", "basis", "lin_vel", "ang_vel")}
    face_off = [0]
    offs = [0]
    kid_cols = {k: [] for k in ("cmp_beg", "cmp_cnt", "child_shape", "child_origin", "child_basis", "child_ratio")}
    kb = 0
    extra = {k: [] for k in ("joint_type", "joint_body", "joint_flag", "joint_real", "ignore_pairs")}
    for s in scenes:
        extra["joint_type"].append(s.joint_type)
        extra["joint_body"].append(s.joint_body + offs[-1])
        extra["joint_flag"].append(s.joint_flag)
        extra["joint_real"].append(s.joint_real)
        extra["ignore_pairs"].append(s.ignore_pairs + offs[-1])
        cb, cc = s.compound_tables()
        kid_cols["cmp_beg"].append(cb + kb)
        kid_cols["cmp_cnt"].append(cc)
        kid_cols["child_shape"].append(s.child_shape + sh_base)
        for k in ("child_origin", "child_basis", "child_ratio"):
            kid_cols[k].append(getattr(s, k))
        kb += s.n_children
        if (s.dt, tuple(s.gravity), s.iterations) != (first.dt, tuple(first.gravity), first.iterations):
            raise ValueError("batched scenes must share dt, gravity and iterations")
        cols["shape_type"].append(s.shape_type)
        cols["shape_param"].append(s.shape_param)
        cols["hull_vbeg"].append(s.hull_vbeg + vb)
        cols["hull_vcnt"].append(s.hull_vcnt)
        cols["hull_fbeg"].append(s.hull_fbeg + fb)
        cols["hull_fcnt"].append(s.hull_fcnt)
        cols["hull_verts"].append(s.hull_verts)
        cols["hull_face_idx"].append(s.hull_face_idx)
        face_off.extend((s.hull_face_off[1:] + ib).tolist())
        cols["body_shape"].append(s.body_shape + sh_base)
        for k in ("body_flags", "mass", "friction", "restitution", "lin_damp", "ang_damp", "origin", "basis", "lin_vel",
                  "ang_vel"):
            cols[k].append(getattr(s, k))
        sh_base += s.n_shapes
        vb += len(s.hull_verts)
        fb += len(s.hull_face_off) - 1
        ib += len(s.hull_face_idx)
        offs.append(offs[-1] + s.n_bodies)
    for k, v in cols.items():
        setattr(out, k, np.concatenate(v))
    out.hull_verts = out.hull_verts.reshape(-1, 3)
    out.hull_face_off = np.array(face_off, np.int32)
    out.joint_type = np.concatenate(extra["joint_type"]).astype(np.int32)
    out.joint_body = np.concatenate(extra["joint_body"]).astype(np.int32).reshape(-1, 2)
    out.joint_flag = np.concatenate(extra["joint_flag"]).astype(np.int32)
    out.joint_real = np.concatenate(extra["joint_real"]).reshape(-1, 15)
    out.ignore_pairs = np.concatenate(extra["ignore_pairs"]).astype(np.int32).reshape(-1, 2)
    if kb:
        for k, v in kid_cols.items():
            setattr(out, k, np.concatenate(v))
        out.child_shape = out.child_shape.astype(np.int32)
        out.child_origin = out.child_origin.reshape(-1, 3)
        out.child_basis = out.child_basis.reshape(-1, 3, 3)
    return out, np.array(offs, np.int32)


def _hull_volumes(verts, faces):
    f = np.asarray(faces, np.int64)
    a, b, c = verts[f[:, 0]], verts[f[:, 1]], verts[f[:, 2]]
    return float(np.einsum("ij,ij->i", a, np.cross(b, c)).sum() / 6.0)


def batched_piles(n_scenes=4096, seed=0, size_range=(8, 512), mix=(0.5, 0.2, 0.1, 0.2), hull_pool=512,
                  hull_range=(8, 64), drop=(0.0, 5.0), density=1000.0, dt=1.0 / 60.0, iterations=10,
                  real_bits=32):
    """``n_scenes`` independent piles, each laid out like ``pile`` (a jittered grid of mixed shapes
    above its own static ground box, lowest layer drop[0]..drop[1] m up), with body counts
    log-uniform in ``size_range``.  Box/sphere/cylinder sizes follow ``random_cube``; convex hulls
    have 8..64 vertices on a sphere scaled U[0.3, 1.0] and are drawn from a seeded pool of
    ``hull_pool`` shapes shared by all scenes (bodies may share a shape, as RigidBody shape
    pointers may in the reference).  Returns (Scene, body offsets [n_scenes + 1]); the bodies of
    scene k are [off[k], off[k+1]), its ground box first.  Vectorised: ~500k bodies in seconds."""
    rng = np.random.default_rng(seed)
    lo, hi = size_range
    sizes = np.floor(np.exp(rng.uniform(np.log(lo), np.log(hi + 1), n_scenes))).astype(np.int64).clip(lo, hi)
    # hull pool
    pool_v, pool_f, pool_vol = [], [], []
    for _ in range(hull_pool):
        nv = int(rng.integers(hull_range[0], hull_range[1] + 1))
        v, f = random_hull(rng, nv, rng.uniform(0.3, 1.0))
        pool_v.append(v)
        pool_f.append(f)
        pool_vol.append(_hull_volumes(v, f))
    pool_vol = np.array(pool_vol)
    sides = np.maximum(2, np.ceil(np.sqrt(sizes / 2.0))).astype(np.int64)
    pitch = 2.2
    n_dyn = int(sizes.sum())
    N = n_dyn + n_scenes
    # body -> scene, index inside the scene's pile
    scene_of = np.repeat(np.arange(n_scenes), sizes)
    start = np.concatenate([[0], np.cumsum(sizes)[:-1]])
    idx = np.arange(n_dyn) - start[scene_of]
    kinds = rng.choice(4, size=n_dyn, p=np.asarray(mix) / np.sum(mix))
    side = sides[scene_of]
    layer, cell = np.divmod(idx, side * side)
    gx, gz = np.divmod(cell, side)
    base = rng.uniform(drop[0], drop[1], n_scenes)[scene_of]
    org = np.stack([(gx - side / 2) * pitch + rng.uniform(-0.1, 0.1, n_dyn), 1.2 + base + layer * pitch,
                    (gz - side / 2) * pitch + rng.uniform(-0.1, 0.1, n_dyn)], axis=1)
    rot = random_rotations(rng, n_dyn)
    # shapes: hull pool first, then one ground box per distinct side, then one shape per primitive body
    he = rng.uniform(0.2, 1.0, size=(n_dyn, 3))
    rs = rng.uniform(0.2, 1.0, n_dyn)
    rc = rng.uniform(0.2, 0.8, n_dyn)
    hc = rng.uniform(0.4, 2.0, n_dyn)
    pick = rng.integers(0, hull_pool, n_dyn)
    uniq_sides, side_idx = np.unique(sides, return_inverse=True)
    prim = kinds != HULL
    n_prim = int(prim.sum())
    S = hull_pool + len(uniq_sides) + n_prim
    shape_type = np.zeros(S, np.int32)
    shape_param = np.zeros((S, 3))
    shape_type[:hull_pool] = HULL
    g0 = hull_pool
    shape_type[g0:g0 + len(uniq_sides)] = BOX
    gs = uniq_sides * pitch + 10.0
    shape_param[g0:g0 + len(uniq_sides)] = np.stack([gs, np.ones_like(gs, dtype=np.float64), gs], axis=1)
    p0 = g0 + len(uniq_sides)
    pk = kinds[prim]
    shape_type[p0:] = pk
    par = np.zeros((n_prim, 3))
    par[pk == BOX] = 2 * he[prim][pk == BOX]
    par[pk == SPHERE, 0] = rs[prim][pk == SPHERE]
    par[pk == CYLINDER, 0] = rc[prim][pk == CYLINDER]
    par[pk == CYLINDER, 1] = hc[prim][pk == CYLINDER]
    shape_param[p0:] = par
    body_shape_dyn = np.where(prim, 0, pick)
    body_shape_dyn[prim] = p0 + np.arange(n_prim)
    vol = np.where(kinds == BOX, np.prod(2 * he, axis=1),
                   np.where(kinds == SPHERE, 4.0 / 3.0 * np.pi * rs ** 3,
                            np.where(kinds == CYLINDER, np.pi * rc * rc * hc, pool_vol[pick])))
    # hull tables
    vbeg, vcnt, fbeg, fcnt = (np.zeros(S, np.int32) for _ in range(4))
    vcnt[:hull_pool] = [len(v) for v in pool_v]
    fcnt[:hull_pool] = [len(f) for f in pool_f]
    vbeg[:hull_pool] = np.concatenate([[0], np.cumsum(vcnt[:hull_pool])[:-1]])
    fbeg[:hull_pool] = np.concatenate([[0], np.cumsum(fcnt[:hull_pool])[:-1]])
    face_idx = np.concatenate([np.asarray(f, np.int32).ravel() for f in pool_f])
    face_off = np.arange(0, 3 * int(fcnt.sum()) + 1, 3, dtype=np.int32)
    # interleave: scene k = [ground_k, its bodies]
    pos = np.arange(n_dyn) + scene_of + 1            # body slot in the merged order
    gpos = start + np.arange(n_scenes)               # ground slot of each scene
    s = Scene(dt=dt, gravity=(0.0, -9.8, 0.0), iterations=iterations, real_bits=64)
    s.shape_type, s.shape_param = shape_type, shape_param
    s.hull_vbeg, s.hull_vcnt, s.hull_fbeg, s.hull_fcnt = vbeg, vcnt, fbeg, fcnt
    s.hull_verts = np.concatenate(pool_v).reshape(-1, 3)
    s.hull_face_off, s.hull_face_idx = face_off, face_idx
    s.body_shape = np.zeros(N, np.int32)
    s.body_shape[pos] = body_shape_dyn
    s.body_shape[gpos] = g0 + side_idx
    s.body_flags = np.zeros(N, np.int32)
    s.body_flags[gpos] = KINEMATIC
    s.mass = np.zeros(N)
    s.mass[pos] = density * vol
    s.friction = np.full(N, 0.5)
    s.restitution = np.zeros(N)
    s.lin_damp = np.zeros(N)
    s.ang_damp = np.zeros(N)
    s.origin = np.zeros((N, 3))
    s.origin[pos] = org
    s.origin[gpos] = (0.0, -0.5, 0.0)
    s.basis = np.tile(np.eye(3), (N, 1, 1))
    s.basis[pos] = rot
    s.lin_vel = np.zeros((N, 3))
    s.ang_vel = np.zeros((N, 3))
    offs = np.concatenate([[0], np.cumsum(sizes + 1)]).astype(np.int32)
    return (s.rounded(real_bits) if real_bits == 32 else s), offs


def extract(scene, offs, k):
    """Scene k of a batch as a standalone Scene (its bodies and the shapes they use)."""
    b0, b1 = int(offs[k]), int(offs[k + 1])
    used = np.unique(scene.body_shape[b0:b1])
    remap = np.full(scene.n_shapes, -1, np.int64)
    remap[used] = np.arange(len(used))
    s = Scene(dt=scene.dt, gravity=scene.gravity, iterations=scene.iterations, real_bits=scene.real_bits)
    s.shape_type = scene.shape_type[used].copy()
    s.shape_param = scene.shape_param[used].copy()
    vbeg, vcnt, fbeg, fcnt = (np.zeros(len(used), np.int32) for _ in range(4))
    verts, face_off, face_idx = [], [0], []
    nv = nf = 0
    for t, sh in enumerate(used):
        if scene.shape_type[sh] != HULL:
            continue
        v0, vc = scene.hull_vbeg[sh], scene.hull_vcnt[sh]
        f0, fc = scene.hull_fbeg[sh], scene.hull_fcnt[sh]
        vbeg[t], vcnt[t], fbeg[t], fcnt[t] = nv, vc, nf, fc
        verts.append(scene.hull_verts[v0:v0 + vc])
        for f in range(f0, f0 + fc):
            face_idx.extend(scene.hull_face_idx[scene.hull_face_off[f]:scene.hull_face_off[f + 1]].tolist())
            face_off.append(len(face_idx))
        nv += vc
        nf += fc
    s.hull_vbeg, s.hull_vcnt, s.hull_fbeg, s.hull_fcnt = vbeg, vcnt, fbeg, fcnt
    s.hull_verts = np.concatenate(verts).reshape(-1, 3) if verts else np.zeros((0, 3))
    s.hull_face_off = np.array(face_off, np.int32)
    s.hull_face_idx = np.array(face_idx, np.int32)
    s.body_shape = remap[scene.body_shape[b0:b1]].astype(np.int32)
    for f in ("body_flags", "mass", "friction", "restitution", "lin_damp", "ang_damp", "origin", "basis", "lin_vel",
              "ang_vel"):
        setattr(s, f, getattr(scene, f)[b0:b1].copy())
    return s


def container_pour(n=262144, seed=0, mix=(0.5, 0.3, 0.0, 0.2), size_range=(0.1, 0.5), floor=(40.0, 40.0),
                   spawn_height=(1.0, 81.0), wall_height=90.0, hull_pool=256, hull_range=(16, 32), density=1000.0,
                   dt=1.0 / 120.0, iterations=10, real_bits=32) -> Scene:
    """One large scene: ``n`` bodies (box/sphere/cylinder/convex hull in ``mix`` proportions; box
    half-extents, sphere radii and hull scales U[size_range]) at uniform random positions and
    rotations in a floor[0] x floor[1] x (spawn_height) volume, above a static floor box and
    inside four static walls.  Hulls (hull_range vertices) come from a seeded pool shared by the
    bodies.  Bodies 0..4 are the floor and the walls."""
    rng = np.random.default_rng(seed)
    fx, fz = floor
    kinds = rng.choice(4, size=n, p=np.asarray(mix) / np.sum(mix))
    lo, hi = size_range
    pool_v, pool_f, pool_vol = [], [], []
    for _ in range(hull_pool):
        nv = int(rng.integers(hull_range[0], hull_range[1] + 1))
        v, f = random_hull(rng, nv, rng.uniform(lo, hi))
        pool_v.append(v)
        pool_f.append(f)
        pool_vol.append(_hull_volumes(v, f))
    pool_vol = np.array(pool_vol)
    he = rng.uniform(lo, hi, size=(n, 3))
    rs = rng.uniform(lo, hi, n)
    rc = rng.uniform(lo, hi, n)
    hc = rng.uniform(2 * lo, 2 * hi, n)
    pick = rng.integers(0, hull_pool, n)
    org = np.stack([rng.uniform(-fx / 2 + hi, fx / 2 - hi, n), rng.uniform(*spawn_height, n),
                    rng.uniform(-fz / 2 + hi, fz / 2 - hi, n)], axis=1)
    rot = random_rotations(rng, n)
    # shapes: hull pool, floor, x-walls, z-walls, then one shape per primitive body
    t = 1.0
    statics = [(BOX, (fx + 2 * t, t, fz + 2 * t), (0.0, -t / 2, 0.0)),
               (BOX, (t, wall_height, fz + 2 * t), (-fx / 2 - t / 2, wall_height / 2, 0.0)),
               (BOX, (t, wall_height, fz + 2 * t), (fx / 2 + t / 2, wall_height / 2, 0.0)),
               (BOX, (fx, wall_height, t), (0.0, wall_height / 2, -fz / 2 - t / 2)),
               (BOX, (fx, wall_height, t), (0.0, wall_height / 2, fz / 2 + t / 2))]
    prim = kinds != HULL
    n_prim = int(prim.sum())
    H, K = hull_pool, len(statics)
    S = H + K + n_prim
    shape_type = np.zeros(S, np.int32)
    shape_param = np.zeros((S, 3))
    shape_type[:H] = HULL
    for k, (ty, p, _) in enumerate(statics):
        shape_type[H + k] = ty
        shape_param[H + k] = p
    pk = kinds[prim]
    shape_type[H + K:] = pk
    par = np.zeros((n_prim, 3))
    par[pk == BOX] = 2 * he[prim][pk == BOX]
    par[pk == SPHERE, 0] = rs[prim][pk == SPHERE]
    par[pk == CYLINDER, 0] = rc[prim][pk == CYLINDER]
    par[pk == CYLINDER, 1] = hc[prim][pk == CYLINDER]
    shape_param[H + K:] = par
    body_shape_dyn = np.where(prim, 0, pick)
    body_shape_dyn[prim] = H + K + np.arange(n_prim)
    vol = np.where(kinds == BOX, np.prod(2 * he, axis=1),
                   np.where(kinds == SPHERE, 4.0 / 3.0 * np.pi * rs ** 3,
                            np.where(kinds == CYLINDER, np.pi * rc * rc * hc, pool_vol[pick])))
    vbeg, vcnt, fbeg, fcnt = (np.zeros(S, np.int32) for _ in range(4))
    vcnt[:H] = [len(v) for v in pool_v]
    fcnt[:H] = [len(f) for f in pool_f]
    vbeg[:H] = np.concatenate([[0], np.cumsum(vcnt[:H])[:-1]])
    fbeg[:H] = np.concatenate([[0], np.cumsum(fcnt[:H])[:-1]])
    N = n + K
    s = Scene(dt=dt, gravity=(0.0, -9.8, 0.0), iterations=iterations, real_bits=64)
    s.shape_type, s.shape_param = shape_type, shape_param
    s.hull_vbeg, s.hull_vcnt, s.hull_fbeg, s.hull_fcnt = vbeg, vcnt, fbeg, fcnt
    s.hull_verts = np.concatenate(pool_v).reshape(-1, 3)
    s.hull_face_idx = np.concatenate([np.asarray(f, np.int32).ravel() for f in pool_f])
    s.hull_face_off = np.arange(0, 3 * int(fcnt.sum()) + 1, 3, dtype=np.int32)
    s.body_shape = np.concatenate([H + np.arange(K), body_shape_dyn]).astype(np.int32)
    s.body_flags = np.concatenate([np.full(K, KINEMATIC), np.zeros(n)]).astype(np.int32)
    s.mass = np.concatenate([np.zeros(K), density * vol])
    s.friction = np.full(N, 0.5)
    s.restitution = np.zeros(N)
    s.lin_damp = np.zeros(N)
    s.ang_damp = np.zeros(N)
    s.origin = np.concatenate([np.array([p for _, _, p in statics]), org])
    s.basis = np.concatenate([np.tile(np.eye(3), (K, 1, 1)), rot])
    s.lin_vel = np.zeros((N, 3))
    s.ang_vel = np.zeros((N, 3))
    return s.rounded(real_bits) if real_bits == 32 else s
