"""The inner ball radius that the narrowphase's SAT axis pruning relies on (hull_radii in
csrc/pe_host_shapes.cpp): for every convex mesh it must not exceed the inradius about the local
origin of the hull of the mesh's vertices without vertex 0 (the projection loop never takes vertex 0
as the maximum), and the certification must refuse meshes whose faces do not close a convex
surface.  The host code is compiled with g++ and checked against scipy's convex hulls."""
import shutil
import struct
import subprocess
from pathlib import Path

import numpy as np
import pytest

from pe_gb300 import scene as sc

ROOT = Path(__file__).resolve().parent.parent
CSRC = ROOT / "physics-engine_gb300" / "csrc"
spatial = pytest.importorskip("scipy.spatial")


@pytest.fixture(scope="module")
def radii_tool(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    exe = tmp_path_factory.mktemp("hull_radii") / "hull_radii_check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", str(CSRC), "-I", "/usr/local/cuda/include",
                    str(ROOT / "tests" / "hull_radii_check.cpp"), str(CSRC / "pe_host_shapes.cpp"), "-o", str(exe)],
                   check=True, capture_output=True)

    def run(meshes):
        """meshes: list of (verts [n,3], faces list of index lists) -> per mesh {32: (inner, outer, V), 64: ...}"""
        buf = [struct.pack("i", len(meshes))]
        for v, faces in meshes:
            off = np.cumsum([0] + [len(f) for f in faces]).astype(np.int32)
            idx = np.concatenate([np.asarray(f, np.int32) for f in faces])
            buf += [struct.pack("iii", len(v), len(faces), len(idx)), np.ascontiguousarray(v, np.float64).tobytes(),
                    off.tobytes(), idx.tobytes()]
        inp = exe.parent / "meshes.bin"
        inp.write_bytes(b"".join(buf))
        out = subprocess.run([str(exe), str(inp)], check=True, capture_output=True, text=True).stdout.split("\n")
        res = []
        for m in range(len(meshes)):
            d = {}
            for line in out[2 * m:2 * m + 2]:
                t = line.split()
                n = int(t[3])
                d[int(t[0])] = (float(t[1]), float(t[2]), np.array(t[4:4 + 3 * n], float).reshape(n, 3))
            res.append(d)
        return res
    return run


def exact_radius(v):
    """Inradius about the origin of the hull of v[1:] (negative if the origin is not inside)."""
    h = spatial.ConvexHull(v[1:])
    return float((-h.equations[:, 3]).min())


def scene_meshes(s, limit):
    out = []
    for k in range(s.n_shapes):
        if s.shape_type[k] != sc.HULL:
            continue
        vb, vc, fb, fc = s.hull_vbeg[k], s.hull_vcnt[k], s.hull_fbeg[k], s.hull_fcnt[k]
        off = s.hull_face_off[fb:fb + fc + 1]
        faces = [s.hull_face_idx[off[i]:off[i + 1]] for i in range(fc)]
        out.append((s.hull_verts[vb:vb + vc], faces))
        if len(out) == limit:
            break
    return out


def cube(inward=False, drop_face=False):
    v = np.array([[x, y, z] for x in (-0.5, 0.5) for y in (-0.5, 0.5) for z in (-0.5, 0.5)])
    quads = [[0, 1, 3, 2], [4, 6, 7, 5], [0, 4, 5, 1], [2, 3, 7, 6], [0, 2, 6, 4], [1, 5, 7, 3]]
    faces = []
    for q in quads:   # outward-wound triangles
        faces += [[q[0], q[1], q[2]], [q[0], q[2], q[3]]]
    if inward:
        faces = [f[::-1] for f in faces]
    if drop_face:
        faces = faces[2:]
    return v, faces


@pytest.mark.parametrize("which", ["batched_piles", "container_pour"])
def test_generated_hulls_radii_are_safe_and_tight(radii_tool, which):
    s = sc.batched_piles(n_scenes=8, seed=0)[0] if which == "batched_piles" else \
        sc.container_pour(n=256, seed=3, floor=(10.0, 10.0), hull_pool=32, real_bits=32)
    meshes = scene_meshes(s, 96)
    assert len(meshes) >= 8
    for m, d in enumerate(radii_tool(meshes)):
        for bits, (inner, outer, v) in d.items():
            r = exact_radius(v)
            assert inner <= r, (which, m, bits, inner, r)
            assert inner >= r - 1e-5 * outer, (which, m, bits, inner, r)   # certified, not refused
            assert outer >= np.linalg.norm(v, axis=1).max()


def test_cube_radius_holds_without_vertex_0(radii_tool):
    """A cube's corner 0 cut off leaves the plane through its three neighbours at 0.5 / sqrt(3) from
    the centre; with either winding the certified radius is that distance (less 1e-6 of the outer
    radius), not the cube's 0.5."""
    for inward in (False, True):
        d = radii_tool([cube(inward=inward)])[0]
        for bits, (inner, outer, v) in d.items():
            assert abs(inner - 0.5 / np.sqrt(3)) < 2e-6, (inward, bits, inner)
            assert inner <= exact_radius(v)


def octahedron_faces():
    faces = []
    for a in (0, 1):
        for b, c in ((2, 4), (4, 3), (3, 5), (5, 2)):
            faces.append([a, b, c] if a == 0 else [a, c, b])
    return faces


def test_spike_at_vertex_0(radii_tool):
    """An octahedron whose vertex 0 is pulled far out: its centroid lies outside the hull of the
    other vertices, so no radius holds for the maximum side and the mesh is refused (-1)."""
    v = np.array([[4.0, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1]])
    for bits, (inner, outer, vp) in radii_tool([(v, octahedron_faces())])[0].items():
        assert exact_radius(vp) < 0
        assert inner == -1.0, (bits, inner)


def test_vertex_exposed_by_removing_vertex_0(radii_tool):
    """A bump at vertex 0 over a vertex that lies on no face: without vertex 0 the hidden vertex
    becomes a corner of the hull, and the certified radius is that hull's inradius."""
    v = np.array([[1.3, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1], [1, 0, 0]])
    for bits, (inner, outer, vp) in radii_tool([(v, octahedron_faces())])[0].items():
        r = exact_radius(vp)
        assert 0 < inner <= r, (bits, inner, r)
        assert inner >= r - 1e-5 * outer, (bits, inner, r)


def test_uncertifiable_meshes_are_refused(radii_tool):
    """An open mesh (two triangles missing) and a non-convex closed mesh get no radius (-1), so the
    SAT prunes none of their axes."""
    v, faces = cube(drop_face=True)
    # an L-shaped prism: closed, but a face plane has vertices in front of it
    L = np.array([[0, 0, 0], [2, 0, 0], [2, 1, 0], [1, 1, 0], [1, 2, 0], [0, 2, 0]], float)
    Lv = np.concatenate([L, L + [0, 0, 1]])
    side = [[i, (i + 1) % 6, 6 + (i + 1) % 6, 6 + i] for i in range(6)]
    bottom = [[0, 3, 2, 1], [0, 5, 4, 3]]
    top = [[6, 7, 8, 9], [6, 9, 10, 11]]
    Lf = []
    for q in side + bottom + top:
        Lf += [[q[0], q[1], q[2]], [q[0], q[2], q[3]]]
    for d in radii_tool([(v, faces), (Lv, Lf)]):
        for bits, (inner, outer, _) in d.items():
            assert inner == -1.0, (bits, inner)


def _rot(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                     [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                     [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])


def _hull_interval(v, basis, origin, axis):
    """The reference's hull projection in FP32 (convex_mesh_shape.cpp:160-183): the minimum over all
    vertices, the maximum over the vertices that were not a running minimum when visited (so never
    vertex 0), both offset by origin . axis."""
    f = np.float32
    la = (basis.T.astype(f) @ axis.astype(f)).astype(f)
    p = (v[:, 0].astype(f) * la[0] + v[:, 1].astype(f) * la[1]).astype(f) + v[:, 2].astype(f) * la[2]
    mn, mx = f(3.4e38), f(-1e30)
    for x in p.astype(f):
        if x < mn:
            mn = x
        elif x > mx:
            mx = x
    off = f(origin.astype(f) @ axis.astype(f))
    return f(mn + off), f(mx + off), float(off)


def test_prune_bound_never_exceeds_the_computed_depth(radii_tool):
    """For hull pairs at random overlapping poses, along random axes and along the directions of each
    hull's vertex 0 (the vertex the projection never takes as the maximum), the SAT's pruning bound
    min(loA - hiB, loB - hiA) with [o - r, o + r] per hull stays below the FP32 depth the projection
    computes, within the bound's roundoff allowance (64 units of the magnitudes).  A radius certified
    for the whole hull instead of the hull without vertex 0 fails this along those directions."""
    s = sc.batched_piles(n_scenes=8, seed=0)[0]
    hulls = [d[32] for d in radii_tool(scene_meshes(s, 40))]
    rng = np.random.default_rng(11)
    u = 1.1920929e-7
    checked = 0
    for t in range(400):
        (ra, oa_, va), (rb, ob_, vb) = hulls[rng.integers(len(hulls))], hulls[rng.integers(len(hulls))]
        if ra <= 0 or rb <= 0:
            continue
        Ba, Bb = _rot(rng), _rot(rng)
        oa = rng.uniform(-50, 50, 3)
        ob = oa + rng.normal(size=3) * 0.3 * (oa_ + ob_)
        axes = [a / np.linalg.norm(a) for a in rng.normal(size=(8, 3))]
        axes += [Ba @ va[0] / np.linalg.norm(va[0]), Bb @ vb[0] / np.linalg.norm(vb[0])]
        axes += [-(Bb @ vb[0]) / np.linalg.norm(vb[0]), -(Ba @ va[0]) / np.linalg.norm(va[0])]
        for ax in axes:
            mnA, mxA, cA = _hull_interval(va, Ba, oa, ax)
            mnB, mxB, cB = _hull_interval(vb, Bb, ob, ax)
            depth = min(float(mxA) - float(mnB), float(mxB) - float(mnA))
            lb = min((cA + ra) - (cB - rb), (cB + rb) - (cA - ra))
            slack = 64 * u * (abs(cA) + oa_ + abs(cB) + ob_)
            assert lb - slack <= depth, (t, lb, depth, slack)
            checked += 1
    assert checked > 1000


def test_ball_lies_within_each_computed_interval(radii_tool):
    """Per hull, along every outward facet normal of the hull without vertex 0 (where the computed
    maximum is smallest), along the vertex-0 directions and along random directions, at a random pose:
    the computed FP32 interval [min, max] holds [o - r, o + r] within the bound's roundoff allowance.
    Along those facet normals a radius certified for the whole hull falls outside on several hulls."""
    s = sc.batched_piles(n_scenes=8, seed=0)[0]
    hulls = [d[32] for d in radii_tool(scene_meshes(s, 40))]
    rng = np.random.default_rng(5)
    u = 1.1920929e-7
    for r, outer, v in hulls:
        assert r > 0
        B, o = _rot(rng), rng.uniform(-50, 50, 3)
        facets = spatial.ConvexHull(v[1:]).equations[:, :3]
        dirs = [B @ n for n in facets] + [B @ v[0] / np.linalg.norm(v[0])]
        dirs += [a / np.linalg.norm(a) for a in rng.normal(size=(16, 3))]
        for ax in dirs:
            for sgn in (1.0, -1.0):
                mn, mx, c = _hull_interval(v, B, o, sgn * ax)
                slack = 64 * u * (abs(c) + outer)
                assert float(mx) >= c + r - slack and float(mn) <= c - r + slack, (r, float(mn), float(mx), c)
