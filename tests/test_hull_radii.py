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
