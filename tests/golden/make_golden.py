"""Generate the golden fixtures of tests/golden/ by running the reference engine itself.

The reference is compiled from its own sources by oracle/build_ref.py (only possible where
those sources exist); each fixture stores a seeded synthetic scene and the reference's
phase records (state seen by the broadphase, ordered pairs, all contact-result cache slots,
post-solve velocities) for chosen steps.

Run from the repository root:  python tests/golden/make_golden.py
"""
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / "physics-engine_gb300"))
sys.path.insert(0, str(ROOT / "oracle"))

from pe_gb300 import scene as sc  # noqa: E402
from pe_gb300.scene_json import load_scene_json  # noqa: E402
import pedump  # noqa: E402
import build_ref  # noqa: E402

OUT = Path(__file__).resolve().parent
FIELDS = ["origin", "basis", "lin_vel", "ang_vel", "aabb_min", "aabb_max", "world_inv_inertia", "pairs", "res_a",
          "res_b", "point_size", "valid_mask", "friction", "restitution", "slots", "lin_vel_post", "ang_vel_post"]

# name -> (scene factory, real bits, steps to run, steps to record)
CASES = {
    "tower3_f64": (lambda: sc.tower(nx=3, ny=3, nz=3, real_bits=64), 64, 60, [0, 1, 2, 20, 21, 58, 59]),
    "tower3_f32": (lambda: sc.tower(nx=3, ny=3, nz=3, real_bits=32), 32, 60, [0, 1, 2, 20, 21, 58, 59]),
    "cube_f32": (lambda: sc.random_cube(n=400, seed=11, extent=12.0, real_bits=32), 32, 2, [0, 1]),
    "cube_f64": (lambda: sc.random_cube(n=400, seed=12, extent=12.0, real_bits=64), 64, 2, [0, 1]),
    "pile_f64": (lambda: sc.pile(48, seed=5, real_bits=64, hull_range=(8, 24), drop=(0.0, 0.3)), 64, 40,
                 [0, 1, 24, 25, 38, 39]),
    "pile_f32": (lambda: sc.pile(48, seed=6, real_bits=32, hull_range=(8, 24), drop=(0.0, 0.3)), 32, 40,
                 [0, 1, 24, 25, 38, 39]),
}
# joints: the reference's constraints demo (ball-joint pendulum, limited hinges, slider) plus a
# motor hinge and a hanging ball-joint chain, with ignored collision pairs
# (the "_nolimit" variants leave out the hinge angle limit, whose angle comes from atan2)
for bits in (64, 32):
    CASES[f"joints_f{bits}"] = (lambda bits=bits: sc.joint_demo(real_bits=bits), bits, 180,
                                [0, 1, 2, 30, 60, 61, 90, 120, 150, 178, 179])
    CASES[f"joints_nolimit_f{bits}"] = (lambda bits=bits: sc.joint_demo(hinge_limits=False, real_bits=bits), bits, 180,
                                        [0, 1, 2, 30, 60, 61, 90, 120, 150, 178, 179])
# static concave terrain: every body kind dropped on a 16 x 16 heightfield (512 faces, one face per
# tree leaf), and on a 64 x 64 one (8,192 faces, four faces per leaf)
for bits in (64, 32):
    CASES[f"terrain_f{bits}"] = (lambda bits=bits: sc.terrain_drop(n=40, seed=11, real_bits=bits), bits, 150,
                                 [0, 1, 30, 45, 60, 61, 90, 120, 148, 149])
CASES["terrain_big_f32"] = (lambda: sc.terrain_drop(n=120, nx=64, nz=64, seed=12, real_bits=32), 32, 90,
                            [0, 1, 40, 60, 61, 88, 89])
# compound bodies (jacks, dumbbells, box + hull caps) among primitives on a ground box
for bits in (64, 32):
    CASES[f"compound_f{bits}"] = (lambda bits=bits: sc.compound_pile(n=24, seed=3 + bits, drop=(0.0, 0.5), real_bits=bits),
                                  bits, 120, [0, 1, 2, 30, 31, 45, 60, 61, 90, 91, 118, 119])
# the reference's own sample scene (a bomb sphere at 70 m/s into a 15-box tower on a kinematic
# ground), read by the scene-file loader; the sphere reaches the tower near step 57
REF = build_ref.reference_dir()
if REF is None:
    raise SystemExit("reference sources not found: set PE_REFERENCE_DIR")
SAMPLES = REF / "SampleScenes"
for bits in (64, 32):
    CASES[f"json_bomb_tower_smaller_f{bits}"] = (
        lambda bits=bits: load_scene_json(SAMPLES / "bomb_crash_tower_smaller.json", real_bits=bits)[0], bits, 120,
        [0, 1, 30, 55, 56, 57, 58, 59, 60, 61, 62, 90, 119])
# a scene file naming the reference's own OBJ test meshes: its vase (589 faces) scaled 8x as a static
# concave body on a ground box, and its convex test mesh (42 faces) as falling bodies among boxes
# and spheres; written to a temporary file and read by the scene-file loader
def obj_scene(bits):
    import json
    import tempfile
    ref = REF / "test"
    bodies = [{"type": "box", "kinematic": True, "position": [0, -0.5, 0], "scale": [40, 1, 40]},
              {"type": "concave", "kinematic": True, "mesh": str(ref / "utils/bvh/vase.obj"), "scale": [8, 8, 8],
               "position": [0, 4.2, 0]}]
    rng = np.random.default_rng(7)
    for i in range(24):
        p = [float(rng.uniform(-3, 3)), float(8.5 + 0.9 * i), float(rng.uniform(-3, 3))]
        if i % 3 == 0:
            bodies.append({"type": "convex", "mesh": str(ref / "rigid/shape/convex_mesh_shape/mesh.obj"),
                           "scale": [0.8, 0.8, 0.8], "position": p, "mass": 2})
        elif i % 3 == 1:
            bodies.append({"type": "sphere", "scale": [0.35], "position": p})
        else:
            bodies.append({"type": "box", "scale": [0.6, 0.4, 0.5], "position": p, "rotation": [0.9, 0.1, 0.3, 0.2]})
    with tempfile.TemporaryDirectory() as td:
        f = Path(td) / "scene.json"
        f.write_text(json.dumps({"RigidBodies": bodies}))
        return load_scene_json(f, real_bits=bits)[0]


for bits in (64, 32):
    CASES[f"json_obj_f{bits}"] = (lambda bits=bits: obj_scene(bits), bits, 150, [0, 1, 40, 60, 61, 90, 120, 148, 149])
# the reference's sample scene compound.json: ten compound bodies (box hubs with cylinder arms)
# and four primitives dropped onto a kinematic ground box
for bits in (64, 32):
    CASES[f"json_compound_f{bits}"] = (
        lambda bits=bits: load_scene_json(SAMPLES / "compound.json", real_bits=bits)[0], bits, 150,
        [0, 1, 40, 60, 61, 90, 91, 120, 148, 149])
for a in range(4):
    for b in range(a, 4):
        CASES[f"zoo_{a}{b}_f64"] = (lambda a=a, b=b: sc.pair_zoo(a, b, m=48, seed=100 + 4 * a + b, real_bits=64), 64, 2, [0, 1])
for a, b in ((0, 0), (0, 2), (2, 2), (2, 3), (3, 3)):
    CASES[f"zoo_{a}{b}_f32"] = (lambda a=a, b=b: sc.pair_zoo(a, b, m=48, seed=200 + 4 * a + b, real_bits=32), 32, 2, [0, 1])

# contact margin 0.005 (the tower configuration's; the reference built with PE_MARGIN = 0.005
# through oracle/ref_margin.h): every pair type, and a small tower over 60 steps
MARGIN = build_ref.MARGIN_VARIANT
MARGIN_CASES = set()
for a in range(4):
    for b in range(a, 4):
        CASES[f"zoo_{a}{b}_m005_f64"] = (lambda a=a, b=b: sc.pair_zoo(a, b, m=48, seed=300 + 4 * a + b, real_bits=64), 64, 2, [0, 1])
        MARGIN_CASES.add(f"zoo_{a}{b}_m005_f64")
for a, b in ((0, 0), (0, 2), (2, 3), (3, 3)):
    CASES[f"zoo_{a}{b}_m005_f32"] = (lambda a=a, b=b: sc.pair_zoo(a, b, m=48, seed=400 + 4 * a + b, real_bits=32), 32, 2, [0, 1])
    MARGIN_CASES.add(f"zoo_{a}{b}_m005_f32")
for bits in (64, 32):
    CASES[f"tower3_m005_f{bits}"] = (lambda bits=bits: sc.tower(nx=3, ny=3, nz=3, real_bits=bits), bits, 60,
                                     [0, 1, 2, 20, 21, 58, 59])
    MARGIN_CASES.add(f"tower3_m005_f{bits}")
# whole trajectories recorded as per-step digests of the body states: the 1,002-body tower of the
# plain single-scene configuration (10 x 10 x 10 boxes, 50 kg sphere at 30 m/s, 20 iterations,
# margin 0.005), 300 steps
TRAJ = {"tower_m005_traj_f64": (lambda: sc.tower(real_bits=64), 64, 300, MARGIN, [149, 299])}


def state_digests(traj):
    """SHA-256 of each step's body states, rows of (origin 3, basis 9, v 3, w 3) doubles in scene
    order: the layout the reference harness writes with PE_TRAJ_OUT."""
    import hashlib
    return np.array([np.frombuffer(hashlib.sha256(np.ascontiguousarray(t, "<f8").tobytes()).digest(), np.uint8)
                     for t in traj])


def make_traj(name, ref_dir):
    import os
    factory, bits, steps, margin, keep = TRAJ[name]
    scene = factory()
    with tempfile.TemporaryDirectory() as td:
        sp = Path(td) / "s.pescene"
        tp = Path(td) / "t.bin"
        scene.write(sp)
        exe = ref_dir / f"ref_harness{bits}{'m' if margin else ''}"
        env = dict(os.environ, PE_TRAJ_OUT=str(tp))
        subprocess.run([str(exe), str(sp), str(Path(td) / "d"), str(steps), "8", "-1"], check=True, capture_output=True, env=env)
        traj = np.fromfile(tp, "<f8").reshape(steps, scene.n_bodies, 18)
    arrays = {"scene": np.frombuffer(scene_bytes(scene), np.uint8), "bits": np.array(bits),
              "steps": np.array(steps), "margin": np.array(margin), "digests": state_digests(traj),
              "kept": np.array(keep)}
    for k in keep:
        arrays[f"state{k}"] = traj[k]
    np.savez_compressed(OUT / f"{name}.npz", **arrays)
    return steps, len(keep)


def scene_bytes(scene):
    with tempfile.TemporaryDirectory() as td:
        sp = Path(td) / "s.pescene"
        scene.write(sp)
        return sp.read_bytes()


def make(name, ref_dir):
    if name in TRAJ:
        return make_traj(name, ref_dir)
    factory, bits, steps, rec = CASES[name]
    margin = MARGIN if name in MARGIN_CASES else 0.0
    scene = factory()
    with tempfile.TemporaryDirectory() as td:
        sp = Path(td) / "s.pescene"
        dp = Path(td) / "d.pedump"
        scene.write(sp)
        exe = ref_dir / f"ref_harness{bits}{'m' if margin else ''}"
        subprocess.run([str(exe), str(sp), str(dp), str(steps), "2", *map(str, rec)], check=True, capture_output=True)
        dumps = pedump.read(dp)
        arrays = {"scene": np.frombuffer(sp.read_bytes(), np.uint8), "bits": np.array(bits), "steps": np.array(steps),
                  "recorded": np.array([d["step"] for d in dumps]), "margin": np.array(margin)}
        for d in dumps:
            for f in FIELDS:
                arrays[f"s{d['step']}_{f}"] = d[f]
            arrays[f"s{d['step']}_axis"] = np.array([d["axis_before"], d["axis_after"]])
        np.savez_compressed(OUT / f"{name}.npz", **arrays)
    return sum(len(d["pairs"]) for d in dumps), sum(int(d["point_size"].sum()) for d in dumps)


if __name__ == "__main__":
    build_ref.build(REF, 8)
    names = sys.argv[1:] or sorted(CASES) + sorted(TRAJ)
    for name in names:
        p, c = make(name, build_ref.OUT)
        print(f"{name}: pairs {p} contact points {c}")
