"""Shared helpers of the test-suite: golden fixtures and result comparison."""
import io
from pathlib import Path

import numpy as np

from pe_gb300.scene import Scene

GOLDEN = Path(__file__).resolve().parent / "golden"
STATE_KEYS = ["origin", "basis", "lin_vel", "ang_vel", "aabb_min", "aabb_max", "world_inv_inertia"]
RESULT_KEYS = ["res_a", "res_b", "point_size", "valid_mask", "friction", "restitution", "slots"]


def golden_names():
    """Fixtures with phase records of chosen steps (the trajectory-digest fixtures are separate)."""
    return sorted(p.stem for p in GOLDEN.glob("*.npz") if "_traj_" not in p.stem)


def traj_names():
    return sorted(p.stem for p in GOLDEN.glob("*_traj_*.npz"))


def _scene_from_bytes(b, bits):
    import tempfile, os
    fd, path = tempfile.mkstemp(suffix=".pescene")
    os.close(fd)
    try:
        Path(path).write_bytes(b)
        return Scene.read(path, real_bits=bits)
    finally:
        os.unlink(path)


def load_traj(name):
    """A trajectory fixture: the scene (with .margin), real bits, step count, the per-step SHA-256
    digests of the body states and the full states of the kept steps ({step: [N, 18]})."""
    z = np.load(GOLDEN / f"{name}.npz")
    bits = int(z["bits"])
    scene = _scene_from_bytes(z["scene"].tobytes(), bits)
    scene.margin = float(z["margin"])
    return scene, bits, int(z["steps"]), z["digests"], {int(k): z[f"state{k}"] for k in z["kept"]}


def state_rows(st):
    """Body states as rows of (origin 3, basis 9 row-major, v 3, w 3) doubles: the layout of the
    trajectory fixtures."""
    n = len(st["origin"])
    return np.concatenate([np.asarray(st["origin"], np.float64), np.asarray(st["basis"], np.float64).reshape(n, 9),
                           np.asarray(st["lin_vel"], np.float64), np.asarray(st["ang_vel"], np.float64)], axis=1)


def state_digest(st):
    import hashlib
    return np.frombuffer(hashlib.sha256(np.ascontiguousarray(state_rows(st), "<f8").tobytes()).digest(), np.uint8)


def load_golden(name):
    """A phase-record fixture: the scene (its contact margin in scene.margin), real bits, step count
    and the records of the chosen steps."""
    z = np.load(GOLDEN / f"{name}.npz")
    bits = int(z["bits"])
    scene = _scene_from_bytes(z["scene"].tobytes(), bits)
    scene.margin = float(z["margin"]) if "margin" in z else 0.0
    steps = {}
    for k in z["recorded"]:
        d = {f: z[f"s{k}_{f}"] for f in STATE_KEYS + RESULT_KEYS + ["pairs", "lin_vel_post", "ang_vel_post"]}
        d["axis_before"], d["axis_after"] = (int(x) for x in z[f"s{k}_axis"])
        steps[int(k)] = d
    return scene, bits, int(z["steps"]), steps


def results_of(d):
    return {k: d[k] for k in RESULT_KEYS}


def slot_masks(point_size):
    full = np.arange(8)[None, :] < np.asarray(point_size)[:, None]
    return full


def compare_results(got, ref, rtol=0.0, atol=0.0, what=""):
    """Contact results: bodies, counts, point slots (all fields below point_size, the carried
    distance of the remaining slots).  rtol = atol = 0 means bitwise equality."""
    assert len(got["res_a"]) == len(ref["res_a"]), f"{what}: result count {len(got['res_a'])} != {len(ref['res_a'])}"
    assert np.array_equal(got["res_a"], ref["res_a"]) and np.array_equal(got["res_b"], ref["res_b"]), f"{what}: bodies differ"
    bad = np.nonzero(got["point_size"] != ref["point_size"])[0]
    assert len(bad) == 0, f"{what}: point counts differ at results {bad[:10]}: {got['point_size'][bad[:10]]} vs {ref['point_size'][bad[:10]]}"
    m = slot_masks(ref["point_size"])
    g, r = got["slots"][m], ref["slots"][m]
    if rtol == 0 and atol == 0:
        diff = np.argwhere(g != r)
        assert len(diff) == 0, f"{what}: {len(diff)} slot values differ; first at {diff[:3]}: {g[tuple(diff[0])]} vs {r[tuple(diff[0])]}"
        assert np.array_equal(got["slots"][~m][:, 12], ref["slots"][~m][:, 12]), f"{what}: carried slot distances differ"
    else:
        np.testing.assert_allclose(g, r, rtol=rtol, atol=atol, err_msg=what)
    np.testing.assert_array_equal(got["friction"], ref["friction"])
    np.testing.assert_array_equal(got["restitution"], ref["restitution"])


def compare_state(got, ref, keys=STATE_KEYS, what=""):
    for k in keys:
        diff = np.argwhere(np.asarray(got[k]) != np.asarray(ref[k]))
        assert len(diff) == 0, f"{what}: {k} differs at {diff[:3]} ({np.asarray(got[k])[tuple(diff[0])]} vs {np.asarray(ref[k])[tuple(diff[0])]})"


def dump_state(d):
    return {k: d[k] for k in STATE_KEYS}


def mechanical_energy(state, scene, g=9.8):
    """Kinetic (linear + rotational, world inertia from the stored inverse) plus potential energy
    of the dynamic bodies."""
    dyn = scene.mass > 0
    m = scene.mass[dyn]
    v, w = state["lin_vel"][dyn], state["ang_vel"][dyn]
    inertia = np.linalg.inv(state["world_inv_inertia"][dyn])
    ke = 0.5 * m * np.einsum("ij,ij->i", v, v) + 0.5 * np.einsum("ni,nij,nj->n", w, inertia, w)
    return float(ke.sum() + (m * g * state["origin"][dyn, 1]).sum())


def max_penetration(results):
    """Deepest contact (positive = penetration) over the valid points of all results."""
    d = [results["slots"][i, :n, 12].min() for i, n in enumerate(results["point_size"]) if n]
    return float(max(0.0, -min(d))) if d else 0.0


def contact_residual(pre, post, results, scene, kerp=0.2, pen_th=0.3, rest_th=0.1):
    """Velocity-level residual of the contact rows after a solve: for every valid point, how far its
    normal relative velocity n . (v_a - v_b) at the contact falls short of the row's target
    (restitution of the pre-solve approach speed, zeroed below rest_th, minus the Baumgarte term
    kerp * max(depth, -pen_th) / dt), as FrictionContactConstraint::initSequentialImpulse sets it
    up.  `pre` and `post` are the body states before and after the solve; returns (rms, max) of
    max(0, target - n . v_rel) over the points."""
    slots, ps = results["slots"], results["point_size"]
    keep = np.arange(slots.shape[1])[None, :] < ps[:, None]
    ia = np.repeat(results["res_a"], slots.shape[1]).reshape(keep.shape)[keep]
    ib = np.repeat(results["res_b"], slots.shape[1]).reshape(keep.shape)[keep]
    rest = np.repeat(results["restitution"], slots.shape[1]).reshape(keep.shape)[keep]
    p = slots[keep]
    n, la, lb, depth = p[:, 3:6], p[:, 6:9], p[:, 9:12], p[:, 12]
    ra = np.einsum("nij,nj->ni", pre["basis"][ia], la)
    rb = np.einsum("nij,nj->ni", pre["basis"][ib], lb)

    def rel(s):
        va = s["lin_vel"][ia] + np.cross(s["ang_vel"][ia], ra)
        vb = s["lin_vel"][ib] + np.cross(s["ang_vel"][ib], rb)
        return np.einsum("ni,ni->n", n, va - vb)

    rev = -rel(pre)
    rev = np.where(np.abs(rev) < rest_th, 0.0, rev) * rest
    target = rev - kerp * np.maximum(depth, -pen_th) / scene.dt
    short = np.maximum(0.0, target - rel(post))
    if short.size == 0:
        return 0.0, 0.0
    return float(np.sqrt(np.mean(short ** 2))), float(short.max())
