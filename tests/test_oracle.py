"""CPU tests: the oracle against the reference's own outputs (golden fixtures produced by
running the reference engine, tests/golden/make_golden.py) and against the known answers
asserted by the reference's unit tests.  No GPU needed."""
import numpy as np
import pytest

import orc
from pe_gb300 import scene as sc
from pe_testlib import (compare_results, compare_state, dump_state, golden_names, load_golden, load_traj, results_of,
                        state_digest, state_rows, traj_names)


@pytest.mark.parametrize("name", golden_names())
def test_oracle_trajectory_matches_reference(name):
    """Stepping the oracle from the scene reproduces the reference bit for bit at every
    recorded step: poses, AABBs, world inertia, ordered pairs, contact caches, velocities."""
    scene, bits, steps, rec = load_golden(name)
    w = orc.OracleWorld(scene, bits, margin=scene.margin)
    done = 0
    for k in sorted(rec):
        w.step(k + 1 - done)
        done = k + 1
        d = rec[k]
        st = w.state()
        compare_state(st, dump_state(d), keys=["origin", "basis", "aabb_min", "aabb_max", "world_inv_inertia"], what=f"{name} step {k}")
        np.testing.assert_array_equal(st["lin_vel"], d["lin_vel_post"])
        np.testing.assert_array_equal(st["ang_vel"], d["ang_vel_post"])
        np.testing.assert_array_equal(w.pairs(), d["pairs"])
        compare_results(w.results(), results_of(d), what=f"{name} step {k}")
        assert w.axis == d["axis_after"]


@pytest.mark.parametrize("name", golden_names())
def test_oracle_phases_from_reference_state(name):
    """Each phase of the oracle, fed the reference's own inputs, gives the reference's outputs."""
    scene, bits, steps, rec = load_golden(name)
    w = orc.OracleWorld(scene, bits, margin=scene.margin)
    for k in sorted(rec):
        d = rec[k]
        # broadphase on the reference's AABBs and sweep axis
        w.set_state(dump_state(d))
        w.axis = d["axis_before"]
        w.broadphase()
        np.testing.assert_array_equal(w.pairs(), d["pairs"])
        assert w.axis == d["axis_after"]
        # narrowphase on the reference's pairs, with the previous step's pooled results
        if k - 1 in rec:
            w.set_results(results_of(rec[k - 1]))
            w.set_pairs(d["pairs"])
            w.narrowphase()
            compare_results(w.results(), results_of(d), what=f"{name} narrowphase step {k}")
        # solver on the reference's contact results
        w.set_state(dump_state(d))
        w.set_results(results_of(d))
        w.solve()
        st = w.state()
        np.testing.assert_array_equal(st["lin_vel"], d["lin_vel_post"])
        np.testing.assert_array_equal(st["ang_vel"], d["ang_vel_post"])
        # integration from the previous step's final state
        if k - 1 in rec:
            p = rec[k - 1]
            s0 = dump_state(p)
            s0["lin_vel"], s0["ang_vel"] = p["lin_vel_post"], p["ang_vel_post"]
            w.set_state(s0)
            w.integrate()
            compare_state(w.state(), dump_state(d), what=f"{name} integrate step {k}")


@pytest.mark.parametrize("name", traj_names())
def test_oracle_whole_trajectory_matches_reference(name):
    """Every step of a long trajectory of the reference (the 1,002-body tower at contact margin
    0.005, 300 steps, the sphere's impact included) is reproduced bit for bit by the oracle: the
    per-step digests of all body states agree, and the kept full states are equal."""
    scene, bits, steps, digests, kept = load_traj(name)
    w = orc.OracleWorld(scene, bits, threads=4, margin=scene.margin)
    for k in range(steps):
        w.step(1)
        st = w.state()
        if k in kept:
            np.testing.assert_array_equal(state_rows(st), kept[k], err_msg=f"{name} step {k}")
        assert np.array_equal(state_digest(st), digests[k]), f"{name}: body states differ from the reference at step {k}"


def test_margin_changes_the_contacts():
    """The margin fixtures are not the plain ones: contact margin 0.005 shifts every contact
    point's depth by 2 margin (pt - n margin, depth + 2 margin in each pair algorithm)."""
    _, _, _, rec = load_golden("zoo_00_m005_f64")
    scene, bits, _, _ = load_golden("zoo_00_m005_f64")
    assert scene.margin == 0.005
    w0 = orc.OracleWorld(scene, bits)
    w1 = orc.OracleWorld(scene, bits, margin=scene.margin)
    for w in (w0, w1):
        w.step(1)
    r0, r1 = w0.results(), w1.results()
    assert np.array_equal(r1["point_size"], rec[0]["point_size"])
    assert not np.array_equal(r0["slots"], r1["slots"])


# ------------------------------------------------------------------ reference unit-test answers
def kat_boxes(positions, sizes, kinematic=(), mass=1.0, friction=0.5, restitution=0.5, dt=0.01, gravity=(0, 0, 0)):
    b = sc.SceneBuilder(dt=dt, gravity=gravity)
    for i, (p, s) in enumerate(zip(positions, sizes)):
        b.body(b.shape(sc.BOX, s), p, mass=mass, friction=friction, restitution=restitution, kinematic=i in kinematic)
    return b.build()


def zero_aabbs(w):
    st = w.state()
    st["aabb_min"][:] = 0
    st["aabb_max"][:] = 0
    w.set_state(st)


def test_kat_broadphase_two_pairs():
    """test/rigid/collision/broad_phase/test.cpp:15-33: four unit boxes, the upper two kinematic -> 2 pairs."""
    s = kat_boxes([(0, 0, 0), (0, 0.5, 0), (0, 1.1, 0), (0, 1.6, 0)], [(1, 1, 1)] * 4, kinematic=(2, 3), dt=1e-30)
    w = orc.OracleWorld(s, 64)
    w.integrate()
    assert w.broadphase() == 2


def test_kat_narrowphase_four_points():
    """test/rigid/collision/narrow_phase/test.cpp:16-25: unit boxes 0.99 apart -> 1 result with 4 points."""
    s = kat_boxes([(0, 0, 0), (0, 0.99, 0)], [(1, 1, 1)] * 2)
    w = orc.OracleWorld(s, 64)
    zero_aabbs(w)
    w.set_pairs([[0, 1]])
    w.narrowphase()
    r = w.results()
    assert len(r["res_a"]) == 1 and r["point_size"][0] == 4


def test_kat_ground_box_four_points():
    """test/rigid/constraint/friction_contact_constraint/test.cpp:20-30: box resting on a slab -> 4 points."""
    s = kat_boxes([(0, -1, 0), (0, 0.999, 0)], [(40, 2, 40), (2, 2, 2)], friction=0.5, restitution=1.0)
    w = orc.OracleWorld(s, 64)
    zero_aabbs(w)
    w.set_pairs([[1, 0]])
    w.narrowphase()
    assert w.results()["point_size"][0] == 4


def test_kat_integration():
    """test/rigid/object/rigidbody/test.cpp:15-24: v=(1,0,0), w=(0,1,0), dt=0.01."""
    b = sc.SceneBuilder(dt=0.01, gravity=(0, 0, 0))
    b.body(b.shape(sc.BOX, (1, 1, 1)), (0, 0, 0), mass=2.0, v=(1, 0, 0), w=(0, 1, 0))
    w = orc.OracleWorld(b.build(), 64)
    w.integrate()
    st = w.state()
    np.testing.assert_allclose(st["origin"][0], [0.01, 0, 0], atol=1e-4)
    c, s_ = np.cos(0.01), np.sin(0.01)
    np.testing.assert_allclose(st["basis"][0], [[c, 0, s_], [0, 1, 0], [-s_, 0, c]], atol=1e-4)


def test_oracle_stale_slot_distances_truncate_results():
    """A pooled contact result keeps the distances of its empty slots from the previous step;
    a stale distance smaller than a new point's distance ends the point list early
    (contact_result.cpp:144-156 sorts all 8 slots).  Seeded here on purpose."""
    s = kat_boxes([(0, 0, 0), (0, 0.99, 0)], [(1, 1, 1)] * 2)
    w = orc.OracleWorld(s, 64)
    w.integrate()
    w.set_pairs([[0, 1]])
    w.narrowphase()
    fresh = w.results()
    assert fresh["point_size"][0] == 4
    seeded = {k: v.copy() for k, v in fresh.items()}
    seeded["slots"][0, :, 12] = -1.0           # every slot carries a deep stale distance
    w.set_results(seeded)
    w.narrowphase()
    assert w.results()["point_size"][0] == 0   # all new points sort behind invalid slots


def test_batched_piles_extract_round_trip():
    """Scenes extracted from a generated batch carry exactly the batch's bodies and shapes."""
    merged, offs = sc.batched_piles(n_scenes=12, seed=3, size_range=(8, 40), hull_pool=6, real_bits=32)
    assert offs[-1] == merged.n_bodies and len(offs) == 13
    parts = [sc.extract(merged, offs, k) for k in range(12)]
    again, offs2 = sc.concat(parts)
    np.testing.assert_array_equal(offs, offs2)
    for f in ("body_flags", "mass", "origin", "basis", "lin_vel"):
        np.testing.assert_array_equal(getattr(again, f), getattr(merged, f))
    for k, p in enumerate(parts):
        assert p.body_flags[0] == sc.KINEMATIC and p.mass[0] == 0.0   # ground first
        for i in range(p.n_bodies):
            t0, t1 = merged.shape_type[merged.body_shape[offs[k] + i]], p.shape_type[p.body_shape[i]]
            assert t0 == t1
            np.testing.assert_array_equal(merged.shape_param[merged.body_shape[offs[k] + i]], p.shape_param[p.body_shape[i]])
