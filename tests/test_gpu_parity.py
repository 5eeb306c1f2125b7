"""GPU parity: the CUDA path through the C ABI against the reference's recorded outputs
(golden fixtures) and against the oracle on seeded scenes, phase by phase and step by step.
Integer outputs (pair sets, contact counts) must match exactly; the arithmetic reproduces the
reference's operation order, so real-valued outputs are compared bit for bit as well, with
the documented tolerance (1e-5 relative for contact geometry, 1e-6 for solved velocities)
used only where an operation order differs by design."""
import numpy as np
import pytest

import orc
import pe_gb300 as pg
from pe_gb300 import scene as sc
from pe_testlib import (compare_results, compare_state, dump_state, golden_names, load_golden, load_traj, results_of,
                        state_digest, state_rows, traj_names)

pytestmark = pytest.mark.gpu


# fixtures whose hinge angle limits are active: the limit angle comes from atan2, where CUDA's
# and the C library's results may differ in the last place, and (min_angle - angle) cancels, so
# their solved velocities are held to a per-step bound instead of bit equality: 1e-6 in FP64,
# 5e-6 in FP32 (a last-place change of a float angle near the limit moves the limit impulse's
# velocities by up to ~3e-6)
ATAN2_FIXTURES = {"joints_f64", "joints_f32"}
PER_STEP_ATOL = {64: 1e-6, 32: 5e-6}


def keys_tie_free(d, axis):
    k = d["aabb_min"][:, axis]
    return len(np.unique(k)) == len(k)


@pytest.mark.parametrize("name", golden_names())
def test_gpu_phases_match_reference(name):
    scene, bits, steps, rec = load_golden(name)
    g = pg.GpuWorld(scene, bits, margin=scene.margin)
    for k in sorted(rec):
        d = rec[k]
        # broadphase: the pair set exactly; the order too when no two sort keys tie
        g.set_state(dump_state(d))
        g.axis = d["axis_before"]
        g.broadphase()
        got = g.pairs()
        ref = d["pairs"]
        assert sorted(map(tuple, np.sort(got, axis=1))) == sorted(map(tuple, np.sort(ref, axis=1))), f"{name} step {k}: pair sets differ"
        if keys_tie_free(d, d["axis_before"]):
            np.testing.assert_array_equal(got, ref)
        # narrowphase on the reference's pairs with the previous step's pooled results
        if k - 1 in rec:
            g.set_results(results_of(rec[k - 1]))
            g.set_pairs(ref)
            g.narrowphase()
            compare_results(g.results(), results_of(d), what=f"{name} narrowphase step {k}")
        # serial-order solver on the reference's contact results
        g.set_state(dump_state(d))
        g.set_results(results_of(d))
        g.solve(pg.SERIAL_ORDER)
        st = g.state()
        if name in ATAN2_FIXTURES:
            for f in ("lin_vel", "ang_vel"):
                np.testing.assert_allclose(st[f], d[f + "_post"], rtol=0, atol=PER_STEP_ATOL[bits],
                                           err_msg=f"{name} solve step {k}")
        else:
            np.testing.assert_array_equal(st["lin_vel"], d["lin_vel_post"], err_msg=f"{name} solve step {k}")
            np.testing.assert_array_equal(st["ang_vel"], d["ang_vel_post"], err_msg=f"{name} solve step {k}")
        # integration from the previous step's end state
        if k - 1 in rec:
            p = rec[k - 1]
            s0 = dump_state(p)
            s0["lin_vel"], s0["ang_vel"] = p["lin_vel_post"], p["ang_vel_post"]
            g.set_state(s0)
            g.integrate()
            compare_state(g.state(), dump_state(d), what=f"{name} integrate step {k}")


@pytest.mark.parametrize("name", ["cube_f32", "cube_f64", "zoo_22_f64", "zoo_23_f32", "zoo_33_f64", "pile_f64", "compound_f64",
                                  "compound_f32", "joints_nolimit_f64", "joints_nolimit_f32", "terrain_f64", "terrain_f32",
                                  "terrain_big_f32", "json_obj_f64", "json_obj_f32"])
def test_gpu_full_steps_serial_order_match_reference(name):
    """Whole steps on the device in serial-order mode reproduce the reference trajectory
    (scenes whose sort keys never tie, so the broadphase order is the reference's)."""
    scene, bits, steps, rec = load_golden(name)
    g = pg.GpuWorld(scene, bits, margin=scene.margin)
    done = 0
    for k in sorted(rec):
        g.step(k + 1 - done, pg.SERIAL_ORDER)
        done = k + 1
        d = rec[k]
        st = g.state()
        compare_state(st, dump_state(d), keys=["origin", "basis", "aabb_min", "aabb_max", "world_inv_inertia"], what=f"{name} step {k}")
        np.testing.assert_array_equal(st["lin_vel"], d["lin_vel_post"])
        np.testing.assert_array_equal(g.pairs(), d["pairs"])
        compare_results(g.results(), results_of(d), what=f"{name} step {k}")


@pytest.mark.parametrize("name", ["json_bomb_tower_smaller_f64", "json_bomb_tower_smaller_f32", "json_compound_f64",
                                  "json_compound_f32"])
def test_gpu_scene_file_full_steps_match_reference(name):
    """The reference's sample scenes bomb_crash_tower_smaller.json and compound.json (read by the
    scene-file loader) stepped on the device in serial-order mode: every whole step after the
    first reproduces the reference's trajectory (through the bomb's impact at steps 58-62; the
    compounds landing from step 40 on).  The steps start from the reference's state after step 0,
    the one step whose sort keys tie (tied keys fix the pair set, not its order)."""
    scene, bits, steps, rec = load_golden(name)
    g = pg.GpuWorld(scene, bits, margin=scene.margin)
    d0 = rec[0]
    s0 = dump_state(d0)
    s0["lin_vel"], s0["ang_vel"] = d0["lin_vel_post"], d0["ang_vel_post"]
    g.set_state(s0)
    g.set_results(results_of(d0))
    g.axis = int(d0["axis_after"])
    done = 1
    for k in sorted(rec)[1:]:
        g.step(k + 1 - done, pg.SERIAL_ORDER)
        done = k + 1
        d = rec[k]
        st = g.state()
        compare_state(st, dump_state(d), keys=["origin", "basis", "aabb_min", "aabb_max", "world_inv_inertia"], what=f"{name} step {k}")
        np.testing.assert_array_equal(st["lin_vel"], d["lin_vel_post"])
        np.testing.assert_array_equal(st["ang_vel"], d["ang_vel_post"])
        np.testing.assert_array_equal(g.pairs(), d["pairs"])
        compare_results(g.results(), results_of(d), what=f"{name} step {k}")


def test_gpu_compound_pile_matches_oracle():
    """300 compound bodies (jacks, dumbbells, box + hull caps) among 200 primitives, FP32: 60
    whole serial-order steps equal the oracle's, checked every 10 steps (state, pairs, every
    contact result), so compound-primitive pairs in both orders and compound-compound pairs all
    run through the compound kernel."""
    scene = sc.compound_pile(n=300, n_primitives=200, seed=9, spacing=2.4, drop=(0.0, 0.5), real_bits=32)
    o = orc.OracleWorld(scene, 32, threads=8)
    g = pg.GpuWorld(scene, 32)
    comp = np.nonzero(scene.shape_type[scene.body_shape] == sc.COMPOUND)[0]
    seen = 0
    for k in range(6):
        o.step(10)
        g.step(10, pg.SERIAL_ORDER)
        compare_state(g.state(), o.state(), what=f"compound pile step {10 * k + 9}")
        np.testing.assert_array_equal(g.pairs(), o.pairs())
        ro = o.results()
        compare_results(g.results(), ro, what=f"compound pile step {10 * k + 9}")
        seen += int(ro["point_size"][np.isin(ro["res_a"], comp)].sum())
    assert seen > 200


def largest_island(res, kinematic):
    """Results with points in the largest island of dynamic bodies (union-find on the host)."""
    a, b = res["res_a"][res["point_size"] > 0], res["res_b"][res["point_size"] > 0]
    parent = {}

    def find(x):
        while parent.setdefault(x, x) != x:
            parent[x] = parent[parent[x]]
            x = parent[x]
        return x
    for x, y in zip(a, b):
        if not kinematic[x] and not kinematic[y]:
            parent[find(x)] = find(y)
    sizes = {}
    for x, y in zip(a, b):
        r = find(y if kinematic[x] else x)
        sizes[r] = sizes.get(r, 0) + 1
    return max(sizes.values())


def test_gpu_big_island_serial_order_matches_oracle():
    """A settled pour of 4,096 bodies in a 10 x 10 m container forms one island of more than 4,096
    contact results, which serial-order mode runs as the grid-wide level schedule (cooperative
    colouring rounds and passes).  From the oracle's state, five steps with the oracle's pair order
    give the oracle's contacts and velocities bit for bit."""
    scene = sc.container_pour(n=4096, seed=3, floor=(10.0, 10.0), spawn_height=(1.0, 21.0), wall_height=25.0, hull_pool=32,
                              real_bits=32)
    o = orc.OracleWorld(scene, 32, threads=16)
    o.step(400)
    assert largest_island(o.results(), (scene.body_flags & sc.KINEMATIC) != 0) > 4096
    g = pg.GpuWorld(scene, 32)
    g.set_state(o.state())
    g.set_results(o.results())
    g.axis = o.axis
    for k in range(5):
        o.integrate()
        g.integrate()
        compare_state(g.state(), o.state(), what=f"integrate {k}")
        o.broadphase()
        g.broadphase()
        po = o.pairs()
        assert sorted(map(tuple, np.sort(po, axis=1))) == sorted(map(tuple, np.sort(g.pairs(), axis=1)))
        g.set_pairs(po)
        o.narrowphase()
        g.narrowphase()
        compare_results(g.results(), o.results(), what=f"narrowphase {k}")
        o.solve()
        g.solve(pg.SERIAL_ORDER)
        so, sg = o.state(), g.state()
        np.testing.assert_array_equal(sg["lin_vel"], so["lin_vel"], err_msg=f"solve {k}")
        np.testing.assert_array_equal(sg["ang_vel"], so["ang_vel"], err_msg=f"solve {k}")


def test_gpu_crowded_windows_match_oracle():
    """A 40 x 40 m container of 40,000 bodies: its floor and walls overlap every body along the sweep
    axis, so their sweep windows hold tens of thousands of candidates and are swept in chunks.  At
    the initial state and after 150 steps (bodies on the floor) the pair list equals the oracle's,
    order included where no two sort keys tie."""
    scene = sc.container_pour(n=40000, seed=8, real_bits=32)
    o = orc.OracleWorld(scene, 32, threads=16)
    g = pg.GpuWorld(scene, 32)
    for k in range(2):
        if k == 1:
            o.step(150)
            g.set_state(o.state())
            g.set_results(o.results())
            g.axis = o.axis
        g.axis = o.axis
        o.integrate()
        g.integrate()
        compare_state(g.state(), o.state(), what=f"integrate {k}")
        o.broadphase()
        g.broadphase()
        po, pgpu = o.pairs(), g.pairs()
        assert len(po) == len(pgpu)
        assert sorted(map(tuple, np.sort(po, axis=1))) == sorted(map(tuple, np.sort(pgpu, axis=1)))

        key = g.state()["aabb_min"][:, o.axis if k == 0 else g.axis]

        def partners(pairs):   # each sweep position's partners in emission order, and their sort keys
            out = {}
            for a, b in pairs:
                out.setdefault(int(a), []).append(int(b))
            return {a: (sorted(v), [float(key[b]) for b in v]) for a, v in out.items()}
        # tied sort keys (the container parts, and a few of the 40,000 float minima) may swap
        # segments or partners with equal keys; otherwise each position's partners (one crowded
        # window swept in chunks) come in the oracle's ascending order
        assert partners(pgpu) == partners(po)
        floor_pairs = int(((po == 0).any(axis=1)).sum())
    assert floor_pairs > 1000


def test_gpu_terrain_matches_oracle():
    """600 bodies of every kind (compounds included) dropped on a 96 x 96 concave heightfield
    (18,432 triangles: face-tree leaves of nine faces), FP32: 60 whole serial-order steps equal the
    oracle's, checked every 10 steps (state, pairs, every contact result)."""
    scene = sc.terrain_drop(n=600, nx=96, nz=96, seed=23, real_bits=32)
    o = orc.OracleWorld(scene, 32, threads=8)
    g = pg.GpuWorld(scene, 32)
    touching = 0
    for k in range(6):
        o.step(10)
        g.step(10, pg.SERIAL_ORDER)
        compare_state(g.state(), o.state(), what=f"terrain step {10 * k + 9}")
        np.testing.assert_array_equal(g.pairs(), o.pairs())
        ro = o.results()
        compare_results(g.results(), ro, what=f"terrain step {10 * k + 9}")
        touching = int(((ro["res_a"] == 0) | (ro["res_b"] == 0)).sum())
    assert touching > 300


def test_gpu_ignore_collision_bodies_match_oracle():
    """Bodies flagged ignore-collision (RigidBody::setIgnoreCollision) take part in no pair: a
    mixed 4,096-body scene with every fifth body flagged gives the oracle's pairs and contacts."""
    scene = sc.random_cube(n=4096, seed=23, extent=24.0, real_bits=32)
    scene.body_flags[::5] |= sc.IGNORE_COLLISION
    o = orc.OracleWorld(scene, 32)
    g = pg.GpuWorld(scene, 32)
    for w in (o, g):
        w.integrate()
        w.broadphase()
    po, pgpu = o.pairs(), g.pairs()
    assert len(po) > 1000
    assert not np.isin(po, np.arange(0, 4096, 5)).any()
    np.testing.assert_array_equal(pgpu, po)
    o.narrowphase()
    g.narrowphase()
    compare_results(g.results(), o.results(), what="ignore-collision narrowphase")


def test_gpu_stress_scene_broadphase_and_narrowphase_match_oracle():
    """65,536 mixed bodies in a 100 m cube (one-step stress): integration bit-exact, the
    pair set exact, and every contact result exact given the oracle's pair order."""
    scene = sc.random_cube(n=65536, seed=7, real_bits=32)
    o = orc.OracleWorld(scene, 32, threads=8)
    g = pg.GpuWorld(scene, 32)
    o.integrate()
    g.integrate()
    compare_state(g.state(), o.state(), what="integrate")
    o.broadphase()
    g.broadphase()
    po, pgpu = o.pairs(), g.pairs()
    assert len(po) > 50000
    so = np.sort(np.sort(po, axis=1).view([("a", np.int32), ("b", np.int32)]).ravel(), order=["a", "b"])
    sg = np.sort(np.sort(pgpu, axis=1).view([("a", np.int32), ("b", np.int32)]).ravel(), order=["a", "b"])
    np.testing.assert_array_equal(so, sg)
    assert o.axis == g.axis
    o.narrowphase()
    g.set_pairs(po)
    g.narrowphase()
    ro = o.results()
    assert ro["point_size"].sum() > 30000
    compare_results(g.results(), ro, what="stress narrowphase")
    o.solve()
    g.solve(pg.SERIAL_ORDER)
    so_, sg_ = o.state(), g.state()
    np.testing.assert_array_equal(sg_["lin_vel"], so_["lin_vel"])
    np.testing.assert_array_equal(sg_["ang_vel"], so_["ang_vel"])


@pytest.mark.parametrize("bits,n_scenes", [(32, 256), (64, 48)])
def test_gpu_settled_piles_narrowphase_matches_oracle(bits, n_scenes):
    """Piles of boxes, spheres, cylinders and convex hulls (8..64 vertices) after 90 coloured GPU
    steps, in contact and settling: from the same state and contact cache, the narrowphase on the
    oracle's pairs gives the oracle's results exactly.  The SAT skips axes whose overlap depth is
    bounded above a depth it has already computed, so this covers its pruned searches of box-hull,
    hull-box and hull-hull pairs, one warp per pair and one block per heavy pair."""
    scene, _ = sc.batched_piles(n_scenes=n_scenes, seed=3, real_bits=bits)
    g = pg.GpuWorld(scene, bits)
    g.step(90, pg.COLORED)
    st, res = g.state(), g.results()
    o = orc.OracleWorld(scene, bits, threads=8)
    o.set_state(st)
    o.set_results(res)
    o.axis = g.axis
    o.broadphase()
    g.broadphase()
    po = o.pairs()
    assert sorted(map(tuple, np.sort(po, axis=1))) == sorted(map(tuple, np.sort(g.pairs(), axis=1)))
    g.set_pairs(po)
    o.narrowphase()
    g.narrowphase()
    ro = o.results()
    assert ro["point_size"].sum() > 2000 * n_scenes // 64
    compare_results(g.results(), ro, what=f"settled piles narrowphase f{bits}")


def test_gpu_state_into_caller_buffers():
    """state(out=...) writes the requested fields into the caller's arrays (the end-to-end loop's
    page-locked buffers) with the same values as a fresh read, leaves the other fields alone, and
    refuses arrays of the wrong shape before touching the device."""
    scene = sc.pile(200, seed=5, real_bits=32)
    g = pg.GpuWorld(scene, 32)
    g.step(20, pg.COLORED)
    ref = g.state()
    io = ("origin", "basis", "lin_vel", "ang_vel")
    out = {f: np.full_like(ref[f], np.nan) for f in io}
    got = g.state(fields=io, out=out)
    assert got is out
    for f in io:
        np.testing.assert_array_equal(out[f], ref[f])
    g.set_state(out)
    np.testing.assert_array_equal(g.state()["origin"], ref["origin"])
    with pytest.raises(ValueError):
        g.state(fields=("origin",), out={"origin": np.zeros((3, 3))})


def test_gpu_tower_serial_order_per_step_replay():
    """The 1,002-body tower in double precision: from identical state, one GPU step with the
    oracle's pair order (ties among the sort keys make the order a property of the host
    sort) gives the oracle's state after the step."""
    scene = sc.tower(real_bits=64)
    o = orc.OracleWorld(scene, 64)
    g = pg.GpuWorld(scene, 64)
    o.step(5)
    g.set_state(o.state())
    g.set_results(o.results())
    g.axis = o.axis
    for _ in range(3):
        g.integrate()
        o.integrate()
        compare_state(g.state(), o.state(), what="tower integrate")
        g.axis = o.axis
        g.broadphase()
        o.broadphase()
        assert sorted(map(tuple, np.sort(g.pairs(), axis=1))) == sorted(map(tuple, np.sort(o.pairs(), axis=1)))
        g.set_pairs(o.pairs())
        g.narrowphase()
        o.narrowphase()
        compare_results(g.results(), o.results(), what="tower narrowphase")
        g.solve(pg.SERIAL_ORDER)
        o.solve()
        compare_state(g.state(), o.state(), keys=["lin_vel", "ang_vel"], what="tower solve")


@pytest.mark.parametrize("name", traj_names())
def test_gpu_tower_whole_trajectory_matches_reference(name):
    """The plain single-scene configuration as stated: the 1,002-body tower hit by the sphere, FP64,
    20 iterations, contact margin 0.005, serial order, 300 whole steps on the device.  Sort keys tie
    all over the tower and the reference's std::sort orders tied keys its own way, so each step's
    pair order is replayed from the oracle (whose order is the reference's; the GPU's own pair set
    is checked against it).  Every step's body states equal the reference's bit for bit: per-step
    digests of all states, and the kept full states."""
    scene, bits, steps, digests, kept = load_traj(name)
    o = orc.OracleWorld(scene, bits, threads=8, margin=scene.margin)
    g = pg.GpuWorld(scene, bits, margin=scene.margin)
    for k in range(steps):
        g.axis = o.axis
        g.integrate()
        o.integrate()
        g.broadphase()
        o.broadphase()
        ref_pairs = o.pairs()
        got = g.pairs()
        assert sorted(map(tuple, np.sort(got, axis=1))) == sorted(map(tuple, np.sort(ref_pairs, axis=1))), f"step {k}: pair sets differ"
        g.set_pairs(ref_pairs)
        g.narrowphase()
        o.narrowphase()
        g.solve(pg.SERIAL_ORDER)
        o.solve()
        st = g.state(fields=("origin", "basis", "lin_vel", "ang_vel"))
        if k in kept:
            np.testing.assert_array_equal(state_rows(st), kept[k], err_msg=f"{name} step {k}")
        assert np.array_equal(state_digest(st), digests[k]), f"{name}: body states differ from the reference at step {k}"


def test_gpu_batched_scenes_equal_scenes_alone():
    """Independent scenes stepped in one batch give, per scene, exactly what each scene gives
    alone (serial-order and coloured modes)."""
    parts = [sc.pile(n, seed=s, real_bits=32, hull_range=(8, 16), drop=(0.0, 0.5)) for n, s in ((20, 1), (35, 2), (9, 3))]
    merged, offs = sc.concat(parts)
    for mode in (pg.SERIAL_ORDER, pg.COLORED):
        g = pg.GpuWorld(merged, 32, scenes=offs)
        g.step(40, mode)
        big = g.state()
        for i, p in enumerate(parts):
            a = pg.GpuWorld(p, 32)
            a.step(40, mode)
            alone = a.state()
            sl = slice(offs[i], offs[i + 1])
            for k in ("origin", "basis", "lin_vel", "ang_vel"):
                np.testing.assert_array_equal(big[k][sl], alone[k], err_msg=f"scene {i} {k} mode {mode}")


def test_gpu_batched_piles_equal_scenes_alone():
    """The batched-pile workload generator (shared hull pool, uneven scene sizes): a batch of 48
    scenes stepped together equals, per scene, the scene extracted and stepped alone."""
    merged, offs = sc.batched_piles(n_scenes=48, seed=7, size_range=(8, 96), hull_pool=16, real_bits=32)
    picks = (0, 5, 17, 47)
    for mode in (pg.SERIAL_ORDER, pg.COLORED):
        g = pg.GpuWorld(merged, 32, scenes=offs)
        g.step(30, mode)
        big = g.state()
        for k in picks:
            a = pg.GpuWorld(sc.extract(merged, offs, k), 32)
            a.step(30, mode)
            alone = a.state()
            sl = slice(offs[k], offs[k + 1])
            for f in ("origin", "basis", "lin_vel", "ang_vel"):
                np.testing.assert_array_equal(big[f][sl], alone[f], err_msg=f"scene {k} {f} mode {mode}")


def test_gpu_colored_tower_stays_physical():
    """Coloured Gauss-Seidel on the tower hit by the sphere: contacts stay resolved (max
    penetration bounded like the serial solver's) and nothing gains energy from nowhere."""
    scene = sc.tower(real_bits=32)
    g = pg.GpuWorld(scene, 32)
    g.step(60, pg.COLORED)
    st = g.state()
    boxes = slice(1, 1001)
    assert np.all(np.isfinite(st["origin"]))
    # resting boxes below the impact height keep their layer height (no sinking, no jumping)
    y = st["origin"][boxes, 1]
    assert y.min() > 0.45
    assert np.abs(st["lin_vel"][boxes]).max() < 40.0
    r = g.results()
    depth = [r["slots"][i, :n, 12].min() for i, n in enumerate(r["point_size"]) if n]
    assert min(depth) > -0.05


def test_gpu_state_single_precision_transfers():
    """The float32 entry points (pe_gpu_get_state_f32 / pe_gpu_set_state_f32, the reference's default
    pe::Real) carry an FP32 world's state exactly: a float32 read equals the float64 read, and
    writing it back through the float32 path and stepping gives the same bits as the float64 path."""
    scene = sc.pile(200, seed=6, real_bits=32)
    a = pg.GpuWorld(scene, 32)
    b = pg.GpuWorld(scene, 32)
    for w in (a, b):
        w.step(15, pg.COLORED)
    io = ("origin", "basis", "lin_vel", "ang_vel")
    s64 = a.state(fields=io)
    s32 = a.state(fields=io, dtype=np.float32)
    for f in io:
        assert s32[f].dtype == np.float32
        np.testing.assert_array_equal(s32[f].astype(np.float64), s64[f])
    a.set_state(s32)
    b.set_state(s64)
    for w in (a, b):
        w.step(10, pg.COLORED)
    ra, rb = a.state(fields=io), b.state(fields=io)
    for f in io:
        np.testing.assert_array_equal(ra[f], rb[f])
    with pytest.raises(ValueError):
        a.state(fields=("origin",), dtype=np.int32)
