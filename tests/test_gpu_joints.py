"""GPU joints (ball / hinge / slider constraints of the sequential-impulse solver) and ignored
collision pairs, through the C ABI: bit-exact against the oracle in serial-order mode, and
physical gates (joint anchors held together) in coloured mode, including an island above the
block-coloured size that the grid-wide colouring path solves."""
import numpy as np
import pytest

import orc
import pe_gb300 as pg
from pe_gb300 import scene as sc
from pe_testlib import compare_results, compare_state

pytestmark = pytest.mark.gpu


def anchor_error(scene, st):
    """Largest distance between the two world anchors of any ball or hinge joint (a slider lets
    its anchors part along the axis)."""
    o, b = st["origin"], st["basis"]
    keep = scene.joint_type != sc.JOINT_SLIDER
    ja, jb = scene.joint_body[keep, 0], scene.joint_body[keep, 1]
    pa = o[ja] + np.einsum("nij,nj->ni", b[ja], scene.joint_real[keep, 0:3])
    pb = o[jb] + np.einsum("nij,nj->ni", b[jb], scene.joint_real[keep, 3:6])
    return float(np.linalg.norm(pa - pb, axis=1).max())


def test_gpu_joint_chains_match_oracle_f64():
    """100 chains of 10 links (ball joints, free and motor-driven hinges, sliders) falling onto a
    ground, FP64: 90 whole serial-order steps equal the oracle's (state, pairs and contacts every
    10 steps)."""
    scene = sc.chain_field(n_chains=100, links=10, seed=4, hinge_limits=False, real_bits=64)
    o = orc.OracleWorld(scene, 64, threads=8)
    g = pg.GpuWorld(scene, 64)
    for k in range(9):
        o.step(10)
        g.step(10, pg.SERIAL_ORDER)
        st = g.state()
        compare_state(st, o.state(), what=f"chains step {10 * k + 9}")
        np.testing.assert_array_equal(g.pairs(), o.pairs())
        compare_results(g.results(), o.results(), what=f"chains step {10 * k + 9}")
    assert anchor_error(scene, st) < 0.1   # the oracle's own run holds the anchors within 6.2 cm here


def test_gpu_joint_chains_f32_per_step():
    """The same field in FP32, one step at a time with the oracle's pair order (two steps have
    tied sort keys): integration, pair sets, contacts and solved velocities bit for bit."""
    scene = sc.chain_field(n_chains=100, links=10, seed=4, hinge_limits=False, real_bits=32)
    o = orc.OracleWorld(scene, 32, threads=8)
    g = pg.GpuWorld(scene, 32)
    for k in range(60):
        o.integrate()
        g.integrate()
        compare_state(g.state(), o.state(), what=f"integrate {k}")
        o.broadphase()
        g.broadphase()
        po, pgpu = o.pairs(), g.pairs()
        assert sorted(map(tuple, np.sort(po, axis=1))) == sorted(map(tuple, np.sort(pgpu, axis=1))), f"pairs {k}"
        g.set_pairs(po)
        o.narrowphase()
        g.narrowphase()
        compare_results(g.results(), o.results(), what=f"narrowphase {k}")
        o.solve()
        g.solve(pg.SERIAL_ORDER)
        so, sg = o.state(), g.state()
        np.testing.assert_array_equal(sg["lin_vel"], so["lin_vel"], err_msg=f"solve {k}")
        np.testing.assert_array_equal(sg["ang_vel"], so["ang_vel"], err_msg=f"solve {k}")


@pytest.mark.parametrize("bits", [32, 64])
def test_gpu_limited_hinges_per_step(bits):
    """With hinge angle limits active (half of the chains), each serial-order step taken from the
    oracle's state matches the oracle's next state within 1e-6 (FP64) / 5e-6 (FP32): the limit
    angle is an atan2, where CUDA's and the C library's last place may differ, so equality is not
    required here."""
    scene = sc.chain_field(n_chains=100, links=10, seed=4, real_bits=bits)
    o = orc.OracleWorld(scene, bits, threads=8)
    g = pg.GpuWorld(scene, bits)
    for k in range(60):
        g.set_state(o.state())
        g.set_results(o.results())
        g.axis = o.axis
        o.step(1)
        g.step(1, pg.SERIAL_ORDER)
        so, sg = o.state(), g.state()
        for f in ("origin", "lin_vel", "ang_vel"):
            err = float(np.abs(sg[f] - so[f]).max())
            assert err <= (1e-6 if bits == 64 else 5e-6), (k, f, err)


def test_gpu_ignored_pairs_match_oracle():
    """Ignored collision pairs leave exactly those pairs out of the broadphase: a mixed scene with
    a few hundred ignored pairs among overlapping bodies gives the oracle's pair list."""
    scene = sc.random_cube(n=4096, seed=31, extent=22.0, real_bits=32)
    rng = np.random.default_rng(5)
    o = orc.OracleWorld(scene, 32)
    o.integrate()
    o.broadphase()
    full = o.pairs()
    pick = full[rng.choice(len(full), size=min(400, len(full) // 4), replace=False)]
    scene.ignore_pairs = np.concatenate([pick[::2], pick[1::2, ::-1]]).astype(np.int32)
    o = orc.OracleWorld(scene, 32)
    g = pg.GpuWorld(scene, 32)
    for w in (o, g):
        w.integrate()
        w.broadphase()
    po, pgpu = o.pairs(), g.pairs()
    assert sorted(map(tuple, np.sort(po, axis=1))) == sorted(map(tuple, np.sort(pgpu, axis=1)))
    assert len(po) == len(full) - len(pick)
    kept = set(map(tuple, np.sort(pgpu, axis=1)))
    assert not kept & set(map(tuple, np.sort(pick, axis=1)))


def test_gpu_colored_joints_hold():
    """Coloured mode orders the rows differently but must hold the joints about as well as the
    reference order does (9.5 cm largest anchor separation after 120 steps in the oracle's run):
    at most twice the serial-order run's separation plus 2 cm, and nothing diverges."""
    scene = sc.chain_field(n_chains=100, links=10, seed=4, real_bits=32)
    errs = {}
    for mode in (pg.SERIAL_ORDER, pg.COLORED):
        g = pg.GpuWorld(scene, 32)
        g.step(120, mode)
        st = g.state()
        assert np.isfinite(st["origin"]).all()
        errs[mode] = anchor_error(scene, st)
    assert errs[pg.COLORED] < 2 * errs[pg.SERIAL_ORDER] + 0.02, errs


def test_gpu_colored_long_chain_big_island():
    """One chain of 5,000 links (ball, hinge and slider joints): an island of 5,000 joint items,
    above the block-coloured limit, so the grid-wide colouring path solves it.  After 30 steps
    the anchors stay within 5 cm (the oracle's serial run: 0.6 cm) and the chain has fallen as far
    as in the serial-order run."""
    scene = sc.chain_field(n_chains=1, links=5000, seed=2, height=3.0, real_bits=32)
    out = {}
    for mode in (pg.SERIAL_ORDER, pg.COLORED):
        g = pg.GpuWorld(scene, 32)
        g.step(30, mode)
        st = g.state()
        assert np.isfinite(st["origin"]).all()
        out[mode] = (anchor_error(scene, st), float(st["origin"][1:, 1].mean()))
    (es, ys), (ec, yc) = out[pg.SERIAL_ORDER], out[pg.COLORED]
    assert ec < 0.05 and ec < es + 0.02, out
    assert abs(yc - ys) < 0.05, out
