"""Accuracy of the coloured Gauss-Seidel solver (GPU, FP32) against the oracle, the reference's
sequential-impulse solver in its own order.

Pour: 4,096 bodies (boxes, spheres, convex hulls) dropped into a 10 x 10 m walled container from
random, partly overlapping positions, 240 steps of 1/120 s.  The tolerance is the spread of the
oracle's own runs of the scene: the FP64 build and the FP32 build, each at two thread counts, and
each with both orders the reference's broadphase may give equal sort keys (its std::sort leaves
that order unspecified; the oracle takes std::sort's or body order).  Thread counts change no bit
(asserted).  For each metric m, spread = max over the runs of |m(run) - m(FP64)|, and the coloured
GPU run must satisfy |m(GPU) - m(FP64)| <= spread, with no extra factor or floor:

* energy: total mechanical energy sampled every 20 steps, the largest deviation from the FP64 run
  over the samples, relative to the initial energy;
* the largest penetration seen over the samples;
* the contact rows' velocity residual after the next solve (RMS over the points of how far the
  normal relative velocity falls short of the row's target).

Batched piles (the benchmark's workload): there the coloured solver's islands keep the exact level
schedule, so a coloured step equals a serial-order step bit for bit.
"""
import numpy as np
import pytest

import orc
import pe_gb300 as pg
from pe_gb300 import scene as sc
from pe_testlib import contact_residual, max_penetration, mechanical_energy

pytestmark = pytest.mark.gpu

STEPS, EVERY = 240, 20


def _pour(real_bits):
    return sc.container_pour(n=4096, seed=3, floor=(10.0, 10.0), spawn_height=(1.0, 21.0), wall_height=25.0, hull_pool=32,
                             real_bits=real_bits)


def _trace(world, scene, step):
    energy, pen = [], []
    for k in range(STEPS):
        step()
        if (k + 1) % EVERY == 0:
            energy.append(mechanical_energy(world.state(), scene))
            pen.append(max_penetration(world.results()))
    return np.array(energy), max(pen)


def _residual(w, scene, solve):
    """The next step by phases, with the body state read before and after the solve."""
    w.integrate()
    w.broadphase()
    w.narrowphase()
    pre, res = w.state(), w.results()
    solve()
    return contact_residual(pre, w.state(), res, scene)[0]


def test_gpu_colored_within_oracle_spread():
    s64, s32 = _pour(64), _pour(32)
    runs = {}
    for bits, scene in ((64, s64), (32, s32)):
        for stable in (False, True):
            for threads in (4, 16):
                o = orc.OracleWorld(scene, bits, threads=threads, stable_ties=stable)
                e, p = _trace(o, scene, lambda: o.step(1))
                r = _residual(o, scene, lambda: o.solve())
                runs[(bits, stable, threads)] = (e, p, r)
    for bits in (64, 32):
        for stable in (False, True):
            a, b = runs[(bits, stable, 4)], runs[(bits, stable, 16)]
            assert np.array_equal(a[0], b[0]) and a[1] == b[1] and a[2] == b[2], "the thread count changed the oracle's result"
    g = pg.GpuWorld(s32, 32)
    eg, pgpu = _trace(g, s32, lambda: g.step(1, pg.COLORED))
    rg = _residual(g, s32, lambda: g.solve(pg.COLORED))
    assert np.all(np.isfinite(eg))
    dyn = s64.mass > 0
    e0 = float((s64.mass[dyn] * 9.8 * s64.origin[dyn, 1]).sum())
    e64, p64, r64 = runs[(64, False, 16)]
    members = [v for k, v in runs.items() if k[2] == 16]
    spread_e = max(float(np.max(np.abs(e - e64))) / e0 for e, _, _ in members)
    spread_p = max(abs(p - p64) for _, p, _ in members)
    spread_r = max(abs(r - r64) for _, _, r in members)
    dev_e = float(np.max(np.abs(eg - e64))) / e0
    assert dev_e <= spread_e, f"energy deviation {dev_e:.4%} of E0 > oracle spread {spread_e:.4%}"
    assert abs(pgpu - p64) <= spread_p, f"max penetration {pgpu:.4f} m vs FP64 {p64:.4f} m, oracle spread {spread_p:.4f} m"
    assert abs(rg - r64) <= spread_r, f"contact residual {rg:.4f} m/s vs FP64 {r64:.4f} m/s, oracle spread {spread_r:.4f} m/s"


def test_gpu_colored_equals_serial_order_on_batched_piles():
    merged, offs = sc.batched_piles(n_scenes=96, seed=77, real_bits=32)
    a = pg.GpuWorld(merged, 32, scenes=offs)
    b = pg.GpuWorld(merged, 32, scenes=offs)
    for k in range(90):
        a.step(1, pg.COLORED)
        b.step(1, pg.SERIAL_ORDER)
        assert a.last_counts()["colors"] < 511   # no island left items after the block path's rounds
        if (k + 1) % 30 == 0:
            sa, sb = a.state(), b.state()
            for f in ("origin", "basis", "lin_vel", "ang_vel"):
                np.testing.assert_array_equal(sa[f], sb[f], err_msg=f"step {k}: {f}")
