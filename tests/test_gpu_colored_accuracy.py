"""Accuracy of the coloured Gauss-Seidel solver (GPU, FP32) against the oracle's serial-order runs
(the reference's sequential impulse order) in FP64 and FP32, on a pour: 4,096 bodies (boxes,
spheres, convex hulls) dropped into a 10 x 10 m walled container from random, partly overlapping
positions, 240 steps of 1/120 s.  Colouring changes the Gauss-Seidel order, so trajectories differ
body by body; the gates are on aggregate physics:

* total mechanical energy, sampled every 20 steps, stays within max(3 x the largest FP32-vs-FP64
  oracle spread, 0.5 %) of the FP64 oracle, relative to the initial energy;
* the largest penetration seen stays within 1.25 x the larger of the two oracle runs' largest;
* the contact rows' velocity residual after the next solve (RMS over the points of how far the
  normal relative velocity falls short of the row's target) stays within 1.25 x the larger of the
  two oracle runs' (measured: 0.444 m/s against 0.455 / 0.433 m/s).
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


def test_gpu_colored_energy_and_penetration_within_oracle_spread():
    s64, s32 = _pour(64), _pour(32)
    o64, o32 = orc.OracleWorld(s64, 64, threads=16), orc.OracleWorld(s32, 32, threads=16)
    e64, p64 = _trace(o64, s64, lambda: o64.step(1))
    e32, p32 = _trace(o32, s32, lambda: o32.step(1))
    g = pg.GpuWorld(s32, 32)
    eg, pgpu = _trace(g, s32, lambda: g.step(1, pg.COLORED))
    dyn = s64.mass > 0
    e0 = float((s64.mass[dyn] * 9.8 * s64.origin[dyn, 1]).sum())
    spread = float(np.max(np.abs(e32 - e64))) / e0
    dev = float(np.max(np.abs(eg - e64))) / e0
    tol = max(3.0 * spread, 0.005)
    assert dev <= tol, f"energy deviation {dev:.4%} of E0 > tolerance {tol:.4%} (oracle FP32/FP64 spread {spread:.4%})"
    assert pgpu <= 1.25 * max(p64, p32), f"max penetration {pgpu:.4f} m vs oracle {p64:.4f} / {p32:.4f} m"
    assert np.all(np.isfinite(eg))
    # the next step by phases, with the body state read before and after the solve
    r = {}
    for name, w, scene, solve in (("o64", o64, s64, lambda: o64.solve()), ("o32", o32, s32, lambda: o32.solve()),
                                  ("gpu", g, s32, lambda: g.solve(pg.COLORED))):
        w.integrate()
        w.broadphase()
        w.narrowphase()
        pre, res = w.state(), w.results()
        solve()
        r[name] = contact_residual(pre, w.state(), res, scene)[0]
    assert r["gpu"] <= 1.25 * max(r["o64"], r["o32"]), f"contact residual {r['gpu']:.4f} m/s vs oracle {r['o64']:.4f} / {r['o32']:.4f} m/s"
