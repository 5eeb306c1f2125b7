"""The contact-row velocity residual used as an accuracy gate of the coloured solver
(pe_testlib.contact_residual), pinned on the oracle: a box landing on a kinematic ground at 1 m/s
with 0.01 m of penetration leaves a shortfall against its rows' targets that Gauss-Seidel
iterations remove, so the residual falls with the iteration count and vanishes once converged."""
import numpy as np

import orc
from pe_gb300 import scene as sc
from pe_testlib import contact_residual


def _landing_box(iterations):
    sb = sc.SceneBuilder(dt=1.0 / 60.0, iterations=iterations)
    ground = sb.shape(sc.BOX, (10.0, 1.0, 10.0))
    sb.body(ground, (0.0, -0.5, 0.0), mass=0.0, kinematic=True, restitution=0.0)
    box = sb.shape(sc.BOX, (1.0, 1.0, 1.0))
    sb.body(box, (0.0, 0.49, 0.0), mass=1.0, v=(0.0, -1.0, 0.0), restitution=0.0)
    return sb.build(64)


def test_residual_falls_with_iterations_and_vanishes_when_converged():
    rms = []
    for iterations in (1, 5, 50):
        scene = _landing_box(iterations)
        o = orc.OracleWorld(scene, 64)
        o.integrate()
        o.broadphase()
        o.narrowphase()
        pre, res = o.state(), o.results()
        assert int(res["point_size"].sum()) == 4
        o.solve()
        r, worst = contact_residual(pre, o.state(), res, scene)
        assert 0.0 <= r <= worst
        rms.append(r)
    assert rms[0] > 0.1 and rms[1] < rms[0] / 10 and rms[2] < 1e-9, rms


def test_residual_of_no_contacts_is_zero():
    scene = _landing_box(10)
    o = orc.OracleWorld(scene, 64)
    st = o.state()
    empty = dict(res_a=np.zeros(0, np.int32), res_b=np.zeros(0, np.int32), point_size=np.zeros(0, np.int32),
                 restitution=np.zeros(0), slots=np.zeros((0, 8, 19)))
    assert contact_residual(st, st, empty, scene) == (0.0, 0.0)
