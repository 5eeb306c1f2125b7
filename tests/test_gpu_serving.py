"""Serving (pe_gpu_server_*): requests that arrive while others run are admitted into the same
batched world, and each request's final state equals its scene stepped alone for the same number
of steps (bit for bit: live scenes keep their state, sweep axes and contact pools across the
repacking the loop does as requests come and go).  Admission follows the HBM budget."""
import numpy as np
import pytest

import pe_gb300 as pg
from pe_gb300 import scene as sc

pytestmark = pytest.mark.gpu


def _scenes(n, seed, size_range):
    merged, offs = sc.batched_piles(n_scenes=n, seed=seed, size_range=size_range, hull_pool=12, real_bits=32)
    return [sc.extract(merged, offs, k) for k in range(n)]


def _alone(scene, k, mode):
    g = pg.GpuWorld(scene, 32)
    g.step(k, mode)
    return g.state(fields=("origin", "basis", "lin_vel", "ang_vel"))


@pytest.mark.parametrize("mode", [pg.COLORED, pg.SERIAL_ORDER])
def test_serving_results_equal_scenes_alone(mode):
    scenes = _scenes(7, seed=21, size_range=(16, 120))
    steps = [40, 25, 60, 30, 20, 35, 15]
    srv = pg.Server(real_bits=32, mode=mode)
    ids = {}
    schedule = {0: [0, 1, 2], 10: [3, 4], 22: [5], 23: [6]}   # arrivals by loop iteration
    done = {}
    it = 0
    while len(done) < len(scenes):
        for k in schedule.get(it, []):
            ids[k] = srv.submit(scenes[k], steps[k])
        srv.step()
        for k, rid in list(ids.items()):
            if k in done:
                continue
            st, res = srv.result(rid)
            if st == pg.DONE:
                done[k] = res
        it += 1
        assert it < 200
    for k, scene in enumerate(scenes):
        alone = _alone(scene, steps[k], mode)
        for f in ("origin", "basis", "lin_vel", "ang_vel"):
            np.testing.assert_array_equal(done[k][f], alone[f], err_msg=f"request {k} {f}")
    st = srv.stats()
    assert st["finished"] == len(scenes) and st["live"] == 0 and st["queued"] == 0
    assert st["p99_step_ms"] >= st["p50_step_ms"] > 0


def _footprint(s, r=4):
    """The server's charge for a scene (float world): per-body state and room for pairs and rows,
    hull vertices and shapes."""
    per_body = 55 * r + 64 + 6 * (40 + 8 * 20 * r) + 6 * 23 * r
    return s.n_bodies * per_body + 3 * len(s.hull_verts) * r * 4 + s.n_shapes * 32.0


def test_serving_admission_by_budget():
    scenes = _scenes(3, seed=5, size_range=(60, 80))
    fp = [_footprint(s) for s in scenes]
    budget = 1.01 * max(fp)             # holds any one of these scenes, never two
    assert min(fp[i] + fp[j] for i in range(3) for j in range(3) if i != j) > budget
    srv = pg.Server(real_bits=32, hbm_budget_bytes=budget)
    ids = [srv.submit(s, 5) for s in scenes]
    live, queued = srv.step()
    assert (live, queued) == (1, 2)
    order = []
    for _ in range(40):
        srv.step()
        for k, rid in enumerate(ids):
            if k not in order and rid in srv.n_bodies:
                st, _ = srv.result(rid)
                if st == pg.DONE:
                    order.append(k)
    assert order == [0, 1, 2]   # admitted and finished in arrival order, one at a time
    assert srv.stats()["peak_footprint_bytes"] <= budget
    small = pg.Server(real_bits=32, hbm_budget_bytes=1e5)
    rid = small.submit(scenes[0], 5)
    assert small.result(rid)[0] == pg.REJECTED


def test_serving_rejects_requests_without_steps():
    scene = _scenes(1, seed=8, size_range=(20, 30))[0]
    srv = pg.Server(real_bits=32)
    for k in (0, -3):
        with pytest.raises(pg.PeGpuError):
            srv.submit(scene, k)
    live, queued = srv.step()
    assert (live, queued) == (0, 0)
    rid = srv.submit(scene, 1)
    srv.step()
    srv.step()
    assert srv.result(rid)[0] == pg.DONE
