"""Steps replayed from captured CUDA graphs (pe_gpu_set_step_graphs, the default) give the bits of
steps launched kernel by kernel: batched piles and a scattered mixed scene in both solver modes, a
run whose parameters and settings change midway (each change is a new capture), a run whose big
islands take the host-driven path after the graph, and the counters the step reports.  The phase
timers still split a graph step into its phases."""
import numpy as np
import pytest

import pe_gb300 as pg
from pe_gb300 import scene as sc

pytestmark = pytest.mark.gpu

FIELDS = ("origin", "basis", "lin_vel", "ang_vel")


def _pair(scene, offs, tuning=None):
    a = pg.GpuWorld(scene, 32, scenes=offs, tuning=tuning)
    b = pg.GpuWorld(scene, 32, scenes=offs, tuning=tuning)
    b.set_step_graphs(False)
    return a, b


def _same(a, b, what):
    sa, sb = a.state(fields=FIELDS), b.state(fields=FIELDS)
    for f in FIELDS:
        np.testing.assert_array_equal(sa[f], sb[f], err_msg=f"{what}: {f}")


@pytest.mark.parametrize("mode", [pg.SERIAL_ORDER, pg.COLORED])
def test_gpu_graph_steps_equal_direct_steps(mode):
    merged, offs = sc.batched_piles(n_scenes=64, seed=5, real_bits=32)
    for scene, o in ((merged, offs), (sc.random_cube(n=3000, seed=8, extent=14.0, real_bits=32), None)):
        a, b = _pair(scene, o)
        for k in range(60):
            a.step(1, mode)
            b.step(1, mode)
            ca, cb = a.last_counts(), b.last_counts()
            assert ca == cb, f"step {k}: counters {ca} vs {cb}"
            if (k + 1) % 20 == 0:
                _same(a, b, f"step {k}")
        a.close()
        b.close()


def test_gpu_graph_steps_follow_parameter_and_setting_changes():
    merged, offs = sc.batched_piles(n_scenes=32, seed=12, real_bits=32)
    a, b = _pair(merged, offs)
    for w in (a, b):
        w.step(20, pg.COLORED)
    for w in (a, b):
        w.set_params(dt=1 / 90, gravity=(0.0, -9.8, 0.0), iterations=6)
        w.step(15, pg.COLORED)
    _same(a, b, "after set_params")
    for w in (a, b):
        w.set_tuning(small_island_items=4, side_streams=2)
        w.step(15, pg.SERIAL_ORDER)
    _same(a, b, "after set_tuning")


def test_gpu_graph_steps_with_big_islands():
    # every island above 64 items takes the grid-wide path, solved after the graph's counters are read
    merged, offs = sc.batched_piles(n_scenes=24, seed=3, real_bits=32)
    a, b = _pair(merged, offs, tuning=dict(big_island_items=64))
    for mode in (pg.SERIAL_ORDER, pg.COLORED):
        for w in (a, b):
            w.step(25, mode)
        _same(a, b, f"mode {mode}")


def test_gpu_graph_step_phase_times():
    merged, offs = sc.batched_piles(n_scenes=64, seed=6, real_bits=32)
    g = pg.GpuWorld(merged, 32, scenes=offs)
    g.step(10, pg.COLORED)
    g.phase_times(reset=True)
    g.step(10, pg.COLORED)
    ms = g.phase_times()
    assert all(m > 0 for m in ms.values()), ms
    parts = ms["integrate"] + ms["broadphase"] + ms["narrowphase"] + ms["solver"]
    assert parts <= ms["step"] * 1.01 + 1e-3, ms
