"""Scheduling settings (pe_gpu_tuning) change no result: the batched piles and a mixed scattered scene
stepped with the defaults, with settings that send every piece of work to another kernel (every SAT
pair to the block-of-warps kernel, every island above one item to the block or grid-wide path, the
radix sort instead of the per-scene sort, one narrowphase stream, the smallest blocks) and with the
autotuner's stored settings give the same bits, in serial-order and in coloured mode.  Invalid
settings are refused."""
import numpy as np
import pytest

import pe_gb300 as pg
from pe_gb300 import scene as sc

pytestmark = pytest.mark.gpu

OTHER = dict(sat_heavy_cost=1, small_island_items=1, big_island_items=64, color_block=32, level_block=64, scene_sort_max=0,
             side_streams=1)


def _run(scene, offs, mode, steps, tuning):
    g = pg.GpuWorld(scene, 32, scenes=offs, tuning=tuning)
    g.step(steps, mode)
    st = g.state(fields=("origin", "basis", "lin_vel", "ang_vel"))
    g.close()
    return st


@pytest.mark.parametrize("mode", [pg.SERIAL_ORDER, pg.COLORED])
def test_gpu_tuning_changes_no_bits(mode):
    merged, offs = sc.batched_piles(n_scenes=48, seed=91, real_bits=32)
    for scene, o in ((merged, offs), (sc.random_cube(n=3000, seed=4, extent=14.0, real_bits=32), None)):
        ref = _run(scene, o, mode, 40, None)
        for tuning in (OTHER, "auto"):
            got = _run(scene, o, mode, 40, tuning)
            for f in ref:
                np.testing.assert_array_equal(got[f], ref[f], err_msg=f"{tuning}: {f}")


def test_gpu_tuning_refuses_invalid_settings():
    g = pg.GpuWorld(sc.pair_zoo(0, 0, m=2, real_bits=32), 32)
    default = g.tuning()
    for bad in (dict(color_block=48), dict(level_block=512), dict(side_streams=0), dict(scene_sort_max=4096),
                dict(small_island_items=64, big_island_items=64)):
        with pytest.raises(pg.PeGpuError):
            g.set_tuning(**bad)
        assert g.tuning() == default
    g.set_tuning(color_block=128)
    assert g.tuning()["color_block"] == 128
