"""Autotuner of the step's scheduling settings (pe_gpu_tuning in include/pe_gpu.h).

The settings decide which kernel takes which work and with how many threads: the estimated SAT work
from which a pair gets a block of warps, the island sizes that run on one thread or grid-wide, the
threads per island block, the largest scene sorted inside one block, the streams the narrowphase's
classes are spread over.  In serial-order mode no setting changes a result bit; in coloured mode
neither do these, as long as no island needs more levels than `exact_levels_colored` (a setting the
tuner leaves alone, because it trades the reference's order for fewer colours).  The reference's
counterpart is the fixed work split of its thread pool, batch = count / threads / 2 + 1
(src/utils/thread_pool.h:85-102).

tune() times the candidates of each setting in turn (coordinate descent, the others at their best
so far) on a reduced batched workload, every candidate over the same steps from the same saved
state, and keeps the fastest; save_table() stores the winners per GPU model and real type in
tuning/<gpu>.json beside this module, where GpuWorld(..., tuning="auto") finds them.

    python -m pe_gb300.autotune [--scenes 4096] [--steps 8] [--bits 32] [--mode colored]
"""
import argparse
import json
import re
import sys
from pathlib import Path

TABLE_DIR = Path(__file__).resolve().parent / "tuning"

# candidate values per setting, tried in this order (defaults included)
CANDIDATES = {
    "sat_heavy_cost": [50000, 100000, 200000, 400000, 1000000, 2000000, 4000000, 8000000, 16000000],
    "side_streams": [1, 2, 4],
    "small_island_items": [2, 4, 8, 16, 32],
    "color_block": [32, 64, 128, 256],
    "level_block": [64, 128, 256],
    "big_island_items": [1024, 4096, 16384],
    "scene_sort_max": [0, 2048],
}
NOISE = 0.005                     # run-to-run spread of the per-candidate timings (0.5 %)
SERIAL_ONLY = {"level_block"}     # used by the serial-order solver only
COLORED_ONLY = {"color_block"}    # used by the coloured solver only


def table_path(gpu_name):
    return TABLE_DIR / (re.sub(r"[^A-Za-z0-9]+", "_", gpu_name).strip("_") + ".json")


def load_table(gpu_name, real_bits):
    """The stored settings for this GPU model and real type ({} when none were tuned)."""
    p = table_path(gpu_name)
    if not p.exists():
        return {}
    d = json.loads(p.read_text())
    return dict(d.get(f"f{real_bits}", {}).get("settings", {}))


def save_table(gpu_name, real_bits, settings, detail, path=None):
    p = Path(path) if path else table_path(gpu_name)
    p.parent.mkdir(parents=True, exist_ok=True)
    d = json.loads(p.read_text()) if p.exists() else {}
    d["gpu"] = gpu_name
    d[f"f{real_bits}"] = {"settings": settings, **detail}
    p.write_text(json.dumps(d, indent=1, sort_keys=True) + "\n")
    return p


def _time_steps(g, snapshot, steps, mode, repeats):
    """Device time of `steps` steps from the snapshot, the best of `repeats` runs (ms per step)."""
    best = None
    for _ in range(repeats):
        g.set_state(snapshot[0])
        g.set_results(snapshot[1])
        g.set_axes(snapshot[2])
        g.step(1, mode)   # first step after a restore: buffers settle, not timed
        t0 = g.phase_times()["step"]
        g.step(steps, mode)
        t = (g.phase_times()["step"] - t0) / steps
        best = t if best is None else min(best, t)
    return best


def tune(device=0, real_bits=32, mode=None, scenes=4096, steps=8, preroll=120, repeats=3, seed=4096, log=print):
    """Coordinate descent over CANDIDATES on `scenes` piles of the batched workload; returns
    (settings, detail) with the winners and every timing."""
    import pe_gb300 as pg
    from pe_gb300 import scene as sc
    mode = pg.COLORED if mode is None else mode
    merged, offs = sc.batched_piles(n_scenes=scenes, seed=seed, real_bits=real_bits)
    g = pg.GpuWorld(merged, real_bits, device=device, scenes=offs)
    g.step(preroll, mode)
    snapshot = (g.state(), g.results(), g.axes(len(offs) - 1))
    best = g.tuning()
    timings = {}
    base = _time_steps(g, snapshot, steps, mode, repeats)
    log(f"defaults: {base:.3f} ms/step")
    for name, values in CANDIDATES.items():
        if (name in SERIAL_ONLY and mode != pg.SERIAL_ORDER) or (name in COLORED_ONLY and mode != pg.COLORED):
            continue
        res = {}
        for v in values:
            try:
                g.set_tuning(**dict(best, **{name: v}))
            except pg.PeGpuError:
                continue   # not a valid combination with the settings chosen so far
            res[v] = _time_steps(g, snapshot, steps, mode, repeats)
        # the current value stays unless a candidate beats it by more than the timing noise
        cur = best[name]
        pick = min(res, key=res.get)
        if cur in res and res[pick] > res[cur] * (1.0 - NOISE):
            pick = cur
        best[name] = pick
        g.set_tuning(**best)
        timings[name] = {str(k): round(t, 4) for k, t in res.items()}
        log(f"{name}: {pick} ({', '.join(f'{k}: {t:.3f}' for k, t in res.items())})")
    final = _time_steps(g, snapshot, steps, mode, repeats)
    log(f"tuned: {final:.3f} ms/step (defaults {base:.3f})")
    g.close()
    detail = {"workload": f"{scenes} piles of the batched workload (seed {seed}), {preroll} steps of pre-roll, "
                          f"best of {repeats} x {steps} steps per candidate",
              "mode": "coloured" if mode == pg.COLORED else "serial-order",
              "ms_per_step_default": round(base, 4), "ms_per_step_tuned": round(final, 4), "timings": timings}
    return best, detail


def main(argv=None):
    import pe_gb300 as pg
    ap = argparse.ArgumentParser()
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--bits", type=int, default=32, choices=(32, 64))
    ap.add_argument("--mode", default="colored", choices=("colored", "serial"))
    ap.add_argument("--scenes", type=int, default=4096)
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--out", default=None, help="write the table here instead of beside the module")
    a = ap.parse_args(argv)
    mode = pg.COLORED if a.mode == "colored" else pg.SERIAL_ORDER
    settings, detail = tune(a.device, a.bits, mode, a.scenes, a.steps)
    print(save_table(pg.device_name(a.device), a.bits, settings, detail, a.out))
    return 0


if __name__ == "__main__":
    sys.exit(main())
