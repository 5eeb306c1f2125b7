"""Benchmark of the rigid-body step on the GPU (and of the reference's CPU step).

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload batched|stress|tower]

Workloads (all synthetic, seeded):
  batched  4,096 independent piles of 8..512 bodies (log-uniform; box/sphere/cylinder/convex hull
           50/20/10/20, hulls of 8..64 vertices on a sphere scaled U[0.3, 1.0]) dropped 0..5 m onto
           their own static ground boxes; FP32; dt 1/60; 10 iterations; coloured Gauss-Seidel; one
           batched step for all scenes; timed after 120 untimed steps (piles in contact).  Beside
           it, a sample of the same scenes stepped one world at a time (the per-scene GPU path).
           Default.
  stress   65,536 bodies (60% boxes, 25% spheres, 15% cylinders, sizes as in the one-step stress
           configuration) scattered in a 100 m cube with N(0,2) m/s velocities; FP32; dt 1/60;
           10 solver iterations; coloured Gauss-Seidel.
  tower    1,000 boxes stacked 10x10x10 with 1 mm gaps on a static ground box, hit by a 50 kg
           sphere at 30 m/s; FP64; dt 1/60; 20 iterations; serial-order solver.
  large    262,144 bodies (box/sphere/convex hull 50/30/20, sizes U[0.1, 0.5] m) poured from a
           40x40x80 m volume into a 40x40 m walled container; FP32; dt 1/120; 10 iterations;
           coloured; timed after 240 untimed steps.

One "step" is one full World::step (integrate, broadphase, narrowphase, solver) of the whole
workload.  `value` = body-steps per second of device time with the state resident in HBM
(CUDA events on the library's stream, L2 flushed between steps); `e2e` = the same metric
through the C ABI with host buffers over the same steps (replayed from a snapshot of the state,
contact results and sweep axes taken before the timed region): every step uploads body poses and
velocities (in the world's real type) from page-locked host arrays and reads the stepped ones back
into them.  `--impl reference` times the reference's CPU step (its
algorithm restated in oracle/, multithreaded over the host cores like the reference's thread
pool) on the same workload.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "physics-engine_gb300"))

METRIC = "body-steps/s batched vs per-scene GPU step at oracle tol; p50/p99 step latency"
UNIT = "body-steps/s"


def make_workload(name, n_scenes=4096):
    from pe_gb300 import scene as sc
    if name == "stress":
        s = sc.random_cube(n=65536, seed=2024, real_bits=32)
        return s, 32, 1, None, dict(workload="65,536 mixed bodies (box/sphere/cylinder 60/25/15) in a 100 m cube, "
                                             "full step, FP32, 10 SI iterations, coloured Gauss-Seidel",
                                    bodies=65536, scenes=1, solver="coloured")
    if name == "tower":
        s = sc.tower(real_bits=64)
        return s, 64, 0, None, dict(workload="1,000-box 10x10x10 tower + ground + sphere at 30 m/s, full step, FP64, "
                                             "20 SI iterations, contact margin 0.005, serial-order solver",
                                    bodies=s.n_bodies, scenes=1, solver="serial-order", margin=0.005)
    if name == "tower_colored":
        s = sc.tower(real_bits=32)
        return s, 32, 1, None, dict(workload="the same tower (1,000 boxes, ground, sphere at 30 m/s), FP32, 20 SI iterations, "
                                             "contact margin 0.005, coloured Gauss-Seidel",
                                    bodies=s.n_bodies, scenes=1, solver="coloured", margin=0.005)
    if name == "batched":
        s, offs = sc.batched_piles(n_scenes=n_scenes, seed=4096, real_bits=32)
        return s, 32, 1, offs, dict(workload=f"{n_scenes:,} independent piles of 8..512 bodies (log-uniform; box/sphere/cylinder/"
                                             "convex hull 50/20/10/20, hulls of 8..64 vertices from a 512-shape pool) "
                                             "on static ground boxes, one batched step, FP32, 10 SI iterations, coloured",
                                    bodies=s.n_bodies, scenes=n_scenes, solver="coloured", preroll_steps=120)
    if name == "large":
        s = sc.container_pour(n=262144, seed=5, real_bits=32)
        return s, 32, 1, None, dict(workload="262,144 bodies (box/sphere/convex hull 50/30/20, sizes U[0.1,0.5] m, hulls of "
                                             "16..32 vertices from a 256-shape pool) poured from a 40x40x80 m volume into a "
                                             "40x40 m walled container, FP32, dt 1/120, 10 SI iterations, coloured",
                                    bodies=s.n_bodies, scenes=1, solver="coloured", preroll_steps=240)
    raise SystemExit(f"unknown workload {name}")


# ------------------------------------------------------------------ measurement helpers
class L2Flush:
    """Writes a buffer larger than L2 (129 MB) between timed steps."""

    def __init__(self, nbytes=256 << 20):
        self.rt = _cudart()
        self.p = ctypes.c_void_p()
        self.n = nbytes
        if self.rt.cudaMalloc(ctypes.byref(self.p), ctypes.c_size_t(nbytes)) != 0:
            raise RuntimeError("cudaMalloc for the L2 flush buffer failed")

    def __call__(self):
        self.rt.cudaMemset(self.p, 1, ctypes.c_size_t(self.n))
        self.rt.cudaDeviceSynchronize()


def _cudart():
    try:
        return ctypes.CDLL("libcudart.so")
    except OSError:
        return ctypes.CDLL("/usr/local/cuda/lib64/libcudart.so")


def _pci_bus_id(device):
    """PCI bus id of a CUDA device (so that NVML samples the GPU this process runs on)."""
    buf = ctypes.create_string_buffer(64)
    if _cudart().cudaDeviceGetPCIBusId(buf, 64, device) != 0:
        return b""
    return buf.value


class ClockSampler:
    """SM clocks and clock-event (throttle) reasons sampled while the timed region runs.

    Reads NVML directly (libnvidia-ml, read-only queries) every 10 ms from a thread, so that a
    timed region of a few tens of milliseconds still gets samples; falls back to
    `nvidia-smi -lms 200` when NVML cannot be loaded."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")
    # nvmlClocksEventReasons bits (nvml.h)
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown",
               0x80: "hw_power_brake_slowdown"}

    def __init__(self, device, period_s=0.01):
        self.device = device
        self.period = period_s
        self.proc = None
        self.nvml = None
        self.samples = []
        self.lines = []
        try:
            lib = ctypes.CDLL("libnvidia-ml.so.1")
            if lib.nvmlInit_v2() == 0:
                h = ctypes.c_void_p()
                if lib.nvmlDeviceGetHandleByPciBusId_v2(_pci_bus_id(device), ctypes.byref(h)) == 0 or \
                        lib.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(device), ctypes.byref(h)) == 0:
                    self.nvml, self.handle = lib, h
        except (OSError, AttributeError):
            self.nvml = None

    def _poll(self):
        lib, h = self.nvml, self.handle
        clk, mx, rs = ctypes.c_uint(), ctypes.c_uint(), ctypes.c_ulonglong()
        lib.nvmlDeviceGetMaxClockInfo(h, 1, ctypes.byref(mx))
        get_reasons = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            lib.nvmlDeviceGetCurrentClocksThrottleReasons
        while not self.stop.is_set():
            if lib.nvmlDeviceGetClockInfo(h, 1, ctypes.byref(clk)) == 0 and get_reasons(h, ctypes.byref(rs)) == 0:
                self.samples.append((clk.value, mx.value, rs.value))
            self.stop.wait(self.period)

    def __enter__(self):
        if self.nvml is not None:
            self.stop = threading.Event()
            self.thread = threading.Thread(target=self._poll, daemon=True)
            self.thread.start()
            return self
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.nvml is not None:
            self.stop.set()
            self.thread.join()
            return
        if self.proc:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, smax, reasons = [], [], set()
        if self.samples:
            for c, m, r in self.samples:
                sm.append(float(c))
                smax.append(float(m))
                reasons.update(n for bit, n in self.REASONS.items() if r & bit)
            src = "nvml, 10 ms"
        else:
            names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
            for l in self.lines:
                f = [x.strip() for x in l.split(",")]
                try:
                    sm.append(float(f[1]))
                    smax.append(float(f[2]))
                except (ValueError, IndexError):
                    continue
                for n, v in zip(names, f[5:9]):
                    if v.lower() == "active":
                        reasons.add(n)
            src = "nvidia-smi, 200 ms"
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm), "source": src}


def measured_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def hull_vertices_per_pair(scene, pairs):
    """Sum over the step's pairs of (V_A + V_B), the vertex counts of the pair's convex hulls (0 for
    boxes, spheres, cylinders): the hull term of the pair bytes."""
    from pe_gb300 import scene as sc
    st = np.asarray(scene.shape_type)
    vc = np.where(st == sc.HULL, np.asarray(scene.hull_vcnt), 0)
    per_body = vc[np.asarray(scene.body_shape)]
    p = np.asarray(pairs).reshape(-1, 2)
    return int(per_body[p[:, 0]].sum() + per_body[p[:, 1]].sum()) if len(p) else 0


def algorithmic_bytes(counts, n_bodies, iters, real_bytes, hull_verts=0):
    """Algorithmic HBM bytes of one step (per phase), from the per-unit figures:
    body 268 B, pair 104 B plus 12 B per hull vertex of the pair (hull_verts = sum of V_A + V_B over
    the pairs), manifold 8 B, contact point 184 B plus 200 B per point and solver iteration (FP32;
    FP64 doubles every real field)."""
    k = real_bytes / 4.0
    P, M, C = counts["pairs"], counts["active"], counts["rows"]
    return {
        "integrate": n_bodies * 124 * k,                                          # read state 72 + write pose 28 + AABB 24
        "broadphase": n_bodies * (8 + 64 + 24 * k) + P * 8,                       # sort records + sorted AABB gather + pairs
        "narrowphase": (P * 104 + 12 * hull_verts + C * 52) * k + M * 8,          # pairs, bodies, hull vertices; points
        "solver": (n_bodies * 48 + C * (52 + 80) + C * iters * 200) * k,          # v, w; setup; row 80 + acc 24 + bodies 96
        "step": (n_bodies * 268 + P * 104 + 12 * hull_verts + M * 8 + C * (184 + iters * 200)) * k,
    }


# The roofline is taken per phase: the narrowphase's class kernels run side by side on several
# streams, so a phase's duration (events on the world's stream around the phase) is the time its
# kernels take together; the phase with the longest duration is the dominant one.
PHASES = ("integrate", "broadphase", "narrowphase", "solver")


def ncu_traffic(phase):
    """DRAM bytes (read + write) per step of a phase's kernels from the committed ncu launch list
    of the batched workload (profiles/launches_batched_dram.md), scaled to the full workload by the
    bodies processed; None when the summary is absent."""
    f = ROOT / "profiles" / "launches_batched_dram.md"
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        m = line.strip().split("|")
        if len(m) > 4 and m[1].strip() == f"phase:{phase}":
            try:
                return float(m[4])   # bytes per step at the full workload
            except ValueError:
                return None
    return None


# ------------------------------------------------------------------ our arm
def run_ours(args, rank, world, device):
    import pe_gb300 as pg
    scene, bits, mode, offs, cfg = make_workload(args.workload, args.scenes)
    g = pg.GpuWorld(scene, bits, device=device, scenes=offs, margin=cfg.get("margin", 0.0), tuning="auto")
    cfg = dict(cfg, tuning=dict(g.tuning(), source="pe_gb300/tuning table for this GPU" if pg.autotune_table_present(device, bits)
                                else "defaults (no tuning table for this GPU)"))
    flush = L2Flush()
    N = scene.n_bodies
    for _ in range(cfg.get("preroll_steps", 0)):   # untimed settling (part of the workload definition)
        g.step(1, mode)
    for _ in range(args.warmup):
        g.step(1, mode)
    if args.profile_one_step:
        # one step between cudaProfilerStart and cudaProfilerStop (ncu --profile-from-start off
        # captures exactly its launches), then stop: nothing is timed
        rt = _cudart()
        g.sync()
        rt.cudaProfilerStart()
        g.step(1, mode)
        g.sync()
        rt.cudaProfilerStop()
        return None, scene, bits, offs
    # the state the timed steps start from: the end-to-end loop below replays the same steps
    n_axes = len(offs) - 1 if offs is not None else 1
    snapshot = (g.state(), g.results(), g.axes(n_axes))
    # device-resident timed region
    g.phase_times(reset=True)
    per_step, launches = [], 0
    with ClockSampler(device) as clk:
        for _ in range(args.steps):
            flush()
            before = g.phase_times()["step"]
            g.step(1, mode)
            per_step.append(g.phase_times()["step"] - before)
            launches += g.last_counts()["launches"]
    counts = g.last_counts()
    dev_ms = float(sum(per_step))
    hull_verts = hull_vertices_per_pair(scene, g.pairs())
    # per-phase durations over the timed steps: the dominant phase and its roofline
    g.phase_times(reset=True)
    for _ in range(args.steps):
        flush()
        g.step(1, mode)
    ph = g.phase_times(reset=True)
    dom = max(PHASES, key=lambda k: ph[k])
    dom_ms = ph[dom] / args.steps
    alg = algorithmic_bytes(counts, N, scene.iterations, bits // 8, hull_verts)
    dom_bytes = alg[dom]   # bytes of the whole phase in one step
    peak, peak_kind = measured_peak()
    achieved = dom_bytes / (dom_ms * 1e-3) / 1e9
    traffic = ncu_traffic(dom) if args.workload == "batched" and args.scenes == 4096 else None
    # latency sample: more steps, each timed alone (no flush between them), for p50/p99
    lat = []
    for _ in range(args.latency_steps):
        before = g.phase_times()["step"]
        g.step(1, mode)
        lat.append(g.phase_times()["step"] - before)
    # per-kernel device time of one profiled step (events around every launch; the narrowphase's
    # kernels overlap on side streams, so their times add up to more than the phase)
    g.set_profiling(True)
    flush()
    g.step(1, mode)
    g.set_profiling(False)
    ks = g.kernel_stats()
    # end to end through the C ABI with host buffers, over the same steps as the timed region
    # (restored from the snapshot): each step copies the poses and velocities in from page-locked
    # host arrays and reads the stepped ones back into them, in the world's real type (float32 for
    # an FP32 world: the reference's default pe::Real)
    import torch   # page-locked host memory
    io = ("origin", "basis", "lin_vel", "ang_vel")
    tdt = torch.float32 if bits == 32 else torch.float64
    st = {f: torch.empty((N, 3, 3) if f == "basis" else (N, 3), dtype=tdt, pin_memory=True).numpy() for f in io}
    g.state(fields=io, out=st)
    g.set_state(st)                      # one untimed pass through the host path
    g.set_state(snapshot[0])
    g.set_results(snapshot[1])
    g.set_axes(snapshot[2])
    g.state(fields=io, out=st)
    e2e_times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        g.set_state(st)
        g.step(1, mode)
        g.state(fields=io, out=st)
        e2e_times.append(time.perf_counter() - t0)
    io_bytes = N * 18 * (4 if bits == 32 else 8)   # poses and velocities through the C ABI, each way
    per_scene = per_scene_gpu(pg, scene, offs, g.state(fields=("origin", "basis", "lin_vel", "ang_vel")), bits, mode,
                              device, args.steps) if offs is not None and not args.no_per_scene else None
    res = dict(dev_ms=dev_ms, per_step=per_step, lat=lat, N=N, launches=launches, counts=counts, cfg=cfg, bits=bits,
               clk=clk.summary(),
               roofline=dict(kernel=f"{dom} phase", bound="hbm", achieved=achieved, peak=peak, unit="GB/s", frac=achieved / peak,
                             traffic=traffic, algorithmic_bytes=dom_bytes, phase_ms=dom_ms, hull_vertices_in_pairs=hull_verts,
                             peak_source=peak_kind, step_bytes=alg["step"],
                             step_frac=alg["step"] / (dev_ms / args.steps * 1e-3) / 1e9 / peak,
                             phases_ms={k: ph[k] / args.steps for k in PHASES},
                             phases_algorithmic_bytes={k: alg[k] for k in PHASES},
                             phases_dram_bytes_ncu={k: ncu_traffic(k) for k in PHASES}
                             if args.workload == "batched" and args.scenes == 4096 else None,
                             traffic_source="profiles/launches_batched_dram.md (ncu, one step of this workload)"
                             if traffic is not None else None),
               e2e=dict(value=N * len(e2e_times) / sum(e2e_times), unit=UNIT, h2d_bytes_per_step=io_bytes,
                        d2h_bytes_per_step=io_bytes, p50_step_ms=sorted(e2e_times)[len(e2e_times) // 2] * 1e3,
                        max_step_ms=max(e2e_times) * 1e3),
               kernels={k: round(v[0], 4) for k, v in ks.items() if v[1]}, per_scene=per_scene)
    return res, scene, bits, offs


def run_leg(name, steps, warmup, device, cpu=False):
    """One of the other configurations on the GPU, device-timed like the main line (L2 flushed
    between steps): body-steps/s, p50/p99 step time, pairs and contact points of the last step;
    with `cpu`, the reference's CPU step (the oracle port, all host threads, serial order) on the
    same scene and precision from its initial state, a few seconds' sample."""
    import pe_gb300 as pg
    scene, bits, mode, offs, cfg = make_workload(name)
    g = pg.GpuWorld(scene, bits, device=device, scenes=offs, margin=cfg.get("margin", 0.0), tuning="auto")
    flush = L2Flush()
    for _ in range(cfg.get("preroll_steps", 0) + warmup):
        g.step(1, mode)
    per = []
    for _ in range(steps):
        flush()
        before = g.phase_times()["step"]
        g.step(1, mode)
        per.append(g.phase_times()["step"] - before)
    c = g.last_counts()
    g.close()
    per_sorted = sorted(per)
    out = dict(value=scene.n_bodies * steps / (sum(per) * 1e-3), unit=UNIT, ms_per_step=sum(per) / steps, steps=steps,
               p50_step_ms=per_sorted[len(per) // 2], p99_step_ms=per_sorted[min(len(per) - 1, int(0.99 * len(per)))],
               pairs=c["pairs"], contact_points=c["rows"], dtype="f64" if bits == 64 else "f32", **cfg)
    if cpu:
        out["cpu_reference"] = cpu_baseline(scene, bits, None, budget_s=4.0, margin=cfg.get("margin", 0.0))
    return out


def per_scene_gpu(pg, scene, offs, state, bits, mode, device, steps, sample=64, warmup=3):
    """The plain one-scene-per-launch GPU path: a stratified sample of the batch's scenes, each
    stepped alone in its own world (same state as in the batch), timed with device events."""
    from pe_gb300 import scene as sc
    S = len(offs) - 1
    picks = np.unique(np.linspace(0, S - 1, min(sample, S)).astype(int))
    bodies, ms, per_step = 0, 0.0, []
    for k in picks:
        b0, b1 = int(offs[k]), int(offs[k + 1])
        w = pg.GpuWorld(sc.extract(scene, offs, k), bits, device=device)
        w.set_state({f: v[b0:b1] for f, v in state.items()})
        for _ in range(warmup):
            w.step(1, mode)
        t0 = w.phase_times()["step"]
        for _ in range(steps):
            w.step(1, mode)
        t = w.phase_times()["step"] - t0
        bodies += (b1 - b0) * steps
        ms += t
        per_step.append(t / steps)
        w.close()
    per_step.sort()
    return dict(value=bodies / (ms * 1e-3), unit=UNIT, scenes=len(picks),
                sample=f"{len(picks)} scenes spread over the batch, each stepped alone {steps} times after {warmup} warm-up steps",
                p50_step_ms=per_step[len(per_step) // 2], p99_step_ms=per_step[min(len(per_step) - 1, int(0.99 * len(per_step)))])


def run_serving(args, device):
    """Serving: Poisson arrivals at 200 requests/s for --serve-seconds (60 s in the configuration);
    each request is a pile of 16..2,048 bodies (log-uniform; drawn from a seeded pool of 256 scenes
    generated like the batched piles) asking for K ~ U[60, 600] steps; admission by a 64 GB budget;
    coloured, FP32.  Throughput = body-steps of all requests / wall time from the first arrival to
    the last completion, through the public API (scenes submitted from host memory, final states
    read back)."""
    import pe_gb300 as pg
    from pe_gb300 import scene as sc
    rng = np.random.default_rng(200)
    merged, offs = sc.batched_piles(n_scenes=256, seed=2048, size_range=(16, 2048), real_bits=32)
    pool = [sc.extract(merged, offs, k) for k in range(256)]
    rate, dur = 200.0, float(args.serve_seconds)
    arr = np.cumsum(rng.exponential(1.0 / rate, size=int(rate * dur * 2) + 16))
    arr = arr[arr < dur]
    ks = rng.integers(60, 601, size=len(arr))
    picks = rng.integers(0, len(pool), size=len(arr))
    srv = pg.Server(real_bits=32, device=device, dt=1.0 / 60.0, iterations=10, mode=pg.COLORED, hbm_budget_bytes=64e9)
    rid = srv.submit(pool[0], 3)           # warm-up request (module loading, first allocations)
    while srv.result(rid)[0] != pg.DONE:
        srv.step()
    base = srv.stats()
    pending, due, lat, loop_ms = {}, {}, [], []
    h2d = d2h = 0
    nxt, steps = 0, 0
    t0 = time.perf_counter()
    with ClockSampler(device) as clk:
        while nxt < len(arr) or pending:
            now = time.perf_counter() - t0
            while nxt < len(arr) and arr[nxt] <= now:
                s = pool[picks[nxt]]
                r = srv.submit(s, int(ks[nxt]))
                pending[r] = arr[nxt]
                due.setdefault(steps + int(ks[nxt]) + 1, []).append(r)
                h2d += s.n_bodies * (18 * 8 + 7 * 8) + s.hull_verts.size * 8
                nxt += 1
            if not pending:
                time.sleep(max(0.0, arr[nxt] - now))
                continue
            t1 = time.perf_counter()
            srv.step()
            loop_ms.append((time.perf_counter() - t1) * 1e3)
            steps += 1
            for r in due.pop(steps, []):
                st, res = srv.result(r)
                if st == pg.DONE:
                    lat.append(time.perf_counter() - t0 - pending.pop(r))
                    d2h += res["origin"].size * 8 * 6
                else:                          # admission was delayed: look again next step
                    due.setdefault(steps + 1, []).append(r)
    wall = time.perf_counter() - t0
    st = srv.stats()
    body_steps = st["body_steps"] - base["body_steps"]
    lat.sort()
    loop_ms.sort()
    pct = lambda a, p: a[min(len(a) - 1, int(p * (len(a) - 1) + 0.5))] if a else None
    value = body_steps / wall
    cfg = dict(workload=f"serving: Poisson arrivals at 200 requests/s over {dur:g} s, piles of 16..2,048 bodies "
                        "(log-uniform, box/sphere/cylinder/convex hull), K ~ U[60,600] steps, 64 GB admission budget, "
                        "FP32, 10 SI iterations, coloured", requests=len(arr), scenes_in_pool=len(pool),
               p50_step_ms=st["p50_step_ms"], p99_step_ms=st["p99_step_ms"], mean_step_ms=st["mean_step_ms"],
               p50_loop_ms=pct(loop_ms, 0.5), p99_loop_ms=pct(loop_ms, 0.99),
               p50_request_s=pct(lat, 0.5), p99_request_s=pct(lat, 0.99), finished=len(lat),
               peak_footprint_gb=st["peak_footprint_bytes"] / 1e9, batched_steps=steps, wall_s=wall)
    return dict(metric=METRIC, value=value, unit=UNIT, n_gpus=1, steps=steps, warmup=0,
                ms_per_step=wall / max(steps, 1) * 1e3, higher_is_better=True, scaling="weak", vs_baseline=None,
                dtype="f32", data="synthetic", config=cfg,
                e2e=dict(value=value, unit=UNIT, h2d_bytes_per_step=h2d / max(steps, 1), d2h_bytes_per_step=d2h / max(steps, 1)),
                gpu_launches=None, clocks=clk.summary())


def cpu_scenes_wall(scene, bits, offs, preroll, steps, sample=256, threads=None):
    """The reference's CPU step (its algorithm restated in oracle/) on a spread sample of the batch's
    scenes, one World per scene (World is not thread-safe; the reference's pool is a process
    singleton), the scenes spread over all host threads.  The pre-roll runs first, untimed; the
    timed region is the wall time of `steps` steps of every sampled scene, all threads busy."""
    import concurrent.futures as cf
    sys.path.insert(0, str(ROOT / "oracle"))
    import orc
    from pe_gb300 import scene as sc
    threads = threads or os.cpu_count() or 1
    S = len(offs) - 1
    picks = np.unique(np.linspace(0, S - 1, min(sample, S)).astype(int))
    worlds = [orc.OracleWorld(sc.extract(scene, offs, int(k)), bits, threads=1) for k in picks]
    bodies = sum(w.n for w in worlds)
    with cf.ThreadPoolExecutor(threads) as ex:   # the oracle's step releases the interpreter lock
        list(ex.map(lambda w: w.step(preroll), worlds))
        t0 = time.perf_counter()
        list(ex.map(lambda w: w.step(steps), worlds))
        wall = time.perf_counter() - t0
    return dict(value=bodies * steps / wall, unit=UNIT, cores=threads, kind="port", ms_per_step=wall / steps * 1e3,
                sample=f"{len(picks)} of the {S:,} scenes ({bodies:,} bodies) spread over the batch, one World per scene on "
                       f"{threads} host threads, {steps} timed steps after {preroll} untimed; wall time {wall:.2f} s")


def cpu_baseline(scene, bits, offs=None, preroll=0, budget_s=20.0, sample=32, steps=5, margin=0.0):
    """The reference's CPU step (its algorithm restated in oracle/) on a bounded sample, all host
    threads.  One scene: the reference's thread pool inside one world.  Independent scenes: one
    scene per host thread (a spawn process pool), a spread sample of the batch."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import orc
    threads = os.cpu_count() or 1
    if offs is None:
        w = orc.OracleWorld(scene, bits, threads=threads, margin=margin)
        t = w.time_steps(1)
        n = 1
        while t < budget_s and n < 64:
            k = max(1, min(int((budget_s - t) / max(t / n, 1e-3)), 8))
            t += w.time_steps(k)
            n += k
        return dict(value=scene.n_bodies * n / t, unit=UNIT, cores=threads, kind="port",
                    sample=f"{n} full steps of the same workload from its initial state ({t:.1f} s, {threads} threads)")
    return cpu_scenes_wall(scene, bits, offs, preroll, steps)


# ------------------------------------------------------------------ replicas (one process per GPU)
def max_over_ranks(x, dist, device=None):
    """The largest value of x over the ranks: the timed region of N replicas ends with the slowest
    (a CUDA tensor under NCCL, a host tensor under gloo)."""
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device if device is not None else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(bodies_per_replica, steps, world, dev_ms):
    """Whole-job body-steps/s of `world` replicas, each stepping its own copy of the workload: every
    rank's bodies over the slowest rank's time (weak scaling)."""
    return bodies_per_replica * steps * world / (dev_ms * 1e-3)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="batched", choices=["batched", "stress", "tower", "tower_colored", "large", "serving"])
    ap.add_argument("--serve-seconds", type=float, default=60.0, help="arrival window of the serving workload")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--scenes", type=int, default=4096, help="scene count of the batched workload")
    ap.add_argument("--no-per-scene", action="store_true", help="skip the one-scene-per-launch comparison")
    ap.add_argument("--profile-one-step", action="store_true",
                    help="after the pre-roll and warm-up, run one step inside cudaProfilerStart/Stop and exit (for ncu)")
    ap.add_argument("--latency-steps", type=int, default=200, help="extra steps timed one by one for p50/p99")
    ap.add_argument("--no-legs", action="store_true",
                    help="skip the other configurations (stress, large, tower, 10 s of serving) reported beside the main line")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local = int(os.environ.get("LOCAL_RANK", 0))

    if args.impl == "reference":
        if rank != 0:
            return 0
        if args.workload == "serving":
            print(json.dumps(dict(impl="reference", unavailable="the reference has no request loop; its CPU step is timed by "
                                                                "the batched workload's reference arm")))
            return 0
        scene, bits, mode, offs, cfg = make_workload(args.workload, args.scenes)
        cfg = dict(cfg, solver="serial: the reference's sequential impulse order (it has no coloured solver)")
        k = max(1, args.steps)
        if offs is None:
            sys.path.insert(0, str(ROOT / "oracle"))
            import orc
            threads = os.cpu_count() or 1
            w = orc.OracleWorld(scene, bits, threads=threads, margin=cfg.get("margin", 0.0))
            for _ in range(args.warmup):   # untimed, like the GPU arm's warm-up
                w.time_steps(1)
            t, done = 0.0, 0
            while done < k and (done == 0 or t < 120.0):   # a bounded sample of the K steps
                t += w.time_steps(1)
                done += 1
            cb = dict(value=scene.n_bodies * done / t, unit=UNIT, cores=threads, kind="port", ms_per_step=t / done * 1e3,
                      sample=f"{done} full steps after {args.warmup} untimed, the whole scene, the reference's thread pool "
                             f"with {threads} host threads")
        else:
            # the GPU arm's untimed pre-roll and warm-up steps, then its K timed steps
            cb = cpu_scenes_wall(scene, bits, offs, cfg.get("preroll_steps", 0) + args.warmup, k)
            done = k
        v = cb["value"]
        print(json.dumps(dict(metric=METRIC, value=v, unit=UNIT, n_gpus=args.gpus, steps=done, warmup=args.warmup,
                              ms_per_step=cb["ms_per_step"], higher_is_better=True, scaling="weak",
                              vs_baseline=None, dtype="f64" if bits == 64 else "f32", data="synthetic", config=cfg,
                              impl="reference", cpu_baseline=cb,
                              e2e=dict(value=v, unit=UNIT, h2d_bytes_per_step=0, d2h_bytes_per_step=0))))
        return 0

    if args.workload == "serving":
        if rank == 0:
            print(json.dumps(run_serving(args, local)))
        return 0

    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
        dist.barrier()
    res, scene, bits, offs = run_ours(args, rank, world, local)
    if res is None:   # --profile-one-step
        print(json.dumps(dict(profiled_step=True, workload=args.workload, bodies=scene.n_bodies)))
        return 0
    dev_ms = res["dev_ms"]
    if dist is not None:
        dev_ms = max_over_ranks(dev_ms, dist, device=f"cuda:{local}")
        dist.barrier()
    if rank != 0:
        return 0
    per = sorted(res["per_step"] + res["lat"])
    value = replica_value(res["N"], args.steps, world, dev_ms)
    cfg = dict(res["cfg"], l2="flushed between timed steps (256 MiB memset)", pairs_last_step=res["counts"]["pairs"],
               contact_points_last_step=res["counts"]["rows"], colors_last_step=res["counts"]["colors"],
               p50_step_ms=per[len(per) // 2], p99_step_ms=per[min(len(per) - 1, int(0.99 * len(per)))],
               latency_sample=f"{len(per)} steps: the {args.steps} timed ones and {len(res['lat'])} more timed one by one",
               contacts_per_s=res["counts"]["rows"] * args.steps * world / (dev_ms * 1e-3), parallelism=f"replicas x{world}")
    if res["per_scene"] is not None:
        cfg["per_scene_gpu"] = res["per_scene"]
        cfg["batched_over_per_scene"] = value / world / res["per_scene"]["value"]
    out = dict(metric=METRIC, value=value, unit=UNIT, n_gpus=world, steps=args.steps, warmup=args.warmup,
               ms_per_step=dev_ms / args.steps, higher_is_better=True, scaling="weak", vs_baseline=None,
               dtype="f64" if bits == 64 else "f32", data="synthetic", config=cfg, roofline=res["roofline"],
               e2e=res["e2e"], gpu_launches=res["launches"], clocks=res["clk"], kernels_ms_one_step=res["kernels"])
    if not args.no_cpu_baseline and world == 1:
        out["cpu_baseline"] = cpu_baseline(scene, bits, offs, preroll=res["cfg"].get("preroll_steps", 0) + args.warmup,
                                           steps=args.steps, margin=res["cfg"].get("margin", 0.0))
    if not args.no_legs and world == 1 and args.workload == "batched" and not args.profile_one_step:
        legs = {}
        for name, k in (("stress", 10), ("large", 10), ("tower", 20), ("tower_colored", 20)):
            legs[name] = run_leg(name, k, 3, local, cpu=name.startswith("tower") and not args.no_cpu_baseline)
        sv = run_serving(argparse.Namespace(serve_seconds=10.0), local)
        legs["serving"] = dict(value=sv["value"], unit=UNIT, **{k: sv["config"][k] for k in (
            "workload", "requests", "finished", "p50_step_ms", "p99_step_ms", "mean_step_ms", "p50_request_s", "p99_request_s",
            "peak_footprint_gb", "batched_steps", "wall_s")})
        out["config"]["other_configs"] = legs
    print(json.dumps(out))
    return 0


if __name__ == "__main__":
    sys.exit(main())
