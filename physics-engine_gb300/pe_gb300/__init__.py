"""Python binding of the GB300 rigid-body step (ctypes over include/pe_gpu.h).

``GpuWorld`` mirrors pe_intf::World (src/intf/world.h): it is built from a ``Scene``
(shapes + bodies, see ``scene.py``), stepped with ``step()``, and exposes the reference's
phase boundaries (integrate / broadphase / narrowphase / solve) for phase-by-phase use.
The CUDA library is required: loading fails loudly when it is missing or no GPU is present.
"""
import ctypes as C
from pathlib import Path

import numpy as np

from .scene import Scene  # noqa: F401

PKG = Path(__file__).resolve().parent.parent
LIB_PATH = PKG / "lib" / "libpe_gpu.so"
HEADER = PKG.parent / "include" / "pe_gpu.h"

SERIAL_ORDER, COLORED = 0, 1
_lib = None


class PeGpuError(RuntimeError):
    pass


def load(build_if_missing: bool = True):
    """Load libpe_gpu.so (building it in-tree first when absent)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        if not build_if_missing:
            raise PeGpuError(f"{LIB_PATH} is missing; run physics-engine_gb300/pe_gb300/build.py")
        from .build import build
        build()
    lib = C.CDLL(str(LIB_PATH))
    P, I, D = C.c_void_p, C.c_int, C.c_double
    dp = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
    ip = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
    sig = {
        "pe_gpu_create": (I, [C.c_void_p, C.POINTER(P)]),
        "pe_gpu_destroy": (I, [P]),
        "pe_gpu_last_error": (C.c_char_p, [P]),
        "pe_gpu_set_shapes": (I, [P, I, ip, dp, ip, ip, ip, ip, I, dp, I, ip, ip]),
        "pe_gpu_set_bodies": (I, [P, I, ip, ip, dp, dp, dp, dp, dp, dp, dp, dp, dp]),
        "pe_gpu_set_compounds": (I, [P, ip, ip, I, ip, dp, dp, dp, P, dp]),
        "pe_gpu_set_joints": (I, [P, I, ip, ip, ip, dp]),
        "pe_gpu_set_ignore_pairs": (I, [P, I, ip]),
        "pe_gpu_set_scenes": (I, [P, I, ip]),
        "pe_gpu_set_params": (I, [P, D, D, D, D, I]),
        "pe_gpu_set_contact_margin": (I, [P, D]),
        "pe_gpu_get_tuning": (I, [P, C.c_void_p]), "pe_gpu_set_tuning": (I, [P, C.c_void_p]),
        "pe_gpu_device_name": (I, [I, C.c_char_p, I]),
        "pe_gpu_step": (I, [P, I, I]),
        "pe_gpu_integrate": (I, [P]),
        "pe_gpu_broadphase": (I, [P, C.POINTER(I)]),
        "pe_gpu_narrowphase": (I, [P]),
        "pe_gpu_solve": (I, [P, I]),
        "pe_gpu_n_bodies": (I, [P]), "pe_gpu_n_pairs": (I, [P]), "pe_gpu_n_results": (I, [P]),
        "pe_gpu_get_state": (I, [P] + [P] * 7),
        "pe_gpu_set_state": (I, [P] + [P] * 7),
        "pe_gpu_get_axes": (I, [P, ip]), "pe_gpu_set_axes": (I, [P, ip]),
        "pe_gpu_get_pairs": (I, [P, ip]), "pe_gpu_set_pairs": (I, [P, I, ip]),
        "pe_gpu_get_results": (I, [P, ip, ip, ip, dp, dp, dp]),
        "pe_gpu_set_results": (I, [P, I, ip, ip, ip, dp, dp, dp]),
        "pe_gpu_phase_times": (I, [P, dp, I]),
        "pe_gpu_last_counts": (I, [P, ip]),
        "pe_gpu_sync": (I, [P]),
        "pe_gpu_set_profiling": (I, [P, I]),
        "pe_gpu_set_step_graphs": (I, [P, I]),
        "pe_gpu_get_state_f32": (I, [P] + [P] * 7),
        "pe_gpu_set_state_f32": (I, [P] + [P] * 7),
        "pe_gpu_kernel_count": (I, []),
        "pe_gpu_kernel_name": (C.c_char_p, [I]),
        "pe_gpu_kernel_stats": (I, [P, dp, np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")]),
        # device pointers throughout (see include/pe_gpu.h)
        "pe_gpu_sap_pairs_noalloc": (I, [I, I, P, P, P, I, P, I, P, P, C.c_char_p, I]),
        "pe_gpu_server_create": (I, [C.c_void_p, D, D, D, D, I, I, D, C.POINTER(P)]),
        "pe_gpu_server_destroy": (I, [P]),
        "pe_gpu_server_last_error": (C.c_char_p, [P]),
        "pe_gpu_server_submit": (I, [P, C.c_void_p, I, C.POINTER(C.c_longlong)]),
        "pe_gpu_server_step": (I, [P, C.POINTER(I), C.POINTER(I)]),
        "pe_gpu_server_result": (I, [P, C.c_longlong, C.POINTER(I), P, P, P, P]),
        "pe_gpu_server_stats": (I, [P, dp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype, f.argtypes = res, args
    _lib = lib
    return lib


class _Config(C.Structure):
    _fields_ = [("real_bits", C.c_int), ("device", C.c_int)]


TUNING_FIELDS = ("sat_heavy_cost", "small_island_items", "big_island_items", "color_block", "level_block",
                 "exact_levels_colored", "scene_sort_max", "side_streams")


class _Tuning(C.Structure):
    _fields_ = [(f, C.c_int) for f in TUNING_FIELDS]


def autotune_table_present(device=0, real_bits=32):
    """Whether the autotuner stored settings for this GPU model and real type."""
    from .autotune import load_table
    return bool(load_table(device_name(device), real_bits))


def device_name(device=0):
    """The CUDA device's name (cudaGetDeviceProperties), e.g. "NVIDIA GB300"."""
    buf = C.create_string_buffer(256)
    rc = load().pe_gpu_device_name(int(device), buf, 256)
    if rc != 0:
        raise PeGpuError(f"pe_gpu_device_name failed ({rc})")
    return buf.value.decode()


def _f64(a, shape=None):
    a = np.ascontiguousarray(a, np.float64)
    return a.reshape(shape) if shape is not None else a


def _i32(a):
    return np.ascontiguousarray(a, np.int32)


class GpuWorld:
    """A device-resident world (or batch of independent scenes) on one GPU."""

    def __init__(self, scene, real_bits=64, device=0, scenes=None, margin=0.0, tuning=None):
        self.lib = load()
        self.h = C.c_void_p()
        cfg = _Config(real_bits, device)
        rc = self.lib.pe_gpu_create(C.byref(cfg), C.byref(self.h))
        if rc != 0:
            raise PeGpuError(f"pe_gpu_create failed ({rc}): no usable CUDA device?")
        self.real_bits = real_bits
        s = scene
        self._ck(self.lib.pe_gpu_set_shapes(
            self.h, s.n_shapes, _i32(s.shape_type), _f64(s.shape_param).ravel(), _i32(s.hull_vbeg), _i32(s.hull_vcnt),
            _i32(s.hull_fbeg), _i32(s.hull_fcnt), len(s.hull_verts), _f64(s.hull_verts).ravel() if len(s.hull_verts) else np.zeros(1),
            len(s.hull_face_off) - 1, _i32(s.hull_face_off), _i32(s.hull_face_idx) if len(s.hull_face_idx) else np.zeros(1, np.int32)))
        self.centroids = np.zeros((s.n_shapes, 3))
        if (np.asarray(s.shape_type) == 5).any():   # compound shapes: addShape + init()
            cb, cc = s.compound_tables()
            C_ = s.n_children
            self._ck(self.lib.pe_gpu_set_compounds(
                self.h, _i32(cb), _i32(cc), C_, _i32(s.child_shape) if C_ else np.zeros(1, np.int32),
                _f64(s.child_origin).ravel() if C_ else np.zeros(3), _f64(s.child_basis).ravel() if C_ else np.zeros(9),
                _f64(s.child_ratio) if C_ else np.zeros(1), None, self.centroids.reshape(-1)))
        self._ck(self.lib.pe_gpu_set_bodies(
            self.h, s.n_bodies, _i32(s.body_shape), _i32(s.body_flags), _f64(s.mass), _f64(s.friction), _f64(s.restitution),
            _f64(s.lin_damp), _f64(s.ang_damp), _f64(s.origin).ravel(), _f64(s.basis).ravel(), _f64(s.lin_vel).ravel(),
            _f64(s.ang_vel).ravel()))
        if s.n_joints:
            self._ck(self.lib.pe_gpu_set_joints(self.h, s.n_joints, _i32(s.joint_type), _i32(s.joint_body).ravel(),
                                                _i32(s.joint_flag), _f64(s.joint_real).ravel()))
        if len(s.ignore_pairs):
            self._ck(self.lib.pe_gpu_set_ignore_pairs(self.h, len(s.ignore_pairs), _i32(s.ignore_pairs).ravel()))
        self._ck(self.lib.pe_gpu_set_params(self.h, float(s.dt), *map(float, s.gravity), int(s.iterations)))
        if margin:
            self._ck(self.lib.pe_gpu_set_contact_margin(self.h, float(margin)))
        if tuning is not None:   # a dict of scheduling settings, or "auto": the stored table for this GPU
            if tuning == "auto":
                from .autotune import load_table
                tuning = load_table(device_name(device), real_bits)
            if tuning:
                self.set_tuning(**tuning)
        if scenes is not None:
            self.set_scenes(scenes)

    def tuning(self):
        t = _Tuning()
        self._ck(self.lib.pe_gpu_get_tuning(self.h, C.byref(t)))
        return {f: getattr(t, f) for f in TUNING_FIELDS}

    def set_tuning(self, **kw):
        """Scheduling settings (pe_gpu_tuning); unknown names are refused, unnamed ones keep their value."""
        cur = self.tuning()
        bad = set(kw) - set(TUNING_FIELDS)
        if bad:
            raise ValueError(f"unknown tuning settings {sorted(bad)}")
        cur.update({k: int(v) for k, v in kw.items()})
        self._ck(self.lib.pe_gpu_set_tuning(self.h, C.byref(_Tuning(**cur))))

    def _ck(self, rc):
        if rc != 0:
            msg = self.lib.pe_gpu_last_error(self.h)
            raise PeGpuError(f"pe_gpu call failed ({rc}): {msg.decode() if msg else ''}")

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            self.lib.pe_gpu_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---------------------------------------------------------------- stepping
    def set_params(self, dt, gravity=(0.0, -9.8, 0.0), iterations=10):
        """World::setDt / setGravity and the solver's iteration count."""
        self._ck(self.lib.pe_gpu_set_params(self.h, float(dt), *map(float, gravity), int(iterations)))

    def set_scenes(self, body_off):
        off = _i32(body_off)
        self._ck(self.lib.pe_gpu_set_scenes(self.h, len(off) - 1, off))

    def step(self, k=1, mode=COLORED):
        self._ck(self.lib.pe_gpu_step(self.h, int(k), int(mode)))

    def integrate(self):
        self._ck(self.lib.pe_gpu_integrate(self.h))

    def broadphase(self):
        n = C.c_int(0)
        self._ck(self.lib.pe_gpu_broadphase(self.h, C.byref(n)))
        return n.value

    def narrowphase(self):
        self._ck(self.lib.pe_gpu_narrowphase(self.h))

    def solve(self, mode=SERIAL_ORDER):
        self._ck(self.lib.pe_gpu_solve(self.h, int(mode)))

    def sync(self):
        self._ck(self.lib.pe_gpu_sync(self.h))

    # ---------------------------------------------------------------- state
    @property
    def n(self):
        return self.lib.pe_gpu_n_bodies(self.h)

    STATE_FIELDS = (("origin", 3), ("basis", 9), ("lin_vel", 3), ("ang_vel", 3), ("aabb_min", 3), ("aabb_max", 3),
                    ("world_inv_inertia", 9))

    def state(self, fields=None, out=None, dtype=np.float64):
        """Body state as arrays of ``dtype`` (float64, or float32: the reference's default pe::Real);
        ``fields`` limits the transfer to the named fields.  With ``out`` (a dict of C-contiguous
        arrays of the fields' shapes and one dtype, e.g. page-locked host memory reused across steps)
        the fields are written there and ``out`` is returned."""
        N = self.n
        dst, out, ptrs = out, {}, []
        if dst is not None and dst:
            dtype = next(iter(dst.values())).dtype
        dtype = np.dtype(dtype)
        if dtype not in (np.dtype(np.float64), np.dtype(np.float32)):
            raise ValueError("state: dtype must be float64 or float32")
        for name, k in self.STATE_FIELDS:
            if fields is None or name in fields:
                shape = (N, 3, 3) if k == 9 else (N, 3)
                if dst is not None:
                    a = dst[name]
                    if a.shape != shape or a.dtype != dtype or not a.flags.c_contiguous:
                        raise ValueError(f"state: out[{name!r}] must be C-contiguous {dtype} of shape {shape}")
                else:
                    a = np.zeros(shape, dtype)
                out[name] = a
                ptrs.append(a.ctypes.data_as(C.c_void_p))
            else:
                ptrs.append(None)
        fn = self.lib.pe_gpu_get_state if dtype == np.float64 else self.lib.pe_gpu_get_state_f32
        self._ck(fn(self.h, *ptrs))
        return dst if dst is not None else out

    def set_state(self, d):
        """Overwrite the given body-state fields (missing keys are left untouched).  All-float32
        arrays go through the single-precision entry point, anything else as float64."""
        given = [d[name] for name, _ in self.STATE_FIELDS if name in d and d[name] is not None]
        f32 = bool(given) and all(isinstance(a, np.ndarray) and a.dtype == np.float32 for a in given)
        keep, ptrs = [], []
        for name, k in self.STATE_FIELDS:
            if name in d and d[name] is not None:
                a = np.ascontiguousarray(d[name], np.float32).reshape(-1) if f32 else _f64(d[name]).reshape(-1)
                keep.append(a)
                ptrs.append(a.ctypes.data_as(C.c_void_p))
            else:
                ptrs.append(None)
        fn = self.lib.pe_gpu_set_state_f32 if f32 else self.lib.pe_gpu_set_state
        self._ck(fn(self.h, *ptrs))

    def axes(self, n_scenes=1):
        out = np.zeros(n_scenes, np.int32)
        self._ck(self.lib.pe_gpu_get_axes(self.h, out))
        return out

    def set_axes(self, axes):
        self._ck(self.lib.pe_gpu_set_axes(self.h, _i32(np.atleast_1d(axes))))

    @property
    def axis(self):
        return int(self.axes(1)[0])

    @axis.setter
    def axis(self, a):
        self.set_axes([a])

    def pairs(self):
        P = self.lib.pe_gpu_n_pairs(self.h)
        out = np.zeros((max(P, 1), 2), np.int32)
        self._ck(self.lib.pe_gpu_get_pairs(self.h, out.reshape(-1)))
        return out[:P]

    def set_pairs(self, p):
        p = _i32(p).reshape(-1, 2)
        self._ck(self.lib.pe_gpu_set_pairs(self.h, len(p), p.reshape(-1) if len(p) else np.zeros(2, np.int32)))

    def results(self):
        R = self.lib.pe_gpu_n_results(self.h)
        n = max(R, 1)
        a, b, ps = (np.zeros(n, np.int32) for _ in range(3))
        fr, re = np.zeros(n), np.zeros(n)
        slots = np.zeros((n, 8, 19))
        self._ck(self.lib.pe_gpu_get_results(self.h, a, b, ps, fr, re, slots.reshape(-1)))
        valid = np.array([(1 << k) - 1 for k in ps[:R]], np.int32) if R else np.zeros(0, np.int32)
        return dict(res_a=a[:R], res_b=b[:R], point_size=ps[:R], friction=fr[:R], restitution=re[:R], slots=slots[:R],
                    valid_mask=valid)

    def set_results(self, d):
        R = len(d["res_a"])
        if R == 0:
            z = np.zeros(1, np.int32)
            self._ck(self.lib.pe_gpu_set_results(self.h, 0, z, z, z, np.zeros(1), np.zeros(1), np.zeros(19 * 8)))
            return
        self._ck(self.lib.pe_gpu_set_results(self.h, R, _i32(d["res_a"]), _i32(d["res_b"]), _i32(d["point_size"]),
                                             _f64(d["friction"]), _f64(d["restitution"]), _f64(d["slots"]).reshape(-1)))

    def phase_times(self, reset=False):
        ms = np.zeros(5)
        self._ck(self.lib.pe_gpu_phase_times(self.h, ms, int(reset)))
        return dict(integrate=ms[0], broadphase=ms[1], narrowphase=ms[2], solver=ms[3], step=ms[4])

    def last_counts(self):
        c = np.zeros(6, np.int32)
        self._ck(self.lib.pe_gpu_last_counts(self.h, c))
        return dict(pairs=int(c[0]), active=int(c[1]), rows=int(c[2]), colors=int(c[3]), launches=int(c[4]), islands=int(c[5]))

    def set_profiling(self, on=True):
        self._ck(self.lib.pe_gpu_set_profiling(self.h, int(bool(on))))

    def set_step_graphs(self, on=True):
        """Replay each step's device part from a captured CUDA graph (default) or launch it kernel by kernel."""
        self._ck(self.lib.pe_gpu_set_step_graphs(self.h, int(bool(on))))

    def kernel_stats(self):
        """{kernel group: (device ms, launches)} accumulated while profiling was on."""
        n = self.lib.pe_gpu_kernel_count()
        ms = np.zeros(n)
        cnt = np.zeros(n, np.int64)
        self._ck(self.lib.pe_gpu_kernel_stats(self.h, ms, cnt))
        return {self.lib.pe_gpu_kernel_name(k).decode(): (float(ms[k]), int(cnt[k])) for k in range(n)}


class _SceneDesc(C.Structure):
    _fields_ = [("n_shapes", C.c_int), ("shape_type", C.c_void_p), ("shape_param", C.c_void_p),
                ("hull_vbeg", C.c_void_p), ("hull_vcnt", C.c_void_p), ("hull_fbeg", C.c_void_p), ("hull_fcnt", C.c_void_p),
                ("n_hull_verts", C.c_int), ("hull_verts", C.c_void_p), ("n_hull_faces", C.c_int), ("hull_face_off", C.c_void_p),
                ("hull_face_idx", C.c_void_p), ("n_bodies", C.c_int), ("body_shape", C.c_void_p), ("body_flags", C.c_void_p),
                ("mass", C.c_void_p), ("friction", C.c_void_p), ("restitution", C.c_void_p), ("lin_damp", C.c_void_p),
                ("ang_damp", C.c_void_p), ("origin", C.c_void_p), ("basis", C.c_void_p), ("lin_vel", C.c_void_p),
                ("ang_vel", C.c_void_p)]


QUEUED, RUNNING, DONE, REJECTED = 0, 1, 2, 3


class Server:
    """Request loop over one device-resident world (pe_gpu_server_*): submit scenes with a step
    count, call step() to retire, admit by HBM footprint and advance all live scenes together."""

    def __init__(self, real_bits=32, device=0, dt=1.0 / 60.0, gravity=(0.0, -9.8, 0.0), iterations=10, mode=COLORED,
                 hbm_budget_bytes=64e9):
        self.lib = load()
        self.h = C.c_void_p()
        cfg = _Config(real_bits, device)
        rc = self.lib.pe_gpu_server_create(C.byref(cfg), float(dt), *map(float, gravity), int(iterations), int(mode),
                                           float(hbm_budget_bytes), C.byref(self.h))
        if rc != 0:
            raise PeGpuError(f"pe_gpu_server_create failed ({rc})")
        self.n_bodies = {}

    def _ck(self, rc):
        if rc != 0:
            msg = self.lib.pe_gpu_server_last_error(self.h)
            raise PeGpuError(f"pe_gpu_server call failed ({rc}): {msg.decode() if msg else ''}")

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            self.lib.pe_gpu_server_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, s, n_steps):
        keep = [_i32(s.shape_type), _f64(s.shape_param).ravel(), _i32(s.hull_vbeg), _i32(s.hull_vcnt), _i32(s.hull_fbeg),
                _i32(s.hull_fcnt), _f64(s.hull_verts).ravel() if len(s.hull_verts) else np.zeros(3),
                _i32(s.hull_face_off), _i32(s.hull_face_idx) if len(s.hull_face_idx) else np.zeros(1, np.int32),
                _i32(s.body_shape), _i32(s.body_flags), _f64(s.mass), _f64(s.friction), _f64(s.restitution),
                _f64(s.lin_damp), _f64(s.ang_damp), _f64(s.origin).ravel(), _f64(s.basis).ravel(), _f64(s.lin_vel).ravel(),
                _f64(s.ang_vel).ravel()]
        ptr = [a.ctypes.data for a in keep]
        d = _SceneDesc(s.n_shapes, ptr[0], ptr[1], ptr[2], ptr[3], ptr[4], ptr[5], len(s.hull_verts), ptr[6],
                       len(s.hull_face_off) - 1, ptr[7], ptr[8], s.n_bodies, ptr[9], ptr[10], ptr[11], ptr[12], ptr[13],
                       ptr[14], ptr[15], ptr[16], ptr[17], ptr[18], ptr[19])
        rid = C.c_longlong()
        self._ck(self.lib.pe_gpu_server_submit(self.h, C.byref(d), int(n_steps), C.byref(rid)))
        self.n_bodies[rid.value] = s.n_bodies
        return rid.value

    def step(self):
        live, queued = C.c_int(), C.c_int()
        self._ck(self.lib.pe_gpu_server_step(self.h, C.byref(live), C.byref(queued)))
        return live.value, queued.value

    def result(self, rid):
        """(state, final state dict or None); a finished request's state is returned once."""
        n = self.n_bodies[rid]
        o, b, v, w = np.zeros((n, 3)), np.zeros((n, 3, 3)), np.zeros((n, 3)), np.zeros((n, 3))
        st = C.c_int()
        self._ck(self.lib.pe_gpu_server_result(self.h, C.c_longlong(rid), C.byref(st), o.ctypes.data, b.ctypes.data,
                                                v.ctypes.data, w.ctypes.data))
        if st.value in (DONE, REJECTED):
            del self.n_bodies[rid]
        return st.value, (dict(origin=o, basis=b, lin_vel=v, ang_vel=w) if st.value == DONE else None)

    def stats(self):
        out = np.zeros(10)
        self._ck(self.lib.pe_gpu_server_stats(self.h, out))
        keys = ("p50_step_ms", "p99_step_ms", "mean_step_ms", "steps", "body_steps", "admitted", "finished",
                "peak_footprint_bytes", "live", "queued")
        return dict(zip(keys, out.tolist()))
