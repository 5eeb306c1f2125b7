"""ctypes wrapper of the oracle library (test infrastructure only).

``OracleWorld`` exposes the four phases of the reference step separately so that
the GPU path can be compared phase by phase on identical inputs.
"""
import ctypes as C
import os
import tempfile
from pathlib import Path

import numpy as np

from build_oracle import build

_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(str(build()))
        P, I, D = C.c_void_p, C.c_int, C.c_double
        dp = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
        ip = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
        sig = {
            "orc_create": (P, [C.c_char_p, I, I]),
            "orc_destroy": (None, [P]),
            "orc_n_bodies": (I, [P]), "orc_n_pairs": (I, [P]), "orc_n_results": (I, [P]),
            "orc_get_axis": (I, [P]), "orc_set_axis": (None, [P, I]), "orc_set_margin": (None, [P, D]), "orc_set_stable_ties": (None, [P, I]),
            "orc_step": (None, [P, I]), "orc_time_steps": (D, [P, I]),
            "orc_integrate": (None, [P]), "orc_broadphase": (I, [P]), "orc_narrowphase": (None, [P]),
            "orc_solve": (None, [P]),
            "orc_get_state": (None, [P, dp, dp, dp, dp, dp, dp, dp]),
            "orc_set_state": (None, [P, dp, dp, dp, dp, dp, dp, dp]),
            "orc_get_pairs": (None, [P, ip]), "orc_set_pairs": (None, [P, ip, I]),
            "orc_get_results": (None, [P, ip, ip, ip, ip, dp, dp, dp]),
            "orc_set_results": (None, [P, I, ip, ip, ip, dp, dp, dp]),
            "orc_shape_counts": (I, [P, I, C.POINTER(I), C.POINTER(I), C.POINTER(I)]),
        }
        for name, (res, args) in sig.items():
            f = getattr(_lib, name)
            f.restype, f.argtypes = res, args
    return _lib


class OracleWorld:
    def __init__(self, scene, real_bits=64, threads=1, margin=0.0, stable_ties=False):
        L = lib()
        fd, path = tempfile.mkstemp(suffix=".pescene")
        os.close(fd)
        try:
            scene.write(path)
            self.h = L.orc_create(path.encode(), real_bits, threads)
        finally:
            os.unlink(path)
        if not self.h:
            raise RuntimeError("oracle could not load the scene")
        self.real_bits = real_bits
        if margin:
            L.orc_set_margin(self.h, float(margin))
        if stable_ties:
            L.orc_set_stable_ties(self.h, 1)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    @property
    def n(self):
        return lib().orc_n_bodies(self.h)

    def step(self, k=1):
        lib().orc_step(self.h, k)

    def time_steps(self, k):
        return lib().orc_time_steps(self.h, k)

    def integrate(self):
        lib().orc_integrate(self.h)

    def broadphase(self):
        return lib().orc_broadphase(self.h)

    def narrowphase(self):
        lib().orc_narrowphase(self.h)

    def solve(self):
        lib().orc_solve(self.h)

    @property
    def axis(self):
        return lib().orc_get_axis(self.h)

    @axis.setter
    def axis(self, a):
        lib().orc_set_axis(self.h, int(a))

    def state(self):
        N = self.n
        o, v, w, mn, mx = (np.zeros((N, 3)) for _ in range(5))
        b, iw = np.zeros((N, 3, 3)), np.zeros((N, 3, 3))
        lib().orc_get_state(self.h, o, b, v, w, mn, mx, iw)
        return dict(origin=o, basis=b, lin_vel=v, ang_vel=w, aabb_min=mn, aabb_max=mx, world_inv_inertia=iw)

    def set_state(self, d):
        a = lambda k: np.ascontiguousarray(d[k], np.float64)
        lib().orc_set_state(self.h, a("origin"), a("basis"), a("lin_vel"), a("ang_vel"), a("aabb_min"),
                            a("aabb_max"), a("world_inv_inertia"))

    def pairs(self):
        P = lib().orc_n_pairs(self.h)
        out = np.zeros((P, 2), np.int32)
        if P:
            lib().orc_get_pairs(self.h, out)
        return out

    def set_pairs(self, p):
        p = np.ascontiguousarray(p, np.int32).reshape(-1, 2)
        lib().orc_set_pairs(self.h, p, len(p))

    def results(self):
        R = lib().orc_n_results(self.h)
        a, b, ps, m = (np.zeros(R, np.int32) for _ in range(4))
        fr, re = np.zeros(R), np.zeros(R)
        slots = np.zeros((R, 8, 19))
        if R:
            lib().orc_get_results(self.h, a, b, ps, m, fr, re, slots)
        return dict(res_a=a, res_b=b, point_size=ps, valid_mask=m, friction=fr, restitution=re, slots=slots)

    def set_results(self, d):
        R = len(d["res_a"])
        lib().orc_set_results(self.h, R, np.ascontiguousarray(d["res_a"], np.int32),
                              np.ascontiguousarray(d["res_b"], np.int32),
                              np.ascontiguousarray(d["point_size"], np.int32),
                              np.ascontiguousarray(d["friction"], np.float64),
                              np.ascontiguousarray(d["restitution"], np.float64),
                              np.ascontiguousarray(d["slots"], np.float64).reshape(R, 8, 19))
