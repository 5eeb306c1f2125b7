"""Reader for ``.pedump`` files: per-step phase records of the reference harness.

Test infrastructure only.  Layout (little-endian), written by oracle/ref_harness.cpp:
  magic "PEDUMP1\\0", int32 real_bytes, then per recorded step:
  int32 step, N, axis_before, axis_after, P, R
  f64 origin[N,3], basis[N,3,3], lin_vel[N,3], ang_vel[N,3], aabb_min[N,3], aabb_max[N,3],
      world_inv_inertia[N,3,3]                       (state seen by the broadphase)
  int32 pairs[P,2]                                   (broadphase output, in order)
  int32 res_a[R], res_b[R], point_size[R], valid_mask[R]
  f64 friction[R], restitution[R], slots[R,8,19]     (narrowphase output, all 8 cache slots)
  f64 lin_vel_post[N,3], ang_vel_post[N,3]           (after the solver)
Slot fields: world_pos(3) world_normal(3) local_a(3) local_b(3) distance(1) tangent0(3) tangent1(3).
"""
import struct
from pathlib import Path

import numpy as np

SLOT_POS, SLOT_NRM, SLOT_LA, SLOT_LB, SLOT_DIST, SLOT_T0, SLOT_T1 = (
    slice(0, 3), slice(3, 6), slice(6, 9), slice(9, 12), 12, slice(13, 16), slice(16, 19))


def read(path):
    b = Path(path).read_bytes()
    if b[:8] != b"PEDUMP1\x00":
        raise ValueError("not a pedump")
    real_bytes = struct.unpack_from("<i", b, 8)[0]
    off = 12
    steps = []
    while off < len(b):
        step, N, ax0, ax1, P, R = struct.unpack_from("<6i", b, off)
        off += 24

        def take(n, t, shape):
            nonlocal off
            a = np.frombuffer(b, dtype=t, count=n, offset=off).copy()
            off += a.nbytes
            return a.reshape(shape)

        d = dict(step=step, n=N, axis_before=ax0, axis_after=ax1, real_bytes=real_bytes)
        d["origin"] = take(N * 3, "<f8", (N, 3))
        d["basis"] = take(N * 9, "<f8", (N, 3, 3))
        d["lin_vel"] = take(N * 3, "<f8", (N, 3))
        d["ang_vel"] = take(N * 3, "<f8", (N, 3))
        d["aabb_min"] = take(N * 3, "<f8", (N, 3))
        d["aabb_max"] = take(N * 3, "<f8", (N, 3))
        d["world_inv_inertia"] = take(N * 9, "<f8", (N, 3, 3))
        d["pairs"] = take(P * 2, "<i4", (P, 2))
        d["res_a"] = take(R, "<i4", (R,))
        d["res_b"] = take(R, "<i4", (R,))
        d["point_size"] = take(R, "<i4", (R,))
        d["valid_mask"] = take(R, "<i4", (R,))
        d["friction"] = take(R, "<f8", (R,))
        d["restitution"] = take(R, "<f8", (R,))
        d["slots"] = take(R * 8 * 19, "<f8", (R, 8, 19))
        d["lin_vel_post"] = take(N * 3, "<f8", (N, 3))
        d["ang_vel_post"] = take(N * 3, "<f8", (N, 3))
        steps.append(d)
    return steps
