"""pe_gpu_sap_pairs_noalloc, the broadphase variant whose temporaries live in a fixed device
scratch array, against the world's broadphase (pe_gpu_broadphase) through the C ABI: the same
pairs in the same order on two steps in a row; against the oracle's sweep-and-prune at the size
limit and with bodies flagged ignore-collision; its argument checks, its size limit, its overflow
report, a NULL flags array, fewer than two bodies and a stream of the caller's own.

The test allocates the device buffers it hands over (cudaMalloc through ctypes); the entry point
itself allocates nothing.  Kept in its own file, collected last, so that it also runs after the
other GPU tests have used the device."""
import ctypes as C

import numpy as np
import pytest

import pe_gb300 as pg
from pe_gb300 import scene as sc

pytestmark = pytest.mark.gpu


def _cudart():
    for name in ("libcudart.so", "libcudart.so.13", "/usr/local/cuda/lib64/libcudart.so"):
        try:
            return C.CDLL(name)
        except OSError:
            pass
    pytest.skip("libcudart not found")


class Dev:
    """A device buffer owned by the test."""

    def __init__(self, rt, nbytes):
        self.rt, self.p = rt, C.c_void_p()
        assert rt.cudaMalloc(C.byref(self.p), C.c_size_t(max(nbytes, 4))) == 0

    def put(self, a):
        a = np.ascontiguousarray(a)
        assert self.rt.cudaMemcpy(self.p, a.ctypes.data_as(C.c_void_p), C.c_size_t(a.nbytes), 1) == 0

    def get(self, dtype, count):
        a = np.zeros(count, dtype)
        assert self.rt.cudaMemcpy(a.ctypes.data_as(C.c_void_p), self.p, C.c_size_t(a.nbytes), 2) == 0
        return a

    def free(self):
        self.rt.cudaFree(self.p)


def _noalloc_pairs(lib, rt, mn, mx, flags, axis, cap, stream=None):
    n = len(mn)
    bufs = [Dev(rt, 12 * n), Dev(rt, 12 * n), Dev(rt, 4 * n), Dev(rt, 8 * max(cap, 1)), Dev(rt, 4)]
    dmn, dmx, dfl, dpairs, dn = bufs
    if n:
        dmn.put(mn.astype(np.float32))
        dmx.put(mx.astype(np.float32))
    if flags is not None and n:
        dfl.put(flags.astype(np.int32))
    dn.put(np.array([-7], np.int32))      # must be overwritten
    err = C.create_string_buffer(256)
    rc = lib.pe_gpu_sap_pairs_noalloc(0, n, dmn.p, dmx.p, dfl.p if flags is not None else None, axis, dpairs.p, cap, dn.p,
                                      stream, err, 256)
    assert rc == 0, err.value
    assert rt.cudaDeviceSynchronize() == 0
    count = int(dn.get(np.int32, 1)[0])
    pairs = dpairs.get(np.int32, 2 * min(count, cap)).reshape(-1, 2)
    for b in bufs:
        b.free()
    return count, pairs


def test_noalloc_pairs_equal_world_broadphase_on_two_steps():
    rt = _cudart()
    scene = sc.pile(3000, seed=11, real_bits=32, hull_range=(8, 16), drop=(0.0, 0.5))
    g = pg.GpuWorld(scene, 32)
    lib = g.lib
    for step in range(2):
        axis = g.axis                      # the axis this step's sweep sorts along
        g.integrate()
        n_ref = g.broadphase()
        ref = g.pairs()
        st = g.state(fields=("aabb_min", "aabb_max"))
        count, got = _noalloc_pairs(lib, rt, st["aabb_min"], st["aabb_max"], scene.body_flags, axis, cap=n_ref + 64)
        assert n_ref > 300
        assert count == n_ref, f"step {step}"
        np.testing.assert_array_equal(got, ref, err_msg=f"step {step}")
        g.narrowphase()
        g.solve(pg.COLORED)


def test_noalloc_limits_and_overflow():
    rt = _cudart()
    lib = pg.load()
    err = C.create_string_buffer(256)
    dummy = Dev(rt, 64)
    # beyond the fixed scratch: rejected before any device work, with a message
    rc = lib.pe_gpu_sap_pairs_noalloc(0, 16385, dummy.p, dummy.p, None, 0, dummy.p, 1, dummy.p, None, err, 256)
    assert rc == -3 and b"16384" in err.value
    rc = lib.pe_gpu_sap_pairs_noalloc(0, 10, dummy.p, dummy.p, None, 3, dummy.p, 1, dummy.p, None, err, 256)
    assert rc == -1
    dummy.free()
    # a pair buffer that is too small: the full count is still reported
    scene = sc.pile(400, seed=3, real_bits=32, hull_range=(8, 12), drop=(0.0, 0.2))
    g = pg.GpuWorld(scene, 32)
    axis = g.axis
    g.integrate()
    n_ref = g.broadphase()
    st = g.state(fields=("aabb_min", "aabb_max"))
    count, _ = _noalloc_pairs(lib, rt, st["aabb_min"], st["aabb_max"], scene.body_flags, axis, cap=n_ref // 2)
    assert n_ref > 10 and count == n_ref


def _oracle_sweep(scene):
    """The oracle's sweep-and-prune on the scene's first step: the AABBs it swept, its axis and pairs."""
    import orc
    o = orc.OracleWorld(scene, 32)
    axis = o.axis
    o.integrate()
    o.broadphase()
    st = o.state()
    return st["aabb_min"], st["aabb_max"], axis, o.pairs()


def test_noalloc_matches_oracle_at_the_size_limit_with_ignored_bodies():
    rt = _cudart()
    lib = pg.load()
    scene = sc.random_cube(n=16384, seed=77, extent=28.0, real_bits=32)
    rng = np.random.default_rng(5)
    scene.body_flags = scene.body_flags.copy()
    scene.body_flags[rng.choice(16384, 700, replace=False)] |= sc.IGNORE_COLLISION
    mn, mx, axis, ref = _oracle_sweep(scene)
    assert len(ref) > 2000
    # the oracle's pair list is the reference's (random positions: no tied sort keys)
    count, got = _noalloc_pairs(lib, rt, mn, mx, scene.body_flags, axis, cap=len(ref) + 16)
    assert count == len(ref)
    np.testing.assert_array_equal(got, ref)
    ign = set(np.flatnonzero(scene.body_flags & sc.IGNORE_COLLISION).tolist())
    assert not (set(got.ravel().tolist()) & ign)
    # the same bodies with no flags array: every body dynamic, so the ignored bodies pair again
    count2, got2 = _noalloc_pairs(lib, rt, mn, mx, None, axis, cap=2 * count + 4096)
    plain = scene.body_flags & ~sc.IGNORE_COLLISION
    s2 = scene
    s2.body_flags = plain.astype(np.int32)
    _, _, _, ref2 = _oracle_sweep(s2)
    assert count2 == len(ref2) > count
    np.testing.assert_array_equal(got2, ref2)


def test_noalloc_small_inputs_and_a_stream_of_the_callers_own():
    rt = _cudart()
    lib = pg.load()
    for n in (0, 1):        # below two bodies: no pairs, *n_pairs written as 0
        mn = np.zeros((n, 3))
        count, got = _noalloc_pairs(lib, rt, mn, mn + 1.0, None, 0, cap=4)
        assert count == 0 and got.size == 0
    st = C.c_void_p()
    assert rt.cudaStreamCreate(C.byref(st)) == 0
    try:
        scene = sc.pile(500, seed=9, real_bits=32, hull_range=(8, 12), drop=(0.0, 0.3))
        mn, mx, axis, ref = _oracle_sweep(scene)
        count, got = _noalloc_pairs(lib, rt, mn, mx, scene.body_flags, axis, cap=len(ref) + 8, stream=st)
        assert count == len(ref) > 50
        assert {tuple(sorted(p)) for p in got.tolist()} == {tuple(sorted(p)) for p in ref.tolist()}
    finally:
        rt.cudaStreamDestroy(st)


def test_noalloc_rejects_misaligned_pointers():
    rt = _cudart()
    lib = pg.load()
    err = C.create_string_buffer(256)
    d = Dev(rt, 4096)
    base = d.p.value
    # pairs 4 bytes past an 8-byte boundary: refused on the host, no device work queued
    rc = lib.pe_gpu_sap_pairs_noalloc(0, 10, C.c_void_p(base), C.c_void_p(base + 256), None, 0, C.c_void_p(base + 1028), 8,
                                      C.c_void_p(base + 2048), None, err, 256)
    assert rc == -1 and b"misaligned" in err.value
    rc = lib.pe_gpu_sap_pairs_noalloc(0, 10, C.c_void_p(base + 2), C.c_void_p(base + 256), None, 0, C.c_void_p(base + 1024), 8,
                                      C.c_void_p(base + 2048), None, err, 256)
    assert rc == -1 and b"misaligned" in err.value
    d.free()
