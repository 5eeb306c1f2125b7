"""CPU checks of the C ABI library: it builds for sm_103a, loads, and exports every entry
point include/pe_gpu.h declares (no device calls)."""
import ctypes
import re

import pe_gb300 as pg


def declared_functions():
    text = pg.HEADER.read_text()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(pe_gpu_\w+)\s*\(", text, re.M)))


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(str(pg.load().__dict__.get("_name", pg.LIB_PATH)))
    names = declared_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_create_rejects_bad_config_without_touching_a_device():
    lib = pg.load()
    h = ctypes.c_void_p()
    cfg = pg._Config(48, 0)
    assert lib.pe_gpu_create(ctypes.byref(cfg), ctypes.byref(h)) == -1
    assert lib.pe_gpu_step(None, 1, 0) == -1
    assert lib.pe_gpu_n_bodies(None) == -1
