"""The reference-side binding (include/pe_gpu_adapters.h) compiled against the reference engine's own
headers and linked with its own engine sources and with libpe_gpu.so, where the reference tree is
present (oracle/build_ref.py's reference_dir()).

tests/adapters_check.cpp installs GpuBroadPhase, GpuNarrowPhase and GpuSequentialImpulseSolver in a
pe_intf::World (World::setBroadPhase / setNarrowPhase / setConstraintSolver, src/intf/world.h:97-99)
and runs the unchanged World::step, then the fused GpuStepper.  Without a usable CUDA device every
path must surface the library's PE_GPU_ERR_CUDA as the adapters' exception; with one, both paths
step.  The adapter code quoted in INTEGRATION.md is checked to be this header."""
import re
import subprocess
from pathlib import Path

import pytest

import build_ref
import pe_gb300 as pg

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "pe_gpu_adapters.h"


def _cuda_device_present():
    try:
        from pe_gb300 import scene as sc
        pg.GpuWorld(sc.pair_zoo(0, 0, m=1, real_bits=32), 32).close()
        return True
    except pg.PeGpuError:
        return False


def test_integration_doc_quotes_the_compiled_header():
    doc = (ROOT / "INTEGRATION.md").read_text()
    blocks = re.findall(r"```cpp\n(.*?)```", doc, flags=re.S)
    quoted = [b for b in blocks if "namespace pe_gpu_adapter" in b]
    assert len(quoted) == 1, "INTEGRATION.md quotes the adapter header once"
    assert quoted[0] == HEADER.read_text()


def test_adapters_compile_link_and_surface_device_errors(tmp_path):
    ref = build_ref.reference_dir()
    if ref is None:
        pytest.skip("reference sources not present")
    build_ref.build(ref, 8, bits_list=(64,), margins=(False,))
    pg.load()   # builds libpe_gpu.so if missing
    libdir = pg.LIB_PATH.parent
    obj = tmp_path / "adapters_check.o"
    exe = tmp_path / "adapters_check"
    cc = ["g++", *[f for f in build_ref.flags(ref, 64) if f != "-w"], "-Wall", f"-I{ROOT / 'include'}", "-c",
          str(ROOT / "tests" / "adapters_check.cpp"), "-o", str(obj)]
    r = subprocess.run(cc, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    own = [l for l in r.stderr.splitlines() if re.search(r"(pe_gpu_adapters\.h|adapters_check\.cpp):\d+:\d+: warning", l)]
    assert not own, "\n".join(own)   # the reference's own headers warn under -Wall; the binding does not
    ld = ["g++", "-O2", "-o", str(exe), str(obj), *build_ref.engine_objects(64), f"-L{libdir}", "-lpe_gpu",
          f"-Wl,-rpath,{libdir}", "-lpthread"]
    r = subprocess.run(ld, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = {l.split()[0]: l for l in r.stdout.splitlines() if l.split() and l.split()[0] in ("phases", "stepper")}
    assert set(lines) == {"phases", "stepper"}, r.stdout
    if _cuda_device_present():
        assert all(l.endswith(" ok") for l in lines.values()), r.stdout
    else:
        for l in lines.values():
            assert l.split()[1:3] == ["error", str(-2)], l   # PE_GPU_ERR_CUDA, raised by World::step
