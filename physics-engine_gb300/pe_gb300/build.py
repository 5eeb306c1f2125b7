"""Build of the GB300 step library ``physics-engine_gb300/lib/libpe_gpu.so`` (in-tree).

Every translation unit is compiled for sm_103a only.  Device code is compiled without
FMA contraction and with IEEE division / square root so that the kernels reproduce the
reference's arithmetic bit for bit; host code is compiled with -ffp-contract=off for the
same reason (aarch64 compilers contract by default).
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent.parent
CSRC = PKG / "csrc"
OUT = PKG / "lib"
OBJ = PKG / "_build"
LIB = OUT / "libpe_gpu.so"

CU_SOURCES = ["pe_util.cu", "pe_world_f32.cu", "pe_world_f64.cu", "pe_capi.cu", "pe_noalloc.cu", "pe_server.cu"]
CPP_SOURCES = ["pe_host_shapes.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "--fmad=false", "-prec-div=true", "-prec-sqrt=true",
                     "-ftz=false", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
                     "-Xptxas", "-warn-spills", "--expt-relaxed-constexpr"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math"]


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(p).exists():
        raise RuntimeError("nvcc not found")
    return p


def _deps():
    return list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + [PKG.parent / "include" / "pe_gpu.h"]


def build(force: bool = False, verbose: bool = False, jobs: int = 0) -> Path:
    OUT.mkdir(exist_ok=True)
    OBJ.mkdir(exist_ok=True)
    dep_time = max(p.stat().st_mtime for p in _deps())
    jobs_list = []
    for s in CU_SOURCES + CPP_SOURCES:
        src = CSRC / s
        obj = OBJ / (s + ".o")
        stale = force or not obj.exists() or obj.stat().st_mtime < max(src.stat().st_mtime, dep_time)
        if s.endswith(".cu"):
            cmd = [nvcc(), *NVCC_FLAGS, "-I", str(CSRC), "-c", str(src), "-o", str(obj)]
        else:
            cmd = ["g++", *CXX_FLAGS, "-I", str(CSRC), "-I", "/usr/local/cuda/include", "-c", str(src), "-o", str(obj)]
        jobs_list.append((cmd if stale else None, obj))

    def run(cmd):
        if cmd is None:
            return 0, ""
        r = subprocess.run(cmd, capture_output=True, text=True)
        return r.returncode, r.stdout + r.stderr

    with cf.ThreadPoolExecutor(jobs or min(len(jobs_list), os.cpu_count() or 4)) as ex:
        for (cmd, obj), (rc, out) in zip(jobs_list, ex.map(lambda j: run(j[0]), jobs_list)):
            if verbose and out:
                sys.stderr.write(out)
            if rc != 0:
                sys.stderr.write(out)
                raise RuntimeError(f"compile failed: {' '.join(cmd)}")
    objs = [str(o) for _, o in jobs_list]
    if force or not LIB.exists() or LIB.stat().st_mtime < max(Path(o).stat().st_mtime for o in objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(LIB), *objs, "-lcudart", "-Xlinker", "--no-undefined"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link failed")
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
