"""Build the oracle library ``oracle/_build/liboracle.so`` (test infrastructure only).

The oracle is a plain C++ restatement of the reference's step; it is compiled with
-ffp-contract=off so that it gives the same bits on x86-64 and on aarch64 (where the
compiler would otherwise fuse multiply-adds).  Used by the tests, by smoke() and by
bench.py's CPU-baseline leg only.
"""
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build"
SRC = [HERE / "orc_capi.cpp"]
DEPS = [HERE / f for f in ("orc_math.h", "orc_shapes.h", "orc_collide.h", "orc_world.h")]


def lib_path() -> Path:
    return OUT / "liboracle.so"


def build(force: bool = False) -> Path:
    OUT.mkdir(exist_ok=True)
    so = lib_path()
    newest = max(p.stat().st_mtime for p in SRC + DEPS)
    if so.exists() and so.stat().st_mtime >= newest and not force:
        return so
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           "-pthread", "-o", str(so)] + [str(s) for s in SRC]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stderr)
        raise RuntimeError("oracle build failed")
    return so


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
