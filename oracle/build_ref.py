"""Build recipe for the reference engine harness (test infrastructure only).

Compiles the reference's own engine sources where they lie (no copy into this
repository) together with ``oracle/ref_harness.cpp`` into ``oracle/_ref/``:

    oracle/_ref/ref_harness64   reference built with PE_USE_DOUBLE (its default, CMakeLists.txt:28)
    oracle/_ref/ref_harness32   reference built with pe::Real = float
    oracle/_ref/ref_harness64m  as ref_harness64, contact margin 0.005 instead of PE_MARGIN = 0
                                (phys_general.h:45), through the forced-include header ref_margin.h
    oracle/_ref/ref_harness32m  the same in FP32

Sources follow the reference's own target lists (src/CMakeLists.txt:4-11): the
PEngine library (intf/world.cpp, rigid/**, cloth/**) plus the four PEUtils
sources.  The viewer and its prebuilt GL binaries are never touched.  Flags follow
CMakeLists.txt:6-29 (-DPE_MULTI_THREAD, -DAMGCL_NO_BOOST, aligned storage on),
compiled with g++ -std=c++14 -O2 like the reference's default build.

Run:  python oracle/build_ref.py [--ref /path/to/reference] [--jobs N]
The reference tree is found by ``reference_dir()``: $PE_REFERENCE_DIR, else a directory named
``reference`` beside this repository.  Where neither holds the sources, nothing is built.
"""
import argparse
import concurrent.futures as cf
import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
OBJ = Path(os.environ.get("TMPDIR", "/tmp")) / "pe_ref_obj"   # objects stay outside the repository


def reference_dir():
    """The reference engine's source tree: $PE_REFERENCE_DIR, else ``reference`` beside this
    repository's root; None when neither holds the engine's sources."""
    env = os.environ.get("PE_REFERENCE_DIR")
    cands = ([Path(env)] if env else []) + [HERE.parent.parent / "reference"]
    for c in cands:
        if (c / "src" / "intf" / "world.cpp").exists():
            return c
    return None


def sources(ref: Path):
    src = ref / "src"
    files = [src / "intf" / "world.cpp"]
    for sub in ("rigid", "cloth"):
        files += sorted((src / sub).rglob("*.cpp"))
    for u in ("logger", "thread_pool", "bvh", "file_system"):
        files.append(src / "utils" / f"{u}.cpp")
    return files


MARGIN_VARIANT = 0.005   # the tower configuration's contact margin


def flags(ref: Path, bits: int, margin: bool = False):
    f = ["-std=c++14", "-O2", "-DPE_MULTI_THREAD", "-DAMGCL_NO_BOOST",
         "-D_ENABLE_EXTENDED_ALIGNED_STORAGE", f"-DPE_DATA_PATH=\"{ref}/data/\"",
         f"-I{ref / 'src'}", f"-I{ref / 'ThirdParty'}", f"-I{ref / 'SimpleViewer' / 'include'}",
         "-w"]
    if bits == 64:
        f.append("-DPE_USE_DOUBLE")
    if margin:
        f += ["-include", str(HERE / "ref_margin.h"), f"-DPE_MARGIN_VALUE={MARGIN_VARIANT!r}"]
    return f


def build(ref: Path, jobs: int, bits_list=(64, 32), margins=(False, True)):
    if not (ref / "src" / "intf" / "world.cpp").exists():
        print(f"reference sources not found under {ref}; skipping reference build")
        return False
    OUT.mkdir(exist_ok=True)
    for bits, margin in [(b, m) for m in margins for b in bits_list]:
        tag = f"{bits}{'m' if margin else ''}"
        obj_dir = OBJ / f"obj{tag}"
        obj_dir.mkdir(parents=True, exist_ok=True)
        fl = flags(ref, bits, margin)
        jobs_list = []
        for s in sources(ref) + [HERE / "ref_harness.cpp"]:
            rel = s.relative_to(ref) if str(s).startswith(str(ref)) else Path(s.name)
            o = obj_dir / (str(rel).replace(os.sep, "__") + ".o")
            newest = max(s.stat().st_mtime, (HERE / "ref_margin.h").stat().st_mtime if margin else 0)
            if o.exists() and o.stat().st_mtime >= newest:
                jobs_list.append((None, o))
                continue
            jobs_list.append((["g++", *fl, "-c", str(s), "-o", str(o)], o))

        def run(cmd):
            if cmd is None:
                return 0, ""
            r = subprocess.run(cmd, capture_output=True, text=True)
            return r.returncode, r.stderr

        with cf.ThreadPoolExecutor(jobs) as ex:
            for (cmd, o), (rc, err) in zip(jobs_list, ex.map(lambda j: run(j[0]), jobs_list)):
                if rc != 0:
                    sys.stderr.write(err)
                    raise SystemExit(f"compile failed: {cmd}")
        exe = OUT / f"ref_harness{tag}"
        cmd = ["g++", "-O2", "-o", str(exe)] + [str(o) for _, o in jobs_list] + ["-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stderr)
            raise SystemExit("link failed")
        print(f"built {exe}")
    return True


def engine_objects(bits=64, margin=False):
    """Object files of the reference engine (PEngine + the four PEUtils sources) from the last
    build() of that variant, without the harness: for linking other drivers against it."""
    obj_dir = OBJ / f"obj{bits}{'m' if margin else ''}"
    return sorted(str(o) for o in obj_dir.glob("*.o") if o.name != "ref_harness.cpp.o")


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=None, help="reference source tree (default: reference_dir())")
    ap.add_argument("--jobs", type=int, default=os.cpu_count() or 4)
    a = ap.parse_args()
    ref = Path(a.ref) if a.ref else reference_dir()
    if ref is None:
        raise SystemExit("reference sources not found: set PE_REFERENCE_DIR or pass --ref")
    build(ref, a.jobs)
