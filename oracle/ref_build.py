"""Build recipe of oracle/_ref/libnbody_ref.so: the reference's own CPU code.

TEST INFRASTRUCTURE ONLY.  Compiles the reference's sources unchanged, where
they lie (nbody/*.cpp of the reference checkout, all but the CUDA and OpenCL
engines), against the Qt-API shim in oracle/qtshim, plus the C-ABI glue
oracle/ref_glue.cpp, with g++ (no qmake, no Qt), into oracle/_ref/.  The
tests use it to check the oracle restatement and the committed fixtures
against what the reference itself computes.  Nothing here is copied: the
sources are read in place.  Without a reference checkout (the GPU host) the
build is skipped and those tests skip.

    python -m oracle.ref_build [--force] [reference_root]

The reference root comes from the argument, else NBODY_REFERENCE, else
/root/reference.  Flags: -O2 -ffp-contract=off (no fused multiply-add, so the
results are those of the C++ source's operation order; the oracle
restatement is compiled the same way), -fopenmp.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
LIB = OUT / "libnbody_ref.so"
SHIM = HERE / "qtshim"
GLUE = HERE / "ref_glue.cpp"
FLAGS = ["-std=c++17", "-O2", "-fPIC", "-fopenmp", "-ffp-contract=off", "-w"]


def reference_root(arg: str = "") -> Path:
    return Path(arg or os.environ.get("NBODY_REFERENCE", "/root/reference"))


def sources(root: Path):
    src = root / "nbody"
    return sorted(p for p in src.glob("*.cpp")
                  if "cuda" not in p.name and "opencl" not in p.name)


def build_ref(root: str = "", force: bool = False):
    """Compile the reference's CPU sources + glue; returns the library path, or
    None when the reference's sources are not present."""
    ref = reference_root(root)
    srcs = sources(ref)
    if not srcs:
        return None
    (OUT / "obj").mkdir(parents=True, exist_ok=True)
    deps = [GLUE] + sorted(SHIM.rglob("*"))

    def newest(paths):
        return max(p.stat().st_mtime for p in paths if p.is_file())

    dep_time = newest(deps)

    def compile_one(src: Path) -> Path:
        obj = OUT / "obj" / (src.stem + ".o")
        if force or not obj.exists() or obj.stat().st_mtime < max(src.stat().st_mtime, dep_time):
            cmd = ["g++", *FLAGS, "-I", str(SHIM), "-I", str(ref / "nbody"), "-c", str(src),
                   "-o", str(obj)]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"g++ failed on {src.name}:\n{r.stderr[-4000:]}")
        return obj

    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        objs = list(ex.map(compile_one, srcs + [GLUE]))
    if force or not LIB.exists() or LIB.stat().st_mtime < newest(objs):
        tmp = LIB.with_name(LIB.name + f".tmp{os.getpid()}")
        cmd = ["g++", "-shared", "-fopenmp", "-o", str(tmp), *map(str, objs),
               "-Wl,--no-undefined"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr[-4000:]}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    print(build_ref(args[0] if args else "", force="--force" in sys.argv))
