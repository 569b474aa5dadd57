"""The reference-side adapter (nbody_gb300/adapter/nbody_engine_gb300.h, the
class a maintainer adds to drons/nbody) compiled against the reference's own
nbody/nbody_engine.h and linked with the reference's objects (oracle/_ref)
and libnbody_gb300.so; then run: without a GPU the factory branch must answer
NULL for invalid parameters and for an engine it cannot create.  Needs the
reference's sources (skips where they are absent)."""
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def test_adapter_compiles_links_and_answers(tmp_path):
    from oracle.ref_build import LIB, SHIM, build_ref, reference_root
    if build_ref() is None:
        pytest.skip("the reference's sources are not present on this host")
    from nbody_gb300 import build as nb_build
    gb = nb_build.build()
    exe = tmp_path / "check_adapter"
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Werror", "-Wno-unused-function",
           "-I", str(SHIM), "-I", str(reference_root() / "nbody"), "-I", str(ROOT / "include"),
           "-I", str(ROOT / "nbody_gb300" / "adapter"),
           str(ROOT / "tests" / "adapter" / "check_adapter.cpp"), "-o", str(exe),
           str(LIB), str(gb), "-fopenmp", f"-Wl,-rpath,{LIB.parent}:{gb.parent}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present: the no-GPU answers do not apply")
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    assert "adapter ok" in r.stdout
