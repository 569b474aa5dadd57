"""CPU checks of the C ABI: the library builds, loads without a GPU and
exports every function include/nbody_gb300.h declares; host-side parameter
mapping follows nbody_create_engine (no compute calls here)."""
import re

import pytest

from conftest import ROOT


def _declared():
    text = (ROOT / "include" / "nbody_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(nbg_[a-z0-9_]+)\s*\(", text)))


def test_header_lists_match(gpulib):
    from nbody_gb300 import _lib
    declared = _declared()
    assert declared, "no declarations parsed"
    missing = [n for n in declared if not hasattr(gpulib, n)]
    assert not missing, f"declared but not exported: {missing}"
    assert set(declared) <= set(_lib.EXPORTS) | set(declared)
    assert set(_lib.EXPORTS) <= set(declared), set(_lib.EXPORTS) - set(declared)


@pytest.mark.parametrize("lang,std", [("c", "-std=c99"), ("c++", "-std=c++17")])
def test_header_compiles_standalone(lang, std):
    """The C ABI header is self-contained C and C++ (the reference-side adapter
    includes it from C++; a C or FFI host may include it from C)."""
    import shutil
    import subprocess
    cc = shutil.which("gcc" if lang == "c" else "g++")
    if cc is None:
        pytest.skip("no host compiler")
    r = subprocess.run([cc, std, "-Wall", "-Wextra", "-Werror", "-fsyntax-only", "-x", lang,
                        str(ROOT / "include" / "nbody_gb300.h")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_ctypes_prototypes_match_header():
    """Every ctypes prototype in nbody_gb300/_lib.py takes as many arguments
    as the header declares for that function."""
    import ast
    text = (ROOT / "include" / "nbody_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    declared = {}
    for m in re.finditer(r"\b(nbg_[a-z0-9_]+)\s*\(([^;{]*?)\)\s*;", text, flags=re.S):
        params = m.group(2).strip()
        declared[m.group(1)] = 0 if params in ("", "void") else params.count(",") + 1
    tree = ast.parse((ROOT / "nbody_gb300" / "_lib.py").read_text())
    proto = {node.args[1].value: len(node.args) - 3 for node in ast.walk(tree)
             if isinstance(node, ast.Call) and getattr(node.func, "id", None) == "_proto"}
    assert set(proto) == set(declared), set(proto) ^ set(declared)
    wrong = {k: (declared[k], v) for k, v in proto.items() if declared[k] != v}
    assert not wrong, f"argument counts (header, ctypes) differ: {wrong}"


def test_tuning_keys_documented():
    """Every tuning key the library reads is documented in the header."""
    used = set()
    for src in (ROOT / "nbody_gb300" / "csrc").glob("*.cu"):
        used |= set(re.findall(r'tune_get\("([a-z0-9_.]+)"', src.read_text()))
    assert {"bh.walk", "direct.symmetric", "ensemble.unroll"} <= used
    header = (ROOT / "include" / "nbody_gb300.h").read_text()
    missing = sorted(k for k in used if f'"{k}"' not in header)
    assert not missing, f"tuning keys read but not documented: {missing}"


def test_status_strings_and_version(gpulib):
    assert gpulib.nbg_abi_version() == 1
    assert gpulib.nbg_status_string(0) == b"ok"
    assert gpulib.nbg_status_string(2) == b"foreign buffer"


def test_params_default(gpulib):
    import ctypes as C
    from nbody_gb300._lib import Params
    p = Params()
    gpulib.nbg_params_default(C.byref(p))
    assert p.struct_size == C.sizeof(Params)
    assert p.distance_to_node_radius_ratio == 10.0
    assert p.tree_layout == 2 and p.traverse_type == 1


def test_null_handles_are_rejected_without_gpu(gpulib):
    import ctypes as C
    # every entry point checks its engine handle before touching CUDA
    assert gpulib.nbg_fcompute(None, 0.0, 0, None, None) == 1
    assert gpulib.nbg_fill_buffer(None, None, 1.0) == 1
    r = C.c_double(0)
    assert gpulib.nbg_fmaxabs(None, None, C.byref(r)) == 1
    assert gpulib.nbg_problem_size(None) == 0
    assert gpulib.nbg_buffer_size(None) == 0


@pytest.mark.parametrize("param", [
    {"engine": "invalid"},
    {"engine": "gb300", "algo": "octree"},
    {"engine": "gb300", "precision": "fp16"},
    {"engine": "gb300", "tree_layout": "tree"},
    {"engine": "gb300", "traverse_type": "infinite"},
    {"engine": "gb300", "device": "a"},
    {"engine": "gb300", "distance_to_node_radius_ratio": "x"},
])
def test_invalid_params_give_none(gpulib, param):
    from nbody_gb300.engine import create_engine
    assert create_engine(param) is None


def test_solver_factory():
    from nbody_gb300.solvers import create_solver, SolverRKButcher
    assert create_solver({"solver": "invalid"}) is None
    s = create_solver({"solver": "rkdp", "error_threshold": 1e-6, "max_step": 0.5})
    assert isinstance(s, SolverRKButcher) and s.error_threshold == 1e-6 and s.max_step == 0.5
    for name, tb in (("rkdp", 7), ("rkck", 6), ("rkf", 13)):
        t = create_solver({"solver": name}).bt
        assert t.steps == tb
        # butcher_table_check (test/solver/test_nbody_solver.cpp:87-144)
        assert abs(sum(t.b1) - 1) < 1e-14 and abs(sum(t.b2) - 1) < 1e-14
        for i in range(t.steps):
            assert abs(sum(t.a[i][:i]) - t.c[i]) < 1e-13 * max(1, max(map(abs, t.a[i][:i] or [1])))
