"""The allocation-free direct sum, called through the C ABI, against the
engine's own mixed-precision fcompute.

nbg_direct_mixed_noalloc serves callers that may not allocate GPU memory (an
application that owns all device memory through its own arena, or a loop that
must not pay for an allocation and its device synchronisation); its scratch
is a fixed array inside the library.  This file is collected last so that a
run stopping at the first failure has already run every other test.  The
first call on a device may load the library's module (CUDA's lazy loading),
which allocates; test_noalloc_first_call_in_fresh_process makes that call
the process's first direct-sum call and checks that later calls leave the
free device memory unchanged.
"""
import ctypes as C

import numpy as np
import pytest

from nbody_gb300.data import NBodyData

pytestmark = pytest.mark.gpu

MAX_BODIES = 131072  # NBG_NOALLOC_MAX_BODIES in include/nbody_gb300.h
RTOL = 1e-12         # same kernel; only the order of FP64 atomic adds may differ


def _engine_reference(make_engine, d, eps):
    """f from the existing entry point: a mixed-precision engine's fcompute
    with the one-sided kernel."""
    n = d.get_count()
    e = make_engine(precision="mixed", softening=eps)
    e.tune_set("direct.symmetric", 0)  # the one-sided kernel the entry point runs
    assert e.init(d)
    f = e.create_buffer(8 * 6 * n)
    e.fcompute(0.0, e.get_y(), f)
    out = np.zeros(6 * n)
    e.read_buffer(out, f)
    return e, out


def _noalloc(gpulib, e, d, eps):
    """Run the allocation-free entry point on buffers the test owns."""
    n = d.get_count()
    y = e.create_buffer(8 * 6 * n)
    m = e.create_buffer(8 * n)
    f = e.create_buffer(8 * 6 * n)
    e.write_buffer(y, d.to_state())
    e.write_buffer(m, np.ascontiguousarray(d.mass, dtype=np.float64))
    e.fill_buffer(f, 1e10)  # poison: every element must be written
    e.synchronize()
    st = gpulib.nbg_direct_mixed_noalloc(y.device_ptr(), m.device_ptr(), f.device_ptr(),
                                         n, eps, gpulib.nbg_stream(e.handle))
    assert st == 0, gpulib.nbg_status_string(st)
    out = np.zeros(6 * n)
    e.read_buffer(out, f)
    return out


@pytest.mark.parametrize("eps", [1e-3, 0.0])
def test_noalloc_matches_fcompute_two_calls(make_engine, gpulib, eps):
    # Two calls in a row on different systems; the second is smaller, so any
    # stale scratch from the first call would show up in its result.
    for n, seed in ((5003, 1), (1200, 2)):
        d = NBodyData.plummer(n, seed=seed)
        e, f_ref = _engine_reference(make_engine, d, eps)
        f = _noalloc(gpulib, e, d, eps)
        assert np.array_equal(f[:3 * n], f_ref[:3 * n])
        a, a_ref = f[3 * n:], f_ref[3 * n:]
        assert np.all(np.isfinite(a))
        assert np.max(np.abs(a - a_ref)) <= RTOL * np.max(np.abs(a_ref))


def test_noalloc_rejects_oversize(make_engine, gpulib):
    d = NBodyData.uniform_cube(64, seed=3)
    e = make_engine(precision="mixed", softening=1e-3)
    assert e.init(d)
    big = MAX_BODIES + 1
    y = e.create_buffer(8 * 6 * 64)
    st = gpulib.nbg_direct_mixed_noalloc(y.device_ptr(), y.device_ptr(), y.device_ptr(),
                                         big, 1e-3, None)
    assert st == 10  # NBG_ERR_TOO_LARGE, nothing launched
    assert gpulib.nbg_status_string(st) == b"exceeds a fixed capacity"
    assert gpulib.nbg_direct_mixed_noalloc(None, None, None, 16, 1e-3, None) == 1


_FRESH = r"""
import ctypes as C, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
from nbody_gb300 import _lib
from nbody_gb300.data import NBodyData
from nbody_gb300.engine import create_engine
lib = _lib.load()
cudart = C.CDLL("libcudart.so.13")  # the runtime the library links (already loaded)
free, total = C.c_size_t(0), C.c_size_t(0)

def free_bytes():
    assert cudart.cudaMemGetInfo(C.byref(free), C.byref(total)) == 0
    return free.value

n, eps = 3000, 1e-3
d = NBodyData.plummer(n, seed=5)
e = create_engine({"engine": "gb300", "precision": "mixed", "softening": eps})
e.tune_set("direct.symmetric", 0)
assert e.init(d)
y, m, f = (e.create_buffer(8 * k) for k in (6 * n, n, 6 * n))
e.write_buffer(y, d.to_state())
e.write_buffer(m, np.ascontiguousarray(d.mass, dtype=np.float64))
e.synchronize()
outs = []
for call in range(3):
    before = free_bytes()
    st = lib.nbg_direct_mixed_noalloc(y.device_ptr(), m.device_ptr(), f.device_ptr(), n, eps,
                                      lib.nbg_stream(e.handle))
    assert st == 0, lib.nbg_status_string(st)
    after = free_bytes()
    if call > 0:  # the first call may load the module (the driver's own allocation)
        assert after == before, (call, before, after)
    out = np.zeros(6 * n)
    e.read_buffer(out, f)
    outs.append(out)
g = e.create_buffer(8 * 6 * n)  # only now does an engine direct kernel run
e.fcompute(0.0, e.get_y(), g)
ref = np.zeros(6 * n)
e.read_buffer(ref, g)
for out in outs:
    assert np.array_equal(out[:3 * n], ref[:3 * n])
    assert np.max(np.abs(out[3 * n:] - ref[3 * n:])) <= 1e-12 * np.max(np.abs(ref[3 * n:]))
e.close()
print("fresh ok")
"""


def test_noalloc_first_call_in_fresh_process(gpulib):
    """A process whose first direct-sum call on the GPU is the entry point
    itself: it does the per-device set-up, gives the engine's result, and
    later calls leave the free device memory unchanged."""
    import subprocess
    import sys
    from pathlib import Path
    root = str(Path(__file__).resolve().parent.parent)
    r = subprocess.run([sys.executable, "-c", _FRESH, root], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "fresh ok" in r.stdout

