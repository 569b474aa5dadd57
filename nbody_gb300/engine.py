"""Host-side mirror of the reference's engine interface over the C ABI.

`NbodyEngineGB300` has the method set of `nbody_engine`
(nbody/nbody_engine.h:16-96) with the same argument meaning, so solver code
written against the reference interface drives it unchanged, and
`create_engine(params)` mirrors `nbody_create_engine` (nbody/nbody_engines.cpp:4)
for the new alias "gb300": it returns None for invalid parameters.

Negative branches keep the reference's behaviour: a buffer that is not this
engine's memory, a NULL coefficient array or a size mismatch is logged and the
call returns without side effects (test/engine/test_nbody_engine.cpp:761-1010).
CUDA failures, which make the reference exit(3), raise NbgError instead.
"""
from __future__ import annotations

import ctypes as C
import logging
from typing import Optional, Sequence

import numpy as np

from . import _lib
from ._lib import NbgError, Params

log = logging.getLogger("nbody_gb300")

# statuses the reference answers with a log line and a plain return
_SOFT = {1, 2, 3}


class Memory:
    """nbody_engine::memory -- a device buffer owned by one engine."""

    __slots__ = ("_h", "_engine", "_size", "__weakref__")

    def __init__(self, handle: int, engine: "NbodyEngineGB300", size: int):
        self._h = handle
        self._engine = engine
        self._size = size

    def size(self) -> int:
        """Memory size in bytes (nbody/nbody_engine.h:27)."""
        return self._size

    @property
    def handle(self) -> int:
        return self._h

    def device_ptr(self) -> int:
        return int(_lib.load().nbg_buffer_device_ptr(self._h) or 0)


class HostBuffer:
    """Page-locked host memory viewed as a float64 numpy array."""

    def __init__(self, count: int):
        lib = _lib.load()
        p = C.c_void_p()
        st = lib.nbg_host_alloc(count * 8, C.byref(p))
        if st != 0:
            raise NbgError(st, "nbg_host_alloc failed")
        self._p = p.value
        self.array = np.ctypeslib.as_array(C.cast(p, C.POINTER(C.c_double)), shape=(count,))

    def free(self) -> None:
        if self._p:
            _lib.load().nbg_host_free(self._p)
            self._p = None
            self.array = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def _params_from(param: dict) -> Optional[Params]:
    """QVariantMap keys -> nbg_params (None when a key has an invalid value)."""
    lib = _lib.load()
    p = Params()
    lib.nbg_params_default(C.byref(p))
    try:
        p.device = int(str(param.get("device", "0")))
        algo = str(param.get("algo", "direct"))
        prec = str(param.get("precision", "fp64"))
        layout = str(param.get("tree_layout", "heap_stackless"))
        trav = str(param.get("traverse_type", "nested_tree"))
        if algo not in _lib.ALGO or prec not in _lib.PRECISION:
            return None
        if layout not in _lib.LAYOUT or trav not in _lib.TRAVERSE:
            return None
        p.algo = _lib.ALGO[algo]
        p.precision = _lib.PRECISION[prec]
        p.tree_layout = _lib.LAYOUT[layout]
        p.traverse_type = _lib.TRAVERSE[trav]
        p.softening = float(param.get("softening", 0.0))
        p.distance_to_node_radius_ratio = float(param.get("distance_to_node_radius_ratio", 10.0))
        p.tree_build_rate = int(param.get("tree_build_rate", 0))
        p.learned = 1 if bool(param.get("learned", False)) else 0
        p.block_size = int(param.get("block_size", 0))
        p.learned_tight_ratio = float(param.get("learned_tight_ratio", 2.0))
    except (TypeError, ValueError):
        return None
    return p


def create_engine(param: dict) -> Optional["NbodyEngineGB300"]:
    """nbody_create_engine for engine == "gb300"; None on invalid params."""
    if str(param.get("engine", "")) != "gb300":
        return None
    p = _params_from(param)
    if p is None:
        return None
    # engine keys that map to tuning knobs of the library
    tune = {}
    try:
        if "tree_refit_within_step" in param:
            tune["bh.refit_within_step"] = int(bool(param["tree_refit_within_step"]))
        if "tree_freeze_within_step" in param:
            tune["bh.freeze_within_step"] = int(bool(param["tree_freeze_within_step"]))
        if "learned_judge" in param:
            tune["learned.judge"] = int(bool(param["learned_judge"]))
        if "learned_judge_samples" in param:
            tune["learned.judge_samples"] = int(param["learned_judge_samples"])
            if tune["learned.judge_samples"] < 1:
                return None
    except (TypeError, ValueError):
        return None
    try:
        e = NbodyEngineGB300(p)
    except NbgError as err:
        log.warning("gb300 engine not created: %s", err)
        return None
    for k, v in tune.items():
        e.tune_set(k, v)
    return e


class NbodyEngineGB300:
    """The GB300 engine behind the nbody_engine interface."""

    def __init__(self, params: Params):
        self._lib = _lib.load()
        h = C.c_void_p()
        st = self._lib.nbg_engine_create(C.byref(params), C.byref(h))
        if st != 0:
            raise NbgError(st, "nbg_engine_create failed")
        self._h = h.value
        self._params = params
        self._data = None
        self._y: Optional[Memory] = None
        self._compute_count = 0
        self.last_status = 0

    # -- lifetime ------------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.nbg_engine_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- status handling -------------------------------------------------------
    def _check(self, st: int, what: str) -> bool:
        self.last_status = st
        if st == 0:
            return True
        msg = self._lib.nbg_last_error(self._h).decode(errors="replace")
        if st in _SOFT:
            log.warning("%s: %s", what, msg)
            return False
        raise NbgError(st, f"{what}: {msg}")

    def _mem(self, m, name: str) -> Optional[int]:
        if isinstance(m, Memory) and m._engine is self and m._h is not None:
            return m._h
        log.warning("%s is not gb300 memory", name)
        self.last_status = 2
        return None

    # -- nbody_engine interface --------------------------------------------------
    def type_name(self) -> str:
        return self._lib.nbg_type_name(self._h).decode()

    def init(self, data) -> bool:
        """Upload bodies (nbody/nbody_engine.h:43)."""
        self._data = data
        n = data.get_count()
        v = np.ascontiguousarray(data.vertices, dtype=np.float64)
        u = np.ascontiguousarray(data.velocities, dtype=np.float64)
        m = np.ascontiguousarray(data.mass, dtype=np.float64)
        st = self._lib.nbg_init(self._h, n, v.ctypes.data, u.ctypes.data, m.ctypes.data)
        self.last_status = st
        if st != 0:
            log.warning("init: %s", self._lib.nbg_last_error(self._h).decode())
            return False
        yh = self._lib.nbg_get_y(self._h)
        self._y = Memory(yh, self, self._lib.nbg_buffer_size(yh))
        return True

    def get_data(self, data) -> None:
        n = data.get_count()
        v = np.empty((n, 3))
        u = np.empty((n, 3))
        self._check(self._lib.nbg_get_data(self._h, v.ctypes.data, u.ctypes.data), "get_data")
        data.vertices = v
        data.velocities = u

    def problem_size(self) -> int:
        return int(self._lib.nbg_problem_size(self._h))

    def get_y(self) -> Memory:
        return self._y

    def advise_time(self, dt: float) -> None:
        self._data.advise_time(dt)

    def get_time(self) -> float:
        return self._data.get_time()

    def set_time(self, t: float) -> None:
        self._data.set_time(t)

    def get_step(self) -> int:
        return self._data.get_step()

    def set_step(self, s: int) -> None:
        self._data.set_step(s)

    def fcompute(self, t: float, y: Memory, f: Memory) -> None:
        hy = self._mem(y, "y")
        hf = self._mem(f, "f")
        if hy is None or hf is None:
            return
        step = self._data.get_step() if self._data is not None else 0
        if self._check(self._lib.nbg_fcompute(self._h, t, step, hy, hf), "fcompute"):
            self._compute_count += 1

    def clamp(self, y: Memory, b: float) -> None:
        hy = self._mem(y, "y")
        if hy is not None:
            self._check(self._lib.nbg_clamp(self._h, hy, b), "clamp")

    def create_buffer(self, size: int) -> Optional[Memory]:
        h = C.c_void_p()
        st = self._lib.nbg_create_buffer(self._h, int(size), C.byref(h))
        self.last_status = st
        if st != 0:
            return None
        return Memory(h.value, self, int(size))

    def free_buffer(self, m) -> None:
        if m is None:
            return
        hm = self._mem(m, "buffer")
        if hm is None:
            return
        if self._check(self._lib.nbg_free_buffer(self._h, hm), "free_buffer"):
            m._h = None

    def create_buffers(self, size: int, count: int) -> list:
        """nbody/nbody_engine.cpp:21-36: all or nothing."""
        out = []
        for _ in range(count):
            m = self.create_buffer(size)
            if m is None:
                self.free_buffers(out)
                return []
            out.append(m)
        return out

    def free_buffers(self, mema: list) -> None:
        for m in mema:
            self.free_buffer(m)
        mema.clear()

    def read_buffer(self, dst: np.ndarray, src: Memory) -> None:
        hs = self._mem(src, "src")
        if hs is None:
            return
        if dst is None or not dst.flags.c_contiguous or dst.nbytes < src.size():
            log.warning("read_buffer: destination smaller than the buffer")
            self.last_status = 3
            return
        self._check(self._lib.nbg_read_buffer(self._h, dst.ctypes.data, hs), "read_buffer")

    def write_buffer(self, dst: Memory, src: np.ndarray) -> None:
        hd = self._mem(dst, "dst")
        if hd is None:
            return
        if src is None or not src.flags.c_contiguous or src.nbytes < dst.size():
            log.warning("write_buffer: source smaller than the buffer")
            self.last_status = 3
            return
        self._check(self._lib.nbg_write_buffer(self._h, hd, src.ctypes.data), "write_buffer")

    def copy_buffer(self, a: Memory, b: Memory) -> None:
        ha, hb = self._mem(a, "a"), self._mem(b, "b")
        if ha is not None and hb is not None:
            self._check(self._lib.nbg_copy_buffer(self._h, ha, hb), "copy_buffer")

    def fill_buffer(self, a: Memory, value: float) -> None:
        ha = self._mem(a, "a")
        if ha is not None:
            self._check(self._lib.nbg_fill_buffer(self._h, ha, float(value)), "fill_buffer")

    def fmadd_inplace(self, a: Memory, b: Memory, c: float) -> None:
        ha, hb = self._mem(a, "a"), self._mem(b, "b")
        if ha is not None and hb is not None:
            self._check(self._lib.nbg_fmadd_inplace(self._h, ha, hb, float(c)), "fmadd_inplace")

    def fmadd(self, a: Memory, b: Memory, c: Memory, d: float) -> None:
        ha, hb, hc = self._mem(a, "a"), self._mem(b, "b"), self._mem(c, "c")
        if ha is not None and hb is not None and hc is not None:
            self._check(self._lib.nbg_fmadd(self._h, ha, hb, hc, float(d)), "fmadd")

    def _arrays(self, mems: Sequence, coeff, count: int, name: str):
        """Handle array for the first `count` buffers (all must be ours) and
        the matching coefficient array."""
        for m in mems[:count]:
            if not (isinstance(m, Memory) and m._engine is self and m._h is not None):
                log.warning("%s is not gb300 memory", name)
                self.last_status = 2
                return None, None
        handles = [m._h if isinstance(m, Memory) and m._engine is self else 0 for m in mems]
        harr = (C.c_void_p * max(1, len(handles)))(*handles)
        carr = np.zeros(max(1, count))
        carr[:count] = np.asarray(coeff, dtype=np.float64)[:count]
        return harr, carr

    def fmaddn_inplace(self, a: Memory, b: Sequence, c, csize: int) -> None:
        if c is None:
            return  # nbody/nbody_engine.cpp:49-52
        ha = self._mem(a, "a")
        if ha is None:
            return
        if csize > len(b):
            log.warning("csize > b.size()")
            self.last_status = 1
            return
        harr, carr = self._arrays(b, c, csize, "b")
        if harr is None:
            return
        self._check(self._lib.nbg_fmaddn_inplace(
            self._h, ha, harr, len(b), carr.ctypes.data_as(C.POINTER(C.c_double)), csize),
            "fmaddn_inplace")

    def fmaddn_corr(self, a: Memory, corr: Memory, b: Sequence, c, csize: int) -> None:
        ha, hc = self._mem(a, "a"), self._mem(corr, "corr")
        if ha is None or hc is None:
            return
        if c is None:
            log.warning("c must not be nullptr")
            self.last_status = 1
            return
        if csize > len(b):
            log.warning("csize > b.size()")
            self.last_status = 1
            return
        harr, carr = self._arrays(b, c, csize, "b")
        if harr is None:
            return
        self._check(self._lib.nbg_fmaddn_corr(
            self._h, ha, hc, harr, len(b), carr.ctypes.data_as(C.POINTER(C.c_double)), csize),
            "fmaddn_corr")

    def fmaddn(self, a: Memory, b: Optional[Memory], c: Sequence, d, dsize: int) -> None:
        if d is None:
            log.warning("d == NULL")
            self.last_status = 1
            return
        ha = self._mem(a, "a")
        if ha is None:
            return
        hb = None
        if b is not None:
            hb = self._mem(b, "b")
            if hb is None:
                return
        if dsize > len(c):
            log.warning("dsize > c.size()")
            self.last_status = 1
            return
        harr, darr = self._arrays(c, d, dsize, "c")
        if harr is None:
            return
        self._check(self._lib.nbg_fmaddn(
            self._h, ha, hb, harr, len(c), darr.ctypes.data_as(C.POINTER(C.c_double)), dsize),
            "fmaddn")

    def fmaxabs(self, a: Memory) -> float:
        """nbody_engine::fmaxabs; returns the result instead of an out-parameter."""
        ha = self._mem(a, "a")
        if ha is None:
            return 0.0
        r = C.c_double(0.0)
        self._check(self._lib.nbg_fmaxabs(self._h, ha, C.byref(r)), "fmaxabs")
        return r.value

    def print_info(self) -> None:
        p = self._params
        log.info("\tengine: %s precision=%s softening=%g lambda=%g", self.type_name(),
                 "fp64" if p.precision == 0 else "mixed", p.softening,
                 p.distance_to_node_radius_ratio)

    def get_compute_count(self) -> int:
        return self._compute_count

    # -- measurement / extras ------------------------------------------------------
    def synchronize(self) -> None:
        self._check(self._lib.nbg_synchronize(self._h), "synchronize")

    def profile_enable(self, on: bool = True) -> None:
        self._check(self._lib.nbg_profile_enable(self._h, 1 if on else 0), "profile_enable")

    def profile_query(self, kernel_id: int):
        ms = C.c_double(0.0)
        n = C.c_uint64(0)
        self._check(self._lib.nbg_profile_query(self._h, kernel_id, C.byref(ms), C.byref(n)),
                    "profile_query")
        return ms.value, n.value

    def launch_count(self) -> int:
        return int(self._lib.nbg_launch_count(self._h))

    def measure_fp32_peak(self) -> float:
        r = C.c_double(0.0)
        self._check(self._lib.nbg_measure_fp32_peak(self._h, C.byref(r)), "measure_fp32_peak")
        return r.value

    def statistics(self, y: Optional[Memory] = None) -> np.ndarray:
        """P[3], L[3], KE, PE, mass centre[3], mass of state y (default: get_y()),
        FP64 on the GPU (nbody/nbody_data.cpp:57-145)."""
        hy = self._mem(y if y is not None else self._y, "y")
        out = np.zeros(12)
        if hy is not None:
            self._check(self._lib.nbg_statistics(self._h, hy,
                                                 out.ctypes.data_as(C.POINTER(C.c_double))),
                        "statistics")
        return out

    def bh_fallback_groups(self) -> int:
        """Groups handed to the per-body fallback walk since the last bh_counters."""
        g = C.c_uint64(0)
        self._check(self._lib.nbg_bh_fallback_groups(self._h, C.byref(g)), "bh_fallback_groups")
        return g.value

    def bh_stack_peak(self):
        """(deepest group-walk stack since the last bh_counters, capacity)."""
        p, c = C.c_uint64(0), C.c_uint64(0)
        self._check(self._lib.nbg_bh_stack_peak(self._h, C.byref(p), C.byref(c)), "bh_stack_peak")
        return p.value, c.value

    def bh_counters(self):
        """(node visits, interactions) of the mixed Barnes-Hut walk since the last call."""
        v = C.c_uint64(0)
        i = C.c_uint64(0)
        self._check(self._lib.nbg_bh_counters(self._h, C.byref(v), C.byref(i)), "bh_counters")
        return v.value, i.value

    # -- learned correction ---------------------------------------------------------
    def learn_param_count(self) -> int:
        return int(self._lib.nbg_learn_param_count())

    def learn_set_weights(self, w) -> None:
        w = np.ascontiguousarray(w, dtype=np.float32)
        self._check(self._lib.nbg_learn_set_weights(
            self._h, w.ctypes.data_as(C.POINTER(C.c_float)), w.size), "learn_set_weights")

    def learn_get_weights(self) -> np.ndarray:
        w = np.zeros(self.learn_param_count(), dtype=np.float32)
        self._check(self._lib.nbg_learn_get_weights(
            self._h, w.ctypes.data_as(C.POINTER(C.c_float)), w.size), "learn_get_weights")
        return w

    def learn_init_weights(self, seed: int = 1) -> None:
        self._check(self._lib.nbg_learn_init_weights(self._h, seed), "learn_init_weights")

    def learn_generate(self, max_samples: int, seed: int = 1, max_subtree_log2: int = 16) -> int:
        got = C.c_size_t(0)
        self._check(self._lib.nbg_learn_generate(self._h, max_samples, seed, max_subtree_log2,
                                                 C.byref(got)), "learn_generate")
        return got.value

    def learn_sample_count(self) -> int:
        return int(self._lib.nbg_learn_sample_count(self._h))

    def learn_read_samples(self, offset: int, count: int):
        x = np.zeros((count, 16), dtype=np.float32)
        t = np.zeros((count, 4), dtype=np.float32)
        m = np.zeros((count, 2), dtype=np.int32)
        fp = C.POINTER(C.c_float)
        self._check(self._lib.nbg_learn_read_samples(
            self._h, offset, count, x.ctypes.data_as(fp), t.ctypes.data_as(fp),
            m.ctypes.data_as(C.POINTER(C.c_int))), "learn_read_samples")
        return x, t, m

    def learn_clear_samples(self) -> None:
        self._check(self._lib.nbg_learn_clear_samples(self._h), "learn_clear_samples")

    def learn_train(self, epochs: int, batch: int = 16384, lr: float = 3e-3, seed: int = 1,
                    val_fraction: float = 0.1):
        tr = C.c_double(0.0)
        va = C.c_double(0.0)
        self._check(self._lib.nbg_learn_train(self._h, epochs, batch, lr, seed, val_fraction,
                                              C.byref(tr), C.byref(va)), "learn_train")
        return tr.value, va.value

    def learn_loss_grad(self, x, t):
        x = np.ascontiguousarray(x, dtype=np.float32)
        t = np.ascontiguousarray(t, dtype=np.float32)
        g = np.zeros(self.learn_param_count(), dtype=np.float32)
        loss = C.c_double(0.0)
        fp = C.POINTER(C.c_float)
        self._check(self._lib.nbg_learn_loss_grad(self._h, x.ctypes.data_as(fp),
                                                  t.ctypes.data_as(fp), x.shape[0],
                                                  C.byref(loss), g.ctypes.data_as(fp)),
                    "learn_loss_grad")
        return loss.value, g

    def learn_predict(self, x) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float32)
        out = np.zeros((x.shape[0], 3), dtype=np.float32)
        fp = C.POINTER(C.c_float)
        self._check(self._lib.nbg_learn_predict(self._h, x.ctypes.data_as(fp), x.shape[0],
                                                out.ctypes.data_as(fp)), "learn_predict")
        return out

    def learn_predict_tc(self, x) -> np.ndarray:
        """The network's outputs from the tcgen05 tensor-core inference."""
        x = np.ascontiguousarray(x, dtype=np.float32)
        out = np.zeros((x.shape[0], 3), dtype=np.float32)
        fp = C.POINTER(C.c_float)
        self._check(self._lib.nbg_learn_predict_tc(self._h, x.ctypes.data_as(fp), x.shape[0],
                                                   out.ctypes.data_as(fp)), "learn_predict_tc")
        return out

    def learn_tc_accumulators(self, x) -> np.ndarray:
        """[count, 144]: the tcgen05 forward pass's accumulators, D1 (columns
        0..63), D2 (64..127) and D3 (128..143), biases included."""
        x = np.ascontiguousarray(x, dtype=np.float32)
        out = np.zeros((x.shape[0], 144), dtype=np.float32)
        fp = C.POINTER(C.c_float)
        self._check(self._lib.nbg_learn_tc_accumulators(self._h, x.ctypes.data_as(fp), x.shape[0],
                                                        out.ctypes.data_as(fp)),
                    "learn_tc_accumulators")
        return out

    def learn_judge_stats(self) -> dict:
        """The learned path's judge (nbg_learn_judge_stats): the last judged
        step's p50 / p99 / RMS relative force errors of the learned and the
        plain walk on the sampled bodies, whether that step fell back, and
        the counts of judged and fallen-back steps."""
        out = np.zeros(_lib.JUDGE_STATS)
        self._check(self._lib.nbg_learn_judge_stats(
            self._h, out.ctypes.data_as(C.POINTER(C.c_double)), out.size), "learn_judge_stats")
        keys = ("step", "p50_learned", "p99_learned", "p50_plain", "p99_plain", "rms_learned",
                "rms_plain", "used_plain", "samples", "judged_steps", "fallback_steps")
        d = dict(zip(keys, out.tolist()))
        for k in ("step", "used_plain", "samples", "judged_steps", "fallback_steps"):
            d[k] = int(d[k])
        d["used_plain"] = bool(d["used_plain"])
        return d

    def learn_band_rows(self) -> int:
        """Network rows of the learned walk since the last bh_counters call
        (read it before bh_counters, which resets it)."""
        r = C.c_uint64(0)
        self._check(self._lib.nbg_learn_band_rows(self._h, C.byref(r)), "learn_band_rows")
        return r.value

    def tree_leaves(self) -> np.ndarray:
        n = self.problem_size() // 6
        out = np.zeros(n, dtype=np.int32)
        self._check(self._lib.nbg_tree_leaves(self._h, out.ctypes.data_as(C.POINTER(C.c_int))),
                    "tree_leaves")
        return out

    def tune_set(self, key: str, value: int) -> None:
        self._check(self._lib.nbg_tune_set(self._h, key.encode(), int(value)), "tune_set")

    def autotune(self, reps: int = 3) -> dict:
        """nbg_autotune: time every candidate configuration of the force path
        on the current state, keep the fastest; returns the JSON report."""
        import json
        buf = C.create_string_buffer(8192)
        self._check(self._lib.nbg_autotune(self._h, int(reps), buf, len(buf)), "autotune")
        return json.loads(buf.value.decode())

    def tune_variant(self) -> str:
        """Which force path this engine runs (part of the autotuner cache key)."""
        p = self._params
        algo = "bh" if p.algo == 1 else "direct"
        prec = "fp64" if p.precision == 0 else "mixed"
        order = self.tune_get("bh.order") if algo == "bh" else None
        return f"{algo}/{prec}/{'soft' if p.softening > 0 else 'clamp'}" + \
            ("/learned" if p.learned else "") + \
            ("/quadrupole" if order is not None and order >= 2 else "")

    @property
    def device(self) -> int:
        return int(self._params.device)

    def tune_get(self, key: str):
        v = C.c_int64(0)
        st = self._lib.nbg_tune_get(self._h, key.encode(), C.byref(v))
        return v.value if st == 0 else None

    @property
    def handle(self) -> int:
        return self._h
