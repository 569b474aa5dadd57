"""Frame stream writer (nbody/nbody_data_stream.cpp) through the C ABI.

CPU: files written from host frames are byte-identical to the oracle's
restatement of the reference writer (index, parts with rollover, colours,
masses); the reference's negative branches (test/stream/test_nbody_stream.cpp:
129-200) and appending to an existing stream.  GPU: the reference's stream
test (the same file, :64-127) driven by the GB300 engine with frames taken
from device memory, byte-identical to frames taken through get_data, and the
time per step with a frame after every step on both paths.
"""
import filecmp
import os
import time

import numpy as np
import pytest

from nbody_gb300.data import NBodyData
from nbody_gb300.stream import DataStream, StreamReader
from oracle.stream_oracle import OracleStream


def _frames(d, count, seed=0):
    rng = np.random.default_rng(seed)
    n = d.get_count()
    out = []
    for k in range(count):
        out.append((k, 0.1 * k, rng.normal(size=(n, 3)), rng.normal(size=(n, 3))))
    return out


def _same_tree(a, b):
    fa, fb = sorted(os.listdir(a)), sorted(os.listdir(b))
    assert fa == fb, (fa, fb)
    for name in fa:
        assert filecmp.cmp(os.path.join(a, name), os.path.join(b, name), shallow=False), name


def test_host_frames_match_oracle(tmp_path):
    d = NBodyData.make_universe(128, 100, 100, 100)  # 256 bodies, 12288 B per frame
    assert d.get_count() == 256 and d.box_size == 100
    frames = _frames(d, 5)
    s = DataStream()
    assert s.open(str(tmp_path / "gb/new"), 14000) == 0
    for step, t, v, u in frames:
        d.vertices, d.velocities = v, u
        d.set_step(step)
        d.set_time(t)
        assert s.write(d) == 0
    assert s.close() == 0
    o = OracleStream(str(tmp_path / "ref/new"), 14000)
    for step, t, v, u in frames:
        o.write(step, t, v, u, d.box_size, d.get_color(), d.mass)
    o.close()
    _same_tree(tmp_path / "gb", tmp_path / "ref")
    # two frames per part, as the reference's test expects of 14000-byte parts
    assert sorted(os.listdir(tmp_path / "gb")) == ["new.col", "new.idx", "new.mass", "new0.dat",
                                                   "new1.dat", "new2.dat"]
    lines = (tmp_path / "gb/new.idx").read_text().split("\n")
    assert lines[:3] == ["#coord_size 8", "#body_count 256", "#box_size 100"]
    assert [ln for ln in lines if ln] == [ln for ln in lines if ln][:8]
    r = StreamReader()
    assert r.load(str(tmp_path / "gb/new")) == 0
    assert r.get_frame_count() == 5 and r.get_steps_count() == 4 and r.get_max_time() == 0.4
    assert r.get_body_count() == 256 and r.get_coord_size() == 8
    assert r.seek(77) != 0 and r.seek(3) == 0
    e = NBodyData()
    assert r.read(e) == 0
    assert np.array_equal(e.vertices, frames[3][2]) and np.array_equal(e.velocities, frames[3][3])
    assert e.get_step() == 3 and e.get_time() == 0.3


def test_append_continues_the_stream(tmp_path):
    d = NBodyData.make_universe(64, 10, 10, 10)
    frames = _frames(d, 6, seed=1)
    base = str(tmp_path / "gb/s")
    s = DataStream()
    assert s.open(base, 20000) == 0
    for step, t, v, u in frames[:3]:
        d.vertices, d.velocities, d.step, d.time = v, u, step, t
        assert s.write(d) == 0
    s.close()
    r = StreamReader()
    assert r.load(base) == 0
    s2 = DataStream()
    assert s2.open(base, 20000, append_to=r) == 0
    for step, t, v, u in frames[3:]:
        d.vertices, d.velocities, d.step, d.time = v, u, step, t
        assert s2.write(d) == 0
    s2.close()
    o = OracleStream(str(tmp_path / "ref/s"), 20000)
    for step, t, v, u in frames[:3]:
        o.write(step, t, v, u, d.box_size, d.get_color(), d.mass)
    o.close()
    o = OracleStream(str(tmp_path / "ref/s"), 20000, append_part=r.get_last_file_n())
    for step, t, v, u in frames[3:]:
        o.write(step, t, v, u, d.box_size, d.get_color(), d.mass)
    o.close()
    _same_tree(tmp_path / "gb", tmp_path / "ref")
    r2 = StreamReader()
    assert r2.load(base) == 0 and r2.get_frame_count() == 6


def test_negative_branches(tmp_path):
    d = NBodyData.make_universe(32, 1, 1, 1)
    s = DataStream()
    assert s.write(None) != 0
    assert s.write(d) != 0                                   # not open
    assert s.open("/dev/null/:nameless", 1000) != 0
    assert s.write(d) != 0
    s = DataStream()
    assert s.open(str(tmp_path / "00/stream"), 1000) == 0
    assert s.open(str(tmp_path / "01/stream"), 1000) == 0   # reopen elsewhere
    assert s.write(d) == 0
    s.close()
    os.makedirs(tmp_path / "0/stream0.dat")                  # part 0 cannot be a file
    assert DataStream().open(str(tmp_path / "0/stream"), 1) != 0
    os.makedirs(tmp_path / "1/stream.idx")                   # nor the index
    assert DataStream().open(str(tmp_path / "1/stream"), 1) != 0
    os.makedirs(tmp_path / "2/stream1.dat")                  # part 1 fails at the rollover
    s = DataStream()
    assert s.open(str(tmp_path / "2/stream"), 1) == 0
    assert s.write(d) == 0
    assert s.write(d) != 0
    s.close()
    assert StreamReader().load("/dev/null/:nameless") != 0


@pytest.mark.gpu
def test_reference_stream_run_on_gpu(make_engine, tmp_path):
    """test/stream/test_nbody_stream.cpp:64-127 with the GB300 engine (FP64)
    and frames taken from device memory; the same run with frames through
    get_data gives byte-identical files."""
    from nbody_gb300.solvers import create_solver

    def run(base, device_frames):
        d = NBodyData.make_universe(128, 100, 100, 100)
        e = make_engine(precision="fp64")
        assert e.init(d)
        s = create_solver({"solver": "euler"})
        s.set_engine(e)
        s.set_time_step(0.01, 0.1)
        st = DataStream()
        assert st.open(base, 14000, engine=e if device_frames else None) == 0
        assert s.run(d, 0.31, stream=st, dump_dt=0.1, check_dt=0.1) == 0
        assert st.close() == 0
        return d, e

    d, e = run(str(tmp_path / "dev/new"), True)
    run(str(tmp_path / "host/new"), False)
    _same_tree(tmp_path / "dev", tmp_path / "host")
    for k in range(3):
        assert os.path.exists(tmp_path / f"dev/new{k}.dat")
    lines = [ln for ln in (tmp_path / "dev/new.idx").read_text().split("\n") if ln]
    assert len(lines) == 8
    r = StreamReader()
    assert r.load(str(tmp_path / "dev/new")) == 0
    assert r.get_frame_count() == 5 and r.get_steps_count() == 4 and r.get_max_time() == 0.4
    expected = NBodyData(mass=d.mass)
    e.get_data(expected)
    got = NBodyData(mass=d.mass)
    assert r.seek(0) == 0 and r.read(got) == 0
    assert not np.array_equal(got.vertices, expected.vertices)
    assert got.get_time() == 0 and got.get_step() == 0
    assert r.seek(r.get_frame_count() - 1) == 0 and r.read(got) == 0
    assert np.array_equal(got.vertices, expected.vertices)
    assert np.array_equal(got.velocities, expected.velocities)
    assert got.get_time() == 0.4 and got.get_step() == 4


@pytest.mark.gpu
def test_device_frames_overlap_the_run(make_engine, tmp_path):
    """20 rk4 steps at N = 131072 (mixed) with a frame after every step.
    Device frames are copied behind the step's kernels and written by the
    library's thread while the next steps run, so they add almost nothing to
    the run; frames through get_data (the reference's path) stop the queue
    for the copy, the host-side transpose and the file write."""
    from nbody_gb300.solvers import create_solver
    n, steps = 131072, 20
    wall = {}
    for rnd in range(2):  # best of two rounds per mode: a shared box is noisy
        for mode in ("none", "device", "host"):
            d = NBodyData.plummer(n, seed=3)
            e = make_engine(precision="mixed", softening=1e-3)
            assert e.init(d)
            s = create_solver({"solver": "rk4"})
            s.set_engine(e)
            s.set_time_step(1e-3, 1e-3)
            st = None
            if mode in ("device", "host"):
                st = DataStream()
                assert st.open(str(tmp_path / f"{mode}{rnd}" / "f"), 1 << 30,
                               engine=e if mode == "device" else None) == 0

            def frame():
                if mode == "device":
                    assert st.write_engine(e, d) == 0
                elif mode == "host":
                    e.get_data(d)
                    assert st.write(d) == 0

            for _ in range(2):  # warm-up
                s.advise(1e-3)
                frame()
            e.synchronize()
            if st is not None:
                st.flush()
            t0 = time.perf_counter()
            for _ in range(steps):
                s.advise(1e-3)
                frame()
            e.synchronize()
            if st is not None:
                assert st.close() == 0
            t = (time.perf_counter() - t0) / steps
            wall[mode] = min(wall.get(mode, t), t)
            e.close()
    none = wall["none"]
    print(f"\nms per rk4 step with a frame of {n} bodies after each: device frames "
          f"{wall['device'] * 1e3:.2f}, get_data frames {wall['host'] * 1e3:.2f}, "
          f"no frames {none * 1e3:.2f}")
    assert wall["device"] <= 1.08 * none + 1e-3
    # both streams hold the same trajectory (same kernels in the same order)
    assert (tmp_path / "device0" / "f0.dat").read_bytes() == (tmp_path / "host0" / "f0.dat").read_bytes()
