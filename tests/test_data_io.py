"""Body-data loaders and writer against the reference's own fixtures
(test/stream/test_nbody_stream.cpp:344-372: save_load, load_zeno_ascii,
negative) and the unit systems of load_initial (nbody/nbody_data.cpp:616-673)."""
from pathlib import Path

import numpy as np
import pytest

from nbody_gb300.data import MASS_FACTOR, NBodyData

GOLDEN = Path(__file__).resolve().parent / "golden"


def test_save_load_roundtrip(tmp_path):
    d1 = NBodyData.load(str(GOLDEN / "initial_state.txt"))
    d1.save(str(tmp_path / "test_save.txt"))
    d2 = NBodyData.load(str(tmp_path / "test_save.txt"))
    assert d2.is_equal(d1, 1e-16)


def test_load_zeno_ascii_equals_table():
    d1 = NBodyData.load_zeno_ascii(str(GOLDEN / "zeno_ascii.txt"))
    d2 = NBodyData.load(str(GOLDEN / "zeno_table.txt"))
    assert d1.get_count() == 16 and d1.box_size == 1
    assert d2.is_equal(d1, 1e-16)


@pytest.mark.parametrize("name", ["inv_column", "inv_columns_count", "inv_radius"])
def test_load_rejects_malformed_tables(name):
    assert (GOLDEN / f"{name}.txt").exists()
    with pytest.raises(ValueError):
        NBodyData.load(str(GOLDEN / f"{name}.txt"))


def test_load_zeno_rejects_malformed(tmp_path):
    bad = {"dim": "16\n2\nx\n", "count": "many\n3\nx\n", "short": "2\n3\nx\n1\n1\n0 0 0\n",
           "vector": "1\n3\nx\n1\n0 0\n0 0 0\n"}
    for name, text in bad.items():
        p = tmp_path / f"{name}.txt"
        p.write_text(text)
        with pytest.raises(ValueError):
            NBodyData.load_zeno_ascii(str(p))


def test_load_initial_units_and_box():
    g1 = NBodyData.load_initial(str(GOLDEN / "initial_state.txt"), "G1")
    si = NBodyData.load_initial(str(GOLDEN / "initial_state.txt"), "si")
    adk = NBodyData.load_initial(str(GOLDEN / "initial_state.txt"), "ADK")
    assert np.array_equal(si.mass, g1.mass * 6.67259e-11)
    assert np.array_equal(adk.mass, g1.mass * MASS_FACTOR["ADK"])
    assert abs(MASS_FACTOR["ADK"] / 1.4880e-34 - 1.0) < 1e-3  # G in au^3/(kg day^2)
    expect_box = int(max(1.0, g1.vertices.max()))
    assert g1.box_size == expect_box
    z = NBodyData.load_initial(str(GOLDEN / "zeno_ascii.txt"), "zeno")
    assert z.box_size == int(max(1.0, z.vertices.max()))
    with pytest.raises(ValueError):
        NBodyData.load_initial(str(GOLDEN / "initial_state.txt"), "parsec")
