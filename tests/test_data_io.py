"""The G1 table loader and writer against the reference's own fixtures
(test/stream/test_nbody_stream.cpp:344-372: save_load and the malformed
tables); they read and write the golden vectors of the solver tests."""
from pathlib import Path

import pytest

from nbody_gb300.data import NBodyData

GOLDEN = Path(__file__).resolve().parent / "golden"


def test_save_load_roundtrip(tmp_path):
    d1 = NBodyData.load(str(GOLDEN / "initial_state.txt"))
    d1.save(str(tmp_path / "test_save.txt"))
    d2 = NBodyData.load(str(tmp_path / "test_save.txt"))
    assert d2.is_equal(d1, 1e-16)


@pytest.mark.parametrize("name", ["inv_column", "inv_columns_count", "inv_radius"])
def test_load_rejects_malformed_tables(name):
    assert (GOLDEN / f"{name}.txt").exists()
    with pytest.raises(ValueError):
        NBodyData.load(str(GOLDEN / f"{name}.txt"))
