"""The table container format (simpimc_gb300/tables.py, src/framework/table_io.h) that holds pair
action tables and run output."""
import numpy as np


def test_container_round_trip_with_strings(tmp_path):
    """Numbers, arrays and string datasets (the run output's names and type tags) survive the
    container exactly."""
    from simpimc_gb300.tables import read_table, write_table
    vals = {"Moves/B/type": "Bisect", "x": np.array([0.1, 1e-300, -3.0, np.pi, 7.0]), "n": 3,
            "Observables/gr/species_a": "e up", "y": np.arange(9.0)}
    write_table(tmp_path / "t.pat", vals)
    back = read_table(tmp_path / "t.pat")
    assert back["Moves/B/type"] == "Bisect" and back["Observables/gr/species_a"] == "e up"
    np.testing.assert_array_equal(back["x"], vals["x"])
    np.testing.assert_array_equal(back["y"], vals["y"])
    assert back["n"].tolist() == [3.0]
