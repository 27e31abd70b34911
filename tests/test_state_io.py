"""State files with the reference driver's dataset names (/coef1 and the grid scalars) and
init::load_initial's checks (binsrc/sphTDSE.cpp:119-163)."""
import importlib

import numpy as np


def test_round_trip_and_checks(tmp_path):
    io = importlib.import_module("qpc-tdse-cpc_gb300.state_io")
    rng = np.random.default_rng(0)
    c = rng.standard_normal((3, 4, 20)) + 1j * rng.standard_normal((3, 4, 20))
    f = str(tmp_path / "s.npz")
    io.save_state(f, c, 20, 6, 4, 3, -1, 0.0, 50.0)
    rc, back = io.load_initial(f, 20, 6, 4, 3, -1, 0.0, 50.0)
    assert rc == 0 and np.array_equal(back, c)
    # into a larger grid: m -2..2, 6 l channels; the file's m = -1..1 land at im = 1..3
    rc, big = io.load_initial(f, 20, 6, 6, 5, -2, 0.0, 50.0)
    assert rc == 0 and np.array_equal(big[1:4, :4], c) and not big[0].any() and not big[:, 4:].any()
    assert io.load_initial(f, 21, 6, 4, 3, -1, 0.0, 50.0)[0] == -1
    assert io.load_initial(f, 20, 6, 4, 3, -1, 0.0, 60.0)[0] == -1
    assert io.load_initial(f, 20, 7, 4, 3, -1, 0.0, 50.0)[0] == -2
    assert io.load_initial(f, 20, 6, 4, 3, 0, 0.0, 50.0)[0] == -3
    assert io.load_initial(f, 20, 6, 3, 3, -1, 0.0, 50.0)[0] == -4
