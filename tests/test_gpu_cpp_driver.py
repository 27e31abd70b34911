"""C++ host code over the C ABI, without Python in the loop: tests/cpp/lgwz_driver.cpp runs the
reference driver's length-gauge loop (setup, create, put, the step loop as one run or as one
propagate per step, get, S-norm) and its result is compared with the reference's own output
(tests/golden/small_prop.npz: 50 field steps and 5 field-free steps on the small grid)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT, golden, rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def driver(q, tmp_path_factory):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no C++ compiler")
    q.load()
    pkg = os.path.dirname(q.LIB_PATH)
    exe = str(tmp_path_factory.mktemp("cpp") / "lgwz_driver")
    subprocess.run([cxx, "-std=c++17", "-O2", os.path.join(ROOT, "tests", "cpp", "lgwz_driver.cpp"), "-I", os.path.join(ROOT, "include"),
                    "-o", exe, q.LIB_PATH, "-Wl,-rpath," + pkg], check=True)
    return exe


@pytest.mark.parametrize("mode", ["run", "stepwise"])
def test_cpp_driver_matches_reference(driver, tmp_path, mode):
    g, s = golden("small_prop"), golden("small_setup")
    n_r, p, n_l = int(s["n_r"]), int(s["p"]), int(s["n_l"])
    init, f = tmp_path / "init.bin", tmp_path / "field.bin"
    np.ascontiguousarray(g["init"], np.complex128).tofile(init)
    np.ascontiguousarray(g["f"], np.float64).tofile(f)
    out = tmp_path / "out.bin"
    args = [driver, str(n_r), str(p), str(n_l), repr(float(s["rmax"])), repr(float(s["dt"])), str(init), str(f), str(int(g["nt"])),
            str(int(g["nfree"])), str(out)] + (["stepwise"] if mode == "stepwise" else [])
    subprocess.run(args, check=True, stdout=subprocess.PIPE)
    res = np.fromfile(out)
    coef = res[:-1].view(np.complex128).reshape(n_l, n_r)
    assert rel_l2(coef, g["coef"]) < 1e-12
    assert abs(res[-1] - g["norm"][0]) < 1e-12 * g["norm"][0]
