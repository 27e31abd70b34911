"""The C++ drop-in binding include/qpc_gb300_lgwz.hpp, compiled together with the
reference's own headers (with the MKL/GSL/HDF5 shims of oracle/ref/shim) and linked
against the engine library, as a reference maintainer would build it (the
select_cond swap at binsrc/sphTDSE.cpp:574-579).  The program initialises the
reference's propagator_cn_hc_lgwz and the binding from the same integrators and
steps both.  Without a GPU the binding's initialize must report the engine's error
as the reference's errn_t (exit 3); with one, both results must agree.

Needs the reference checkout (QPC_REFERENCE_DIR, else the development machine's
location); skipped where it is absent, as on a GPU machine."""
import os
import subprocess

import pytest

from conftest import ROOT


def _reference_include():
    for c in (os.environ.get("QPC_REFERENCE_DIR"), "/root/reference"):
        if c and os.path.isfile(os.path.join(c, "include", "spherical", "inventory.h")):
            return os.path.join(c, "include")
    return None


def _openblas():
    import glob
    import scipy
    libs = glob.glob(os.path.join(os.path.dirname(scipy.__file__), "..", "scipy.libs", "libscipy_openblas-*.so"))
    return os.path.abspath(libs[0]) if libs else None


def test_binding_compiles_links_and_runs_against_the_reference(q, tmp_path):
    inc = _reference_include()
    if inc is None:
        pytest.skip("reference checkout absent")
    blas = _openblas()
    if blas is None:
        pytest.skip("no OpenBLAS for the reference's BLAS calls")
    lib = q.load()
    libdir = os.path.dirname(os.path.abspath(q.LIB_PATH))
    exe = str(tmp_path / "adapter_driver")
    cmd = ["g++", "-std=c++17", "-O2", "-march=native", "-fopenmp",
           "-I", os.path.join(ROOT, "oracle", "ref", "shim"), "-I", inc, "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "adapter_driver.cpp"), "-o", exe,
           "-L" + libdir, "-l:libqpc_gb300.so", "-Wl,-rpath," + libdir, blas, "-Wl,-rpath," + os.path.dirname(blas)]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout[-4000:]
    run = subprocess.run([exe], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=600)
    try:
        import torch
        have_gpu = torch.cuda.is_available()
    except Exception:
        have_gpu = False
    if have_gpu:
        assert run.returncode == 0, run.stdout
    else:
        assert run.returncode == 3, run.stdout
        assert "qpc_lgwz_create" in run.stdout and "CUDA" in run.stdout, run.stdout
