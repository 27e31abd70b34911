"""The C ABI library: loads, exports what include/qpc_gb300.h declares, and
rejects bad arguments with status codes (no GPU needed)."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def _declared():
    txt = open(os.path.join(ROOT, "include", "qpc_gb300.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(qpc_[a-z0-9_]+)\s*\(", txt)))


def test_exports_every_declared_symbol(q):
    lib = q.load()
    names = _declared()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(names) == set(q.EXPORTS)


def test_library_is_in_tree(q):
    lib = q.load()
    assert os.path.dirname(os.path.abspath(q.LIB_PATH)).startswith(ROOT)
    assert b"sm_103a" in lib.qpc_version()


def test_bad_arguments_return_codes(q):
    lib = q.load()
    assert lib.qpc_linear_knots(10, 6, 0.0, 1.0, None) == 1
    assert lib.qpc_radial_setup(5, 6, 1, None, None, 1.0, None, None, None, None, None) == 1
    assert lib.qpc_lgwz_create(None, 0.05, None, None, None, None) == 1
    d = q.qpc_dims(10, 6, 4, 1, 0, 1)  # n_r < 2p+2
    h = ctypes.c_void_p()
    S = np.zeros((10, 7))
    assert lib.qpc_lgwz_create(ctypes.byref(d), 0.05, S.ctypes.data, S.ctypes.data, S.ctypes.data, ctypes.byref(h)) == 1
    assert b"bad dims" in lib.qpc_last_error()
    assert lib.qpc_lgwz_destroy(None) == 0


def test_no_device_is_an_error_not_a_fallback(q):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    t = q.linear_knots(32, 6, 0.0, 20.0)
    S, R, _, _, H = q.radial_setup(32, 6, 4, t)
    with pytest.raises(q.QpcError) as e:
        q.propagator_cn_hc_lgwz().initialize(32, 6, 4, S, R, H, 0.05)
    assert e.value.code == 8  # QPC_ERR_NODEVICE


def test_field_and_setup_errors(q):
    with pytest.raises(q.QpcError):
        q.field_sinen(0.05, -1.0, 4, 0, 0, 0.05)
    with pytest.raises(q.QpcError):
        q.radial_setup(8, 6, 1, np.zeros(17))


def test_other_engines_check_arguments_and_device(q):
    """Arnoldi, velocity-gauge and surrogate handles: argument errors before any device use,
    QPC_ERR_NODEVICE (not a CPU path) without a GPU."""
    torch = pytest.importorskip("torch")
    lib = q.load()
    t = q.linear_knots(32, 6, 0.0, 20.0)
    S, R, Ri, D, H = q.radial_setup(32, 6, 6, t)
    y10 = q.y10_coupling(4)
    h = ctypes.c_void_p()
    d = q.qpc_dims(32, 6, 4, 1, 0, 1)
    P = lambda a: a.ctypes.data
    # emin > emax: rejected as the reference's arnoldi_workspace constructor does
    assert lib.qpc_arnoldi_create(ctypes.byref(d), P(S), P(R), P(H), 0, P(y10), 0.1, 12, 1e-8, 1e-14, ctypes.byref(h)) == 1
    assert lib.qpc_arnoldi_create(ctypes.byref(d), P(S), P(R), P(H), 0, P(y10), 0.1, 0, 1e-14, 1e-8, ctypes.byref(h)) == 1
    assert lib.qpc_vgwr_create(ctypes.byref(d), -0.05, P(S), P(Ri), P(D), P(H), ctypes.byref(h)) == 1
    assert lib.qpc_mlp_create(6, 250, 4, 384, 5, 0, ctypes.byref(h)) == 1       # n_hidden not a multiple of 16
    if torch.cuda.is_available():
        return
    with pytest.raises(q.QpcError) as e:
        q.propagator_hc_lgwz(12, 1e-14, 1e-8).initialize(32, 6, 4, S, R, H, y10, 0.1)
    assert e.value.code == 8
    with pytest.raises(q.QpcError) as e:
        q.propagator_cn_hc_vgwr().initialize(32, 6, 2, 3, -1, S, Ri, D, H, 0.05)
    assert e.value.code == 8
    with pytest.raises(q.QpcError) as e:
        q.mlp_ensemble(6, 384)
    assert e.value.code == 8


def test_momentum_handles_check_arguments_and_device(q):
    """PCS projector and t-SURFF accumulator: bad tables are rejected before any device use,
    and without a GPU the handles report QPC_ERR_NODEVICE (no CPU path)."""
    torch = pytest.importorskip("torch")
    lib = q.load()
    kn = q.linear_knots(32, 6, 0.0, 20.0)
    h = ctypes.c_void_p()
    d = q.qpc_dims(32, 6, 4, 1, 0, 2)
    g = q.qpc_kgrid(6, 3, 2, 0.2, 1.0, 0.0, 3.0, 0.0, 6.0, 0)
    t = q.pcs_tables(32, 6, 4, kn, 6, 3, 2, 0.2, 1.0, 0.0, 3.0, 0.0, 6.0, 1.0)
    P = lambda a: a.ctypes.data
    assert lib.qpc_pcs_create(ctypes.byref(d), ctypes.byref(g), None, P(t["ijl"]), P(t["plm"]), P(t["exm"]), P(t["cps"]), ctypes.byref(h)) == 1
    ts = q.tsurff_tables(32, 6, 4, kn, 12.0, 0.0, 6, 3, 2, 0.2, 1.0, 0.0, 3.0, 0.0, 6.0)
    bad = np.full(ts["ib"].size, 40, np.int32)      # spline index outside the grid
    args = [P(ts[k]) for k in ("kr", "kt", "kp")]
    assert lib.qpc_tsurff_create(ctypes.byref(d), ctypes.byref(g), *args, bad.size, P(bad), P(ts["b0"]), P(ts["br"]), P(ts["j0"]),
                                 P(ts["jr"]), P(ts["y0"]), P(ts["e0"]), P(ts["pmat"]), ctypes.byref(h)) == 1
    assert lib.qpc_pcs_measure(None, 0, None, 0, 1, None) == 1
    assert lib.qpc_tsurff_accumulate(None, 0, None, 0.05, None, 0) == 1
    if torch.cuda.is_available():
        return
    with pytest.raises(q.QpcError) as e:
        q.spectrum_c_pcs(6, 3, 2).initialize(32, 6, 4, kn, 0.2, 1.0, 0.0, 3.0, 0.0, 6.0, 1.0, tables=t)
    assert e.value.code == 8
    with pytest.raises(q.QpcError) as e:
        q.spectrum_c_tsf(6, 3, 2).initialize(32, 6, 4, kn, 12.0, 0.0, 0.2, 1.0, 0.0, 3.0, 0.0, 6.0, n_inst=2, tables=ts)
    assert e.value.code == 8
