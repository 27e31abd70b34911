"""The length-gauge l-space transform on the tcgen05 tensor cores (qpc_ltrans.cu) through the C ABI
(qpc_lspace_transform): bit for bit equal to its oracle (oracle/ltrans_oracle.py) for every n_l of
the tensor-core form, ragged tile counts, rows spanning hundreds of binary orders of magnitude and
zero rows; and the engine with the tensor-core transforms for every launch (QPC_LTRANS_TC=1) against
the engine with the FP64 kernel (QPC_LTRANS_TC=0) over a batched run."""
import numpy as np
import pytest

from conftest import engine, rel_l2
from oracle import ltrans_oracle as lo
from test_ltrans_oracle import vtable

pytestmark = pytest.mark.gpu


def _rows(rng, n_pos, n_l, wide):
    c = rng.standard_normal((n_pos, n_l)) + 1j * rng.standard_normal((n_pos, n_l))
    if wide:
        c *= 2.0 ** rng.integers(-300, 300, (n_pos, 1))
        c[::7] = 0
        c[1::5, 1::2] *= 2.0 ** -45	# odd channels far below the even ones
        c[2::9] = c[2::9].real + 0j	# zero imaginary rows
    return c


@pytest.mark.parametrize("n_l", [1, 2, 3, 20, 21, 32, 33, 41, 47, 48])
@pytest.mark.parametrize("forward", [True, False])
def test_bit_exact(q, n_l, forward):
    rng = np.random.default_rng(100 * n_l + forward)
    for n_pos, table, wide in ((1, "y10", False), (63, "random", True), (64, "y10", True), (130, "y10", False)):
        V = vtable(q, n_l) if table == "y10" else rng.standard_normal((n_l // 2 + 1, n_l))
        c = _rows(rng, n_pos, n_l, wide)
        got = q.lspace_transform(V, c, forward)
        want = lo.transform(V, c, forward)
        assert np.array_equal(got.view(np.float64), want.view(np.float64)), (n_l, n_pos, table)
        fp = lo.transform_fp64(V, c, forward)
        assert rel_l2(got, fp) < 1e-15 or not np.any(fp)


def test_many_tiles(q):
    """a few thousand tiles over the persistent blocks (more tiles than SMs)"""
    rng = np.random.default_rng(9)
    n_l, n_pos = 41, 64 * 700 + 17
    V = vtable(q, n_l)
    c = _rows(rng, n_pos, n_l, True)
    got = q.lspace_transform(V, c, True)
    idx = np.r_[0:200, n_pos - 200:n_pos, rng.integers(0, n_pos, 300)]
    want = lo.transform(V, c[idx], True)
    assert np.array_equal(got[idx].view(np.float64), want.view(np.float64))
    assert rel_l2(got, lo.transform_fp64(V, c, True)) < 1e-15


def _grid(q, n_r, p, n_l, rmax):
    t = q.linear_knots(n_r, p, 0.0, rmax)
    S, R, Ri, D, H = q.radial_setup(n_r, p, n_l, t)
    return S, R, H


@pytest.mark.parametrize("n_l", [21, 41])
def test_engine_paths_agree(q, monkeypatch, n_l):
    """a batched run with uneven pulses: the tensor-core transforms and the FP64 kernel k_transform
    give the same states to rounding"""
    n_r, p, B, dt = 200, 6, 5, 0.05
    S, R, H = _grid(q, n_r, p, n_l, 100.0)
    rng = np.random.default_rng(n_l)
    c0 = rng.standard_normal((B, 1, n_l, n_r)) + 1j * rng.standard_normal((B, 1, n_l, n_r))
    nt = np.array([120, 60, 121, 1, 90])
    ftab = np.zeros((B, int(nt.max()) + 1))
    for i in range(B):
        ftab[i, :nt[i] + 1] = 0.08 * np.sin(np.arange(nt[i] + 1) * dt * 0.057 + i)
    out = {}
    for mode in ("0", "1"):
        monkeypatch.setenv("QPC_LTRANS_TC", mode)
        prop = q.propagator_cn_hc_lgwz().initialize(n_r, p, n_l, S, R, H, dt, n_inst=B)
        prop.put(c0)
        prop.run(ftab, nt, nt + 3)
        out[mode] = prop.get()
        prop.close()
    assert rel_l2(out["1"], out["0"]) < 1e-12	# the short-run bar of the parity tests
