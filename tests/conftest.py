import ctypes
import importlib
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def engine():
    """The package (its directory name has dashes, so it is imported by name)."""
    return importlib.import_module("qpc-tdse-cpc_gb300")


def golden(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


class OracleGrid(ctypes.Structure):
    _fields_ = [("n_r", ctypes.c_int32), ("p", ctypes.c_int32), ("n_l", ctypes.c_int32), ("n_m", ctypes.c_int32),
                ("m0", ctypes.c_int32), ("n_inst", ctypes.c_int32), ("dt", ctypes.c_double),
                ("S", ctypes.c_void_p), ("R", ctypes.c_void_p), ("yeig", ctypes.c_void_p), ("yprj", ctypes.c_void_p),
                ("upper", ctypes.c_void_p), ("lower", ctypes.c_void_p)]


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class Oracle:
    """The CPU oracle (oracle/oracle_cn.cpp), used only as the checker."""

    def __init__(self):
        from importlib import import_module
        b = import_module("qpc-tdse-cpc_gb300.build")
        self.lib = ctypes.CDLL(b.build_oracle())
        self.lib.oracle_cn_bands.restype = ctypes.c_int
        self.lib.oracle_lu_zsb.restype = ctypes.c_int

    def grid(self, S, R, H, dt, n_l, n_m=1, m0=0, n_inst=1):
        """Build the reference's setup (bands, Y10 eigensystems per m) for the oracle."""
        q = engine()
        n_r, ne = S.shape
        p = ne - 1
        lmax = max(abs(m0), abs(m0 + n_m - 1)) + n_l - 1
        nl = lmax + 1
        up = np.zeros((nl, n_r, ne), complex)
        lo = np.zeros((nl, n_r, ne), complex)
        Hc = np.ascontiguousarray(H[:nl])
        err = self.lib.oracle_cn_bands(n_r, p, nl, _p(np.ascontiguousarray(S)), _p(Hc), ctypes.c_double(dt), _p(up), _p(lo))
        assert err == 0
        lam = np.zeros((n_m, n_l))
        P = np.zeros((n_m, n_l, n_l))
        for im in range(n_m):
            lam[im], P[im] = q.y10_eigen(n_l, m0 + im)
        keep = [np.ascontiguousarray(S), np.ascontiguousarray(R), lam, P, up, lo]
        g = OracleGrid(n_r, p, n_l, n_m, m0, n_inst, dt, *[_p(a) for a in keep])
        g._keep = keep
        return g

    def step(self, g, coef, f_ti=None, f_tf=None, threads=1):
        c = np.ascontiguousarray(coef, dtype=complex).copy()
        if f_ti is None:
            self.lib.oracle_lgwz_step(ctypes.byref(g), _p(c), None, None, threads)
        else:
            a = np.ascontiguousarray(np.broadcast_to(f_ti, (g.n_inst,)), dtype=float)
            b = np.ascontiguousarray(np.broadcast_to(f_tf, (g.n_inst,)), dtype=float)
            self.lib.oracle_lgwz_step(ctypes.byref(g), _p(c), _p(a), _p(b), threads)
        return c

    def run(self, g, coef, ftab, nt_field, nt_total, threads=1):
        c = np.ascontiguousarray(coef, dtype=complex).copy()
        ftab = np.ascontiguousarray(np.atleast_2d(ftab), dtype=float)
        nf = np.ascontiguousarray(nt_field, dtype=np.int64)
        ntt = np.ascontiguousarray(nt_total, dtype=np.int64)
        self.lib.oracle_lgwz_run(ctypes.byref(g), _p(c), _p(ftab), ctypes.c_long(ftab.shape[1]), _p(nf), _p(ntt), threads)
        return c

    def norm(self, g, coef):
        out = np.zeros(g.n_inst)
        self.lib.oracle_norm(ctypes.byref(g), _p(np.ascontiguousarray(coef, dtype=complex)), _p(out))
        return out

    def dipole(self, g, F, y10, coef):
        out = np.zeros(2 * g.n_inst)
        self.lib.oracle_dipole(ctypes.byref(g), _p(np.ascontiguousarray(F)), _p(np.ascontiguousarray(y10)),
                               _p(np.ascontiguousarray(coef, dtype=complex)), _p(out))
        return out[0::2] + 1j * out[1::2]


@pytest.fixture(scope="session")
def q():
    return engine()


@pytest.fixture(scope="session")
def oracle():
    return Oracle()


def rel_l2(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


def band_mask(n_r, p):
    return np.array([[r + k < n_r for k in range(p + 1)] for r in range(n_r)])
