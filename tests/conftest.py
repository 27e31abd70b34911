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


class ArnoldiGrid(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int32) for n in ("n_r", "p", "n_l", "n_m", "m0", "n_inst", "kmax", "h_per_inst")] + \
               [(n, ctypes.c_double) for n in ("dt", "emin", "emax")] + \
               [(n, ctypes.c_void_p) for n in ("S", "chol", "R", "H", "y10")]


class ArnoldiOracle:
    """The CPU Arnoldi oracle (oracle/oracle_arnoldi.cpp), used only as the checker."""

    def __init__(self):
        from importlib import import_module
        b = import_module("qpc-tdse-cpc_gb300.build")
        self.lib = ctypes.CDLL(b.build_oracle())
        self.lib.oracle_chol_band.restype = ctypes.c_int
        self.lib.oracle_arnoldi_run.restype = ctypes.c_int

    def chol(self, S):
        S = np.ascontiguousarray(S, dtype=float)
        L = np.zeros_like(S)
        assert self.lib.oracle_chol_band(S.shape[0], S.shape[1] - 1, _p(S), _p(L)) == 0
        return L

    def grid(self, S, R, H, y10, dt, n_l, kmax=12, emin=1e-14, emax=1e-8, n_m=1, m0=0, n_inst=1, chol=None):
        """H [lmax+1][n_r][p+1] shared, or [n_inst][lmax+1][n_r][p+1] per instance."""
        n_r, ne = S.shape
        lmax = max(abs(m0), abs(m0 + n_m - 1)) + n_l - 1
        H = np.asarray(H, float)
        per = H.ndim == 4
        Hc = np.ascontiguousarray(H[:, :lmax + 1] if per else H[:lmax + 1])
        y = np.ascontiguousarray(np.broadcast_to(np.asarray(y10, float).reshape(-1, n_l), (n_m, n_l)))
        L = self.chol(S) if chol is None else np.ascontiguousarray(chol, dtype=float)
        keep = [np.ascontiguousarray(S, dtype=float), L, np.ascontiguousarray(R, dtype=float), Hc, y]
        g = ArnoldiGrid(n_r, ne - 1, n_l, n_m, m0, n_inst, kmax, int(per), dt, emin, emax, *[_p(a) for a in keep])
        g._keep = keep
        return g

    def mask(self, M, chol, coef, n_ch):
        """absorber_mask::operator() restated: c <- S^-1 (M c) per channel."""
        c = np.ascontiguousarray(coef, dtype=complex).copy()
        M = np.ascontiguousarray(M, dtype=float)
        self.lib.oracle_mask(M.shape[0], M.shape[1] - 1, ctypes.c_long(n_ch), _p(M), _p(np.ascontiguousarray(chol, dtype=float)), _p(c))
        return c

    def run(self, g, coef, eztab, nt=None, threads=1):
        """Returns (coef, crit[inst, s], msub[inst, s])."""
        c = np.ascontiguousarray(coef, dtype=complex).copy()
        tab = np.ascontiguousarray(np.broadcast_to(np.atleast_2d(eztab), (g.n_inst, np.atleast_2d(eztab).shape[1])), dtype=float)
        ld = tab.shape[1]
        nt = np.full(g.n_inst, ld, np.int64) if nt is None else np.ascontiguousarray(np.broadcast_to(nt, (g.n_inst,)), dtype=np.int64)
        crit = np.full((g.n_inst, ld), -1, np.int8)
        ms = np.full((g.n_inst, ld), -1, np.int8)
        rc = self.lib.oracle_arnoldi_run(ctypes.byref(g), _p(c), _p(tab), ctypes.c_long(ld), _p(nt), _p(crit), _p(ms), threads)
        assert rc == 0
        return c, crit, ms


class VgwrGrid(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int32) for n in ("n_r", "p", "n_l", "n_m", "m0", "n_inst")] + [("dt", ctypes.c_double)] + \
               [(n, ctypes.c_void_p) for n in ("S", "Rinv", "D", "upper", "lower")] + \
               [("lam", ctypes.c_void_p * 4), ("P", ctypes.c_void_p * 4)]


class VgwrOracle:
    """The CPU oracle of propagator_cn_hc_vgwr (oracle/oracle_cn.cpp), used only as the checker."""

    def __init__(self):
        self.o = Oracle()
        self.lib = self.o.lib

    def grid(self, S, Rinv, D, H, dt, n_l, n_m, m0, n_inst=1):
        q = engine()
        n_r, ne = S.shape
        p = ne - 1
        nlh = max(abs(m0), abs(m0 + n_m - 1)) + n_l
        up = np.zeros((nlh, n_r, ne), complex)
        lo = np.zeros((nlh, n_r, ne), complex)
        assert self.lib.oracle_cn_bands(n_r, p, nlh, _p(np.ascontiguousarray(S)), _p(np.ascontiguousarray(H[:nlh])),
                                        ctypes.c_double(dt), _p(up), _p(lo)) == 0
        eig = [q.vgwr_angular(n_l, n_m, m0, c) for c in range(4)]
        keep = [np.ascontiguousarray(S), np.ascontiguousarray(Rinv), np.ascontiguousarray(D), up, lo] + \
               [e[0] for e in eig] + [e[1] for e in eig]
        g = VgwrGrid(n_r, p, n_l, n_m, m0, n_inst, dt, *[_p(a) for a in keep[:5]])
        for c in range(4):
            g.lam[c] = keep[5 + c].ctypes.data
            g.P[c] = keep[9 + c].ctypes.data
        g._keep = keep
        return g

    def run(self, g, coef, atab, nt_field, nt_total, threads=1):
        c = np.ascontiguousarray(coef, dtype=complex).copy()
        tab = np.ascontiguousarray(atab, dtype=float)
        nf = np.ascontiguousarray(np.broadcast_to(nt_field, (g.n_inst,)), dtype=np.int64)
        ntt = np.ascontiguousarray(np.broadcast_to(nt_total, (g.n_inst,)), dtype=np.int64)
        self.lib.oracle_vgwr_run(ctypes.byref(g), _p(c), _p(tab), ctypes.c_long(tab.shape[-2]), _p(nf), _p(ntt), threads)
        return c


@pytest.fixture(scope="session")
def q():
    return engine()


@pytest.fixture(scope="session")
def oracle():
    return Oracle()


@pytest.fixture(scope="session")
def aoracle():
    return ArnoldiOracle()


@pytest.fixture(scope="session")
def voracle():
    return VgwrOracle()


def rel_l2(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


def band_mask(n_r, p):
    return np.array([[r + k < n_r for k in range(p + 1)] for r in range(n_r)])
