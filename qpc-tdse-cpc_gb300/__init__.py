"""Python host-side mirror of the QPC-TDSE propagation path, over the C ABI of
the GB300 engine (include/qpc_gb300.h, library libqpc_gb300.so built in-tree).

The names follow the reference's C++ interface for the path:
  integrator_radi.initialize(rmin, rmax)      -> radial_setup(...)   (spherical/utilities/basisfunc.hpp:33-36)
  operator_y10::solve_eigen                   -> y10_eigen(...)      (spherical/operators/1e.hpp:304-333)
  coefficient::initialize (ground state)      -> ground_state(...)   (spherical/coefficient/1e.hpp:91-143)
  field<field_component_sinen<2>>             -> field_sinen(...)    (structure/field.h:89-133, 229-311)
  propagator_cn_hc_lgwz::initialize/propagate -> propagator_cn_hc_lgwz (spherical/propagator/cn_1e.hpp:549-619)

Errors from the engine raise QpcError with the engine's message; a missing
library or a missing GPU raises instead of falling back to anything else.
"""
import ctypes
import os

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libqpc_gb300.so")

QPC_OK = 0
ERRORS = {1: "QPC_ERR_ARGS", 2: "QPC_ERR_NOMEM", 3: "QPC_ERR_CUDA", 4: "QPC_ERR_SINGULAR",
          5: "QPC_ERR_NUMERIC", 6: "QPC_ERR_TIMEOUT", 7: "QPC_ERR_STATE", 8: "QPC_ERR_NODEVICE"}
POTENTIAL_HYDROGENIC = 0
POTENTIAL_YUKAWA = 1

# every symbol include/qpc_gb300.h declares
EXPORTS = (
    "qpc_last_error", "qpc_version", "qpc_set_wait_limit", "qpc_get_wait_limit", "qpc_fp64_peak",
    "qpc_lgwz_stream", "qpc_vgwr_set_profiling", "qpc_vgwr_kernel_times", "qpc_vgwr_run_dipole", "qpc_lgwz_run_ex",
    "qpc_hhg_spectra", "qpc_dgemm_slices", "qpc_lspace_transform", "qpc_linear_knots", "qpc_radial_setup", "qpc_y10_coupling",
    "qpc_y10_eigen", "qpc_ldlt_csym", "qpc_gen_eigen", "qpc_field_sinen", "qpc_lgwz_create",
    "qpc_lgwz_destroy", "qpc_lgwz_put", "qpc_lgwz_get", "qpc_lgwz_put_device", "qpc_lgwz_get_device",
    "qpc_lgwz_propagate", "qpc_lgwz_propagate_free", "qpc_lgwz_run", "qpc_lgwz_norm", "qpc_lgwz_dipole",
    "qpc_lgwz_projection", "qpc_lgwz_last_run_ms", "qpc_lgwz_launch_count", "qpc_lgwz_set_profiling",
    "qpc_lgwz_kernel_times", "qpc_lgwz_get_tuning", "qpc_fieldfree_noalloc", "qpc_lgwz_run_dipole",
    "qpc_hhg_spectrum", "qpc_pes_bin", "qpc_cholesky_band", "qpc_arnoldi_create", "qpc_arnoldi_destroy",
    "qpc_arnoldi_put", "qpc_arnoldi_get", "qpc_arnoldi_put_device", "qpc_arnoldi_get_device", "qpc_arnoldi_run",
    "qpc_arnoldi_propagate", "qpc_arnoldi_norm", "qpc_arnoldi_last_run", "qpc_lgwz_run_many",
    "qpc_mlp_create", "qpc_mlp_destroy", "qpc_mlp_param_count", "qpc_mlp_get_params", "qpc_mlp_set_params",
    "qpc_mlp_loss_grad", "qpc_mlp_train", "qpc_mlp_predict", "qpc_vgwr_angular", "qpc_vgwr_create",
    "qpc_vgwr_destroy", "qpc_vgwr_put", "qpc_vgwr_get", "qpc_vgwr_put_device", "qpc_vgwr_get_device",
    "qpc_vgwr_propagate", "qpc_vgwr_propagate_free", "qpc_vgwr_run", "qpc_vgwr_norm", "qpc_vgwr_last_run",
    "qpc_mask_band", "qpc_lgwz_mask", "qpc_lgwz_dims", "qpc_vgwr_dims", "qpc_coulomb_f", "qpc_coulomb_sigma",
    "qpc_sph_legendre", "qpc_pcs_tables", "qpc_tsurff_tables", "qpc_pcs_create", "qpc_pcs_destroy", "qpc_pcs_measure",
    "qpc_lgwz_pcs", "qpc_tsurff_create", "qpc_tsurff_destroy", "qpc_tsurff_clear", "qpc_tsurff_accumulate",
    "qpc_lgwz_tsurff", "qpc_vgwr_tsurff", "qpc_tsurff_get", "qpc_pcs_last_run", "qpc_tsurff_last_run",
    "qpc_lgwz_create_ex", "qpc_pcs_tables_numeric",
)
SPEC_LMD, SPEC_PMD, SPEC_PAD = 0, 1, 2
TSURFF_FREE, TSURFF_Z, TSURFF_XY = 0, 1, 2
NOALLOC_MAX_ELEMS = 1 << 20
KERNELS = ("factor", "transform_fwd", "sweep", "transform_bwd", "fieldfree")


class QpcError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s: %s" % (ERRORS.get(code, code), msg))
        self.code = code


class qpc_potential(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("zc", ctypes.c_double), ("zs", ctypes.c_double), ("sigma", ctypes.c_double)]


class qpc_dims(ctypes.Structure):
    _fields_ = [("n_r", ctypes.c_int32), ("p", ctypes.c_int32), ("n_l", ctypes.c_int32),
                ("n_m", ctypes.c_int32), ("m0", ctypes.c_int32), ("n_inst", ctypes.c_int32)]


class qpc_run_opts(ctypes.Structure):
    _fields_ = [("mask", ctypes.c_void_p), ("tsurff", ctypes.c_void_p)]


class qpc_kgrid(ctypes.Structure):
    _fields_ = [("nkr", ctypes.c_int32), ("nkt", ctypes.c_int32), ("nkp", ctypes.c_int32),
                ("krmin", ctypes.c_double), ("krmax", ctypes.c_double), ("ktmin", ctypes.c_double),
                ("ktmax", ctypes.c_double), ("kpmin", ctypes.c_double), ("kpmax", ctypes.c_double), ("flag", ctypes.c_int32)]


_lib = None


def load(path=None):
    """Load the engine library; builds it first if it is missing (the build
    needs nvcc, not a GPU)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        from . import build as _b
        _b.build_engine()
    lib = ctypes.CDLL(path)
    P = ctypes.c_void_p
    i32, i64, d = ctypes.c_int32, ctypes.c_int64, ctypes.c_double
    sig = {
        "qpc_last_error": (ctypes.c_char_p, []),
        "qpc_version": (ctypes.c_char_p, []),
        "qpc_linear_knots": (ctypes.c_int, [i32, i32, d, d, P]),
        "qpc_radial_setup": (ctypes.c_int, [i32, i32, i32, P, P, d, P, P, P, P, P]),
        "qpc_y10_coupling": (ctypes.c_int, [i32, i32, P]),
        "qpc_y10_eigen": (ctypes.c_int, [i32, i32, P, P]),
        "qpc_ldlt_csym": (ctypes.c_int, [i32, i32, P, P, d, P, P]),
        "qpc_gen_eigen": (ctypes.c_int, [i32, i32, P, P, i32, P, P]),
        "qpc_field_sinen": (ctypes.c_int, [i32, d, d, d, d, d, d, i64, P, P]),
        "qpc_lgwz_create": (ctypes.c_int, [P, d, P, P, P, P]),
        "qpc_lgwz_create_ex": (ctypes.c_int, [P, d, P, P, P, i32, P]),
        "qpc_lgwz_destroy": (ctypes.c_int, [P]),
        "qpc_lgwz_put": (ctypes.c_int, [P, P]),
        "qpc_lgwz_get": (ctypes.c_int, [P, P]),
        "qpc_lgwz_put_device": (ctypes.c_int, [P, P]),
        "qpc_lgwz_get_device": (ctypes.c_int, [P, P]),
        "qpc_lgwz_propagate": (ctypes.c_int, [P, P, P]),
        "qpc_lgwz_propagate_free": (ctypes.c_int, [P]),
        "qpc_lgwz_run": (ctypes.c_int, [P, P, i64, P, P]),
        "qpc_lgwz_run_ex": (ctypes.c_int, [P, P, i64, P, P, P]),
        "qpc_lgwz_norm": (ctypes.c_int, [P, P]),
        "qpc_lgwz_dipole": (ctypes.c_int, [P, P, P]),
        "qpc_lgwz_projection": (ctypes.c_int, [P, P, P, P]),
        "qpc_lgwz_last_run_ms": (ctypes.c_int, [P, P]),
        "qpc_lgwz_launch_count": (ctypes.c_int64, [P]),
        "qpc_lgwz_set_profiling": (ctypes.c_int, [P, ctypes.c_int]),
        "qpc_lgwz_kernel_times": (ctypes.c_int, [P, P, P]),
        "qpc_lgwz_get_tuning": (ctypes.c_int, [P, P]),
        "qpc_fieldfree_noalloc": (ctypes.c_int, [P, P, P, P, P]),
        "qpc_lgwz_run_dipole": (ctypes.c_int, [P, P, i64, P, P, P, P, i64]),
        "qpc_hhg_spectrum": (ctypes.c_int, [P, i64, d, d, d, d, i32, P, P]),
        "qpc_hhg_spectra": (ctypes.c_int, [i32, P, i64, P, d, d, P, P, i32, i64, P]),
        "qpc_dgemm_slices": (ctypes.c_int, [i64, i64, i64, P, i64, P, i64, P, i64, P]),
        "qpc_lspace_transform": (ctypes.c_int, [i64, i32, P, i32, P, P]),
        "qpc_pes_bin": (ctypes.c_int, [P, P, i64, d, d, i32, d, P, P, P]),
        "qpc_cholesky_band": (ctypes.c_int, [i32, i32, P, P]),
        "qpc_lgwz_run_many": (ctypes.c_int, [i32, P, P, P, P, P, P]),
        "qpc_mlp_create": (ctypes.c_int, [i32, i32, i32, i32, i32, ctypes.c_uint64, P]),
        "qpc_vgwr_angular": (ctypes.c_int, [i32, i32, i32, i32, P, P]),
        "qpc_mask_band": (ctypes.c_int, [i32, i32, P, d, d, d, P]),
        "qpc_lgwz_mask": (ctypes.c_int, [P, P]),
        "qpc_vgwr_create": (ctypes.c_int, [P, d, P, P, P, P, P]),
        "qpc_vgwr_destroy": (ctypes.c_int, [P]),
        "qpc_vgwr_put": (ctypes.c_int, [P, P]),
        "qpc_vgwr_get": (ctypes.c_int, [P, P]),
        "qpc_vgwr_put_device": (ctypes.c_int, [P, P]),
        "qpc_vgwr_get_device": (ctypes.c_int, [P, P]),
        "qpc_vgwr_propagate": (ctypes.c_int, [P, P, P, P, P]),
        "qpc_vgwr_propagate_free": (ctypes.c_int, [P]),
        "qpc_vgwr_run": (ctypes.c_int, [P, P, i64, P, P]),
        "qpc_vgwr_run_dipole": (ctypes.c_int, [P, P, i64, P, P, P, P, P, i64]),
        "qpc_vgwr_norm": (ctypes.c_int, [P, P]),
        "qpc_vgwr_last_run": (ctypes.c_int, [P, P, P]),
        "qpc_vgwr_set_profiling": (ctypes.c_int, [P, ctypes.c_int]),
        "qpc_vgwr_kernel_times": (ctypes.c_int, [P, P, P]),
        "qpc_mlp_destroy": (ctypes.c_int, [P]),
        "qpc_mlp_param_count": (ctypes.c_int, [P, P]),
        "qpc_mlp_get_params": (ctypes.c_int, [P, i32, P]),
        "qpc_mlp_set_params": (ctypes.c_int, [P, i32, P]),
        "qpc_mlp_loss_grad": (ctypes.c_int, [P, P, P, i32, P, P]),
        "qpc_mlp_train": (ctypes.c_int, [P, P, P, i32, i32, i32, ctypes.c_float, ctypes.c_uint64, P]),
        "qpc_mlp_predict": (ctypes.c_int, [P, P, i32, P]),
        "qpc_arnoldi_create": (ctypes.c_int, [P, P, P, P, i32, P, d, i32, d, d, P]),
        "qpc_arnoldi_destroy": (ctypes.c_int, [P]),
        "qpc_arnoldi_put": (ctypes.c_int, [P, P]),
        "qpc_arnoldi_get": (ctypes.c_int, [P, P]),
        "qpc_arnoldi_put_device": (ctypes.c_int, [P, P]),
        "qpc_arnoldi_get_device": (ctypes.c_int, [P, P]),
        "qpc_arnoldi_run": (ctypes.c_int, [P, P, i64, P, P, P]),
        "qpc_arnoldi_propagate": (ctypes.c_int, [P, P, P]),
        "qpc_arnoldi_norm": (ctypes.c_int, [P, P]),
        "qpc_arnoldi_last_run": (ctypes.c_int, [P, P, P]),
        "qpc_lgwz_dims": (ctypes.c_int, [P, P]),
        "qpc_lgwz_stream": (ctypes.c_int, [P, P]),
        "qpc_set_wait_limit": (ctypes.c_int, [d]),
        "qpc_fp64_peak": (ctypes.c_int, [P]),
        "qpc_get_wait_limit": (d, []),
        "qpc_vgwr_dims": (ctypes.c_int, [P, P]),
        "qpc_coulomb_f": (ctypes.c_int, [d, d, i32, P, P]),
        "qpc_coulomb_sigma": (ctypes.c_int, [d, i32, P]),
        "qpc_sph_legendre": (ctypes.c_int, [i32, d, P]),
        "qpc_pcs_tables": (ctypes.c_int, [P, P, P, d, d, P, P, P, P, P, P, P]),
        "qpc_pcs_tables_numeric": (ctypes.c_int, [P, P, P, P, P, P, P, P, P, P, P]),
        "qpc_tsurff_tables": (ctypes.c_int, [P, P, P, d, d, P, P, P, P, P, P, P, P, P, P, P, P]),
        "qpc_pcs_create": (ctypes.c_int, [P, P, P, P, P, P, P, P]),
        "qpc_pcs_destroy": (ctypes.c_int, [P]),
        "qpc_pcs_measure": (ctypes.c_int, [P, i32, P, i32, i32, P]),
        "qpc_lgwz_pcs": (ctypes.c_int, [P, P, i32, P]),
        "qpc_tsurff_create": (ctypes.c_int, [P, P, P, P, P, i32, P, P, P, P, P, P, P, P, P]),
        "qpc_tsurff_destroy": (ctypes.c_int, [P]),
        "qpc_tsurff_clear": (ctypes.c_int, [P]),
        "qpc_tsurff_accumulate": (ctypes.c_int, [P, i32, P, d, P, i32]),
        "qpc_lgwz_tsurff": (ctypes.c_int, [P, P, i32, P, d]),
        "qpc_vgwr_tsurff": (ctypes.c_int, [P, P, i32, P, d]),
        "qpc_tsurff_get": (ctypes.c_int, [P, P, P]),
        "qpc_pcs_last_run": (ctypes.c_int, [P, P]),
        "qpc_tsurff_last_run": (ctypes.c_int, [P, P]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _check(rc):
    if rc != QPC_OK:
        raise QpcError(rc, load().qpc_last_error().decode())


def set_wait_limit(seconds):
    """Bound of every host wait of the engine for the GPU (qpc_set_wait_limit)."""
    _check(load().qpc_set_wait_limit(float(seconds)))


def get_wait_limit():
    return float(load().qpc_get_wait_limit())


def fp64_peak():
    """FP64 FMA throughput of the current device in TFLOP/s (qpc_fp64_peak)."""
    v = ctypes.c_double(0)
    _check(load().qpc_fp64_peak(ctypes.byref(v)))
    return v.value


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


# ------------------------------------------------------------------ setup (host)

def linear_knots(n_r, p, rmin, rmax):
    t = np.zeros(n_r + p + 3)
    _check(load().qpc_linear_knots(n_r, p, rmin, rmax, _ptr(t)))
    return t


def radial_setup(n_r, p, n_lh, knots, potential=(POTENTIAL_HYDROGENIC, 1.0, 0.0, 0.0), mass=1.0):
    """S, R, Rinv, D as [n_r, p+1] bands and H as [n_lh, n_r, p+1]
    (integrator_radi integrals, spherical/utilities/basisfunc.hpp:63-106)."""
    knots = _f64(knots)
    pot = qpc_potential(*potential)
    S, R, Ri, D = (np.zeros((n_r, p + 1)) for _ in range(4))
    H = np.zeros((n_lh, n_r, p + 1))
    _check(load().qpc_radial_setup(n_r, p, n_lh, _ptr(knots), ctypes.byref(pot), mass,
                                   _ptr(S), _ptr(R), _ptr(Ri), _ptr(D), _ptr(H)))
    return S, R, Ri, D, H


def y10_coupling(n_l, m=0):
    y = np.zeros(n_l)
    _check(load().qpc_y10_coupling(n_l, m, _ptr(y)))
    return y


def y10_eigen(n_l, m=0):
    lam = np.zeros(n_l)
    P = np.zeros((n_l, n_l))
    _check(load().qpc_y10_eigen(n_l, m, _ptr(lam), _ptr(P)))
    return lam, P


def ldlt_csym(S, H, g):
    n, ne = S.shape
    p = ne - 1
    Lrow = np.zeros((n, p), complex)
    Dinv = np.zeros(n, complex)
    bad = load().qpc_ldlt_csym(n, p, _ptr(_f64(S)), _ptr(_f64(H)), g, _ptr(Lrow), _ptr(Dinv))
    if bad < 0:
        raise QpcError(1, "ldlt arguments")
    return Lrow, Dinv, bad


def gen_eigen(S, Hl, n_want=0):
    n, ne = S.shape
    e = np.zeros(n)
    v = np.zeros((max(n_want, 1), n))
    _check(load().qpc_gen_eigen(n, ne - 1, _ptr(_f64(S)), _ptr(_f64(Hl)), n_want, _ptr(e), _ptr(v)))
    return e, v[:n_want]


def ground_state(S, H, n_l, n_m=1, im=0, il=0, ir=0, m0=0):
    """coefficient::initialize for one (im, il, ir) with cf = 1: the state is the
    ir-th eigenvector of H_l in block (im, il), zero elsewhere; returns (coef, E)."""
    n_r = S.shape[0]
    l = il + abs(m0 + im)
    e, v = gen_eigen(S, H[l], ir + 1)
    c = np.zeros((n_m, n_l, n_r), complex)
    c[im, il] = v[ir]
    return c, e[ir]


def field_sinen(e0, w0, nc, n0, cep, dt, n_pow=2):
    """f(t_i), i = 0..para_nt, of field_component_sinen<n_pow> (CEP in units of pi)."""
    nt = ctypes.c_int64(0)
    _check(load().qpc_field_sinen(n_pow, e0, w0, nc, n0, cep, dt, 0, None, ctypes.byref(nt)))
    f = np.zeros(nt.value + 1)
    _check(load().qpc_field_sinen(n_pow, e0, w0, nc, n0, cep, dt, f.size, _ptr(f), ctypes.byref(nt)))
    return f


def intensity_to_e0(intensity_wcm2):
    """E0 [a.u.] = sqrt(I / 3.50944758e16 W/cm^2)."""
    return float(np.sqrt(intensity_wcm2 / 3.50944758e16))


def wavelength_to_w0(lambda_nm):
    """omega [a.u.] = 45.5633525 / lambda[nm]."""
    return 45.5633525 / lambda_nm


def fieldfree_factors(S, H, dt, lmax):
    """Host-packed LDL^T factors of S + i dt/2 H_l for l = 0..lmax, [lmax+1][n_r][p+1]
    complex128 (L(r, r-1-c) for c < p, 1/D(r) last), as qpc_fieldfree_noalloc takes them."""
    n_r, ne = S.shape
    p = ne - 1
    out = np.zeros((lmax + 1, n_r, ne), complex)
    for l in range(lmax + 1):
        Lrow, Dinv, bad = ldlt_csym(S, H[l], dt * 0.5)
        if bad:
            raise QpcError(4, "zero pivot factorising S + i dt/2 H_%d" % l)
        out[l, :, :p] = Lrow
        out[l, :, p] = Dinv
    return out


def fieldfree_noalloc(dims, S_dev, ffac_dev, coef_dev, stream=0):
    """qpc_fieldfree_noalloc on caller-owned device buffers (raw device pointers)."""
    _check(load().qpc_fieldfree_noalloc(ctypes.byref(dims), ctypes.c_void_p(S_dev), ctypes.c_void_p(ffac_dev),
                                        ctypes.c_void_p(coef_dev), ctypes.c_void_p(stream)))


def hhg_spectrum(z, dt, t0=0.0, tmin=None, tmax=None, dipole_type=1):
    """(omega, S(omega)) from a per-step dipole list (analysis/plot_hhs.m restated);
    the sin^2 window spans (tmin, tmax), by default the whole record."""
    z = _f64(z)
    n = z.size
    tmin = t0 if tmin is None else tmin
    tmax = t0 + dt * (n - 1) if tmax is None else tmax
    nh = (n + 1) // 2
    w, s = np.zeros(nh), np.zeros(nh)
    _check(load().qpc_hhg_spectrum(_ptr(z), n, t0, dt, tmin, tmax, dipole_type, _ptr(w), _ptr(s)))
    return w, s


def hhg_spectra(z, n, dt, kmax, t0=0.0, tmin=None, tmax=None, dipole_type=1):
    """hhg_spectrum of several dipole lists at once on the GPU (qpc_hhg_spectra): z [B][ld], n[B]
    samples each; returns S [B][kmax] at w_k = 2 pi k / (n[i] dt) (0 past ceil(n[i]/2)).  The window
    defaults to (t0, t0 + dt (n - 1)) per list."""
    z = _f64(np.atleast_2d(z))
    B = z.shape[0]
    n = np.ascontiguousarray(np.broadcast_to(n, (B,)), dtype=np.int64)
    tmin = _f64(np.broadcast_to(t0 if tmin is None else tmin, (B,)))
    tmax = _f64(t0 + dt * (n - 1.0) if tmax is None else np.broadcast_to(tmax, (B,)))
    out = np.zeros((B, int(kmax)))
    _check(load().qpc_hhg_spectra(B, _ptr(z), z.shape[1], _ptr(n), t0, dt, _ptr(tmin), _ptr(tmax), dipole_type, int(kmax), _ptr(out)))
    return out


def dgemm_slices(A, B, timed=False):
    """C = A B in FP64 on the tensor cores by exact bf16 digit slices (qpc_dgemm_slices), the
    product the velocity-gauge transforms use.  With timed=True also returns the device time in ms
    of splitting B and the product."""
    A, B = _f64(np.atleast_2d(A)), _f64(np.atleast_2d(B))
    n, K = A.shape
    if B.shape[0] != K:
        raise ValueError("inner dimensions differ: %s %s" % (A.shape, B.shape))
    M = B.shape[1]
    C = np.zeros((n, M))
    ms = np.zeros(1, np.float32)
    _check(load().qpc_dgemm_slices(n, M, K, _ptr(A), K, _ptr(B), M, _ptr(C), M, _ptr(ms)))
    return (C, float(ms[0])) if timed else C


def lspace_transform(V, c, forward=True):
    """The engine's l-space transform of c [n_pos][n_l] (complex) with the eigenvector table
    V [n_l/2 + 1][n_l], on the tensor cores in exact digits (qpc_lspace_transform, n_l <= 48)."""
    c = np.ascontiguousarray(np.atleast_2d(c), dtype=np.complex128)
    V = _f64(np.atleast_2d(V))
    n_pos, n_l = c.shape
    if V.shape != (n_l // 2 + 1, n_l):
        raise ValueError("V must be [n_l/2 + 1][n_l], got %s for n_l = %d" % (V.shape, n_l))
    out = np.zeros_like(c)
    _check(load().qpc_lspace_transform(n_pos, n_l, _ptr(V), 1 if forward else 0, _ptr(c), _ptr(out)))
    return out


def pes_bin(proj, energy, emin, emax, nbins, thres=0.0):
    """(pes[nbins], bound population, ionization yield) from projections and their energies."""
    pr = np.ascontiguousarray(proj, dtype=np.complex128)
    en = _f64(energy)
    pes = np.zeros(max(nbins, 1))
    b, y = ctypes.c_double(0), ctypes.c_double(0)
    _check(load().qpc_pes_bin(_ptr(pr), _ptr(en), pr.size, emin, emax, nbins, thres, _ptr(pes), ctypes.byref(b), ctypes.byref(y)))
    return pes[:nbins], b.value, y.value


def left_eigenbasis(S, H, lmax, emax):
    """eigenstate_sph::initialize (population_1e.hpp:58-118): per l = 0..lmax the field-free
    eigenstates with E < emax, stored as left vectors S v; returns (n_state, basis list, energies)."""
    n_r, ne = S.shape
    p = ne - 1
    n_state, basis, energies = [], [], []
    for l in range(lmax + 1):
        e, _ = gen_eigen(S, H[l], 0)
        k = int((e < emax).sum())
        e, v = gen_eigen(S, H[l], k)
        Sv = np.zeros_like(v)
        for j in range(k):
            x = v[j]
            y = S[:, 0] * x
            for d in range(1, p + 1):
                y[:-d] += S[:-d, d] * x[d:]
                y[d:] += S[:-d, d] * x[:-d]
            Sv[j] = y
        n_state.append(k)
        basis.append(Sv)
        energies.append(e[:k])
    return np.array(n_state, np.int32), basis, energies


# ------------------------------------------------------------------ propagator

class propagator_cn_hc_lgwz:
    """Batched GPU propagator_cn_hc_lgwz: n_inst wavefunctions on one grid.

    initialize(...) mirrors propagator_cn_hc_lgwz::initialize (cn_1e.hpp:565-593);
    propagate(f_ti, f_tf) / propagate() mirror the two propagate overloads
    (cn_1e.hpp:595-618) for every instance at once; run(...) is the driver loop.
    The state lives on the GPU; put()/get() copy c[inst][m][l][r] complex128.
    """

    def __init__(self):
        self._h = None
        self.dims = None

    def initialize(self, n_r, p, n_l, S, R, H, dt, n_m=1, m0=0, n_inst=1):
        """H: [lmax+1][n_r][p+1] shared by the batch, or [n_inst][lmax+1][n_r][p+1] (own potentials)"""
        lib = load()
        self.close()
        d = qpc_dims(n_r, p, n_l, n_m, m0, n_inst)
        h = ctypes.c_void_p()
        S, R, H = _f64(S), _f64(R), _f64(H)
        lmax = max(abs(m0), abs(m0 + n_m - 1)) + n_l - 1
        per_inst = H.ndim == 4      # H[inst][l][r][k]: one potential per wavefunction (qpc_lgwz_create_ex)
        if per_inst and H.shape[0] != n_inst:
            raise QpcError(1, "H has %d potentials for %d instances" % (H.shape[0], n_inst))
        if H.shape[-3] < lmax + 1:
            raise QpcError(1, "H needs lmax+1 = %d blocks" % (lmax + 1))
        Hc = _f64(H[:, :lmax + 1] if per_inst else H[:lmax + 1])
        _check(lib.qpc_lgwz_create_ex(ctypes.byref(d), dt, _ptr(S), _ptr(R), _ptr(Hc), int(per_inst), ctypes.byref(h)))
        self._h = h
        self.dims = d
        self.shape = (n_inst, n_m, n_l, n_r)
        return self

    def close(self):
        if self._h is not None:
            load().qpc_lgwz_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def put(self, coef):
        c = np.ascontiguousarray(coef, dtype=np.complex128).reshape(self.shape)
        _check(load().qpc_lgwz_put(self._h, _ptr(c)))

    def get(self):
        c = np.zeros(self.shape, np.complex128)
        _check(load().qpc_lgwz_get(self._h, _ptr(c)))
        return c

    def stream(self):
        """The handle's cudaStream_t as an integer (qpc_lgwz_stream)."""
        v = ctypes.c_void_p()
        _check(load().qpc_lgwz_stream(self._h, ctypes.byref(v)))
        return int(v.value or 0)

    def put_device(self, dev_ptr):
        _check(load().qpc_lgwz_put_device(self._h, ctypes.c_void_p(dev_ptr)))

    def get_device(self, dev_ptr):
        _check(load().qpc_lgwz_get_device(self._h, ctypes.c_void_p(dev_ptr)))

    def propagate(self, f_ti=None, f_tf=None):
        if f_ti is None:
            _check(load().qpc_lgwz_propagate_free(self._h))
            return
        a = _f64(np.broadcast_to(f_ti, (self.shape[0],)))
        b = _f64(np.broadcast_to(f_tf, (self.shape[0],)))
        _check(load().qpc_lgwz_propagate(self._h, _ptr(a), _ptr(b)))

    def run(self, ftab, nt_field, nt_total=None):
        nt_field = np.ascontiguousarray(np.broadcast_to(nt_field, (self.shape[0],)), dtype=np.int64)
        nt_total = nt_field.copy() if nt_total is None else np.ascontiguousarray(
            np.broadcast_to(nt_total, (self.shape[0],)), dtype=np.int64)
        if ftab is None:
            _check(load().qpc_lgwz_run(self._h, None, 1, _ptr(nt_field), _ptr(nt_total)))
            return
        ftab = _f64(np.atleast_2d(ftab))
        if ftab.shape[0] != self.shape[0]:
            ftab = _f64(np.broadcast_to(ftab, (self.shape[0], ftab.shape[1])))
        _check(load().qpc_lgwz_run(self._h, _ptr(ftab), ftab.shape[1], _ptr(nt_field), _ptr(nt_total)))

    def run_ex(self, ftab, nt_field, nt_total=None, mask=None, tsurff=None):
        """run() with, after every step of every instance, the t-SURFF accumulate into `tsurff`
        (a spectrum_c_tsf over the same grid and batch) and then the absorbing mask `mask`
        (a band from mask_band), as the reference's driver loop applies them
        (binsrc/sphTDSE.cpp:797-810), all on the device."""
        nt_field = np.ascontiguousarray(np.broadcast_to(nt_field, (self.shape[0],)), dtype=np.int64)
        nt_total = nt_field.copy() if nt_total is None else np.ascontiguousarray(
            np.broadcast_to(nt_total, (self.shape[0],)), dtype=np.int64)
        mk = None if mask is None else _f64(mask)
        opts = qpc_run_opts(None if mk is None else mk.ctypes.data, None if tsurff is None else tsurff._h.value)
        if ftab is None:
            tab, ld = None, 1
        else:
            tab = _f64(np.atleast_2d(ftab))
            if tab.shape[0] != self.shape[0]:
                tab = _f64(np.broadcast_to(tab, (self.shape[0], tab.shape[1])))
            ld = tab.shape[1]
        _check(load().qpc_lgwz_run_ex(self._h, _ptr(tab), ld, _ptr(nt_field), _ptr(nt_total), ctypes.byref(opts)))

    def run_dipole(self, ftab, nt_field, nt_total, F):
        """run() that also returns zlist[inst, s] = <psi(t_s)| f(r) cos(theta) |psi(t_s)>
        for s < nt_total[inst] (F = <B|f|B>, f(r) = r for the dipole)."""
        nt_field = np.ascontiguousarray(np.broadcast_to(nt_field, (self.shape[0],)), dtype=np.int64)
        nt_total = np.ascontiguousarray(np.broadcast_to(nt_total, (self.shape[0],)), dtype=np.int64)
        ldz = int(max(1, nt_total.max()))
        z = np.zeros((self.shape[0], ldz))
        if ftab is None:
            tab, ld = None, 1
        else:
            tab = _f64(np.atleast_2d(ftab))
            if tab.shape[0] != self.shape[0]:
                tab = _f64(np.broadcast_to(tab, (self.shape[0], tab.shape[1])))
            ld = tab.shape[1]
        _check(load().qpc_lgwz_run_dipole(self._h, _ptr(tab), ld, _ptr(nt_field), _ptr(nt_total),
                                          _ptr(_f64(F)), _ptr(z), ldz))
        return z

    def last_run_ms(self):
        v = ctypes.c_double(0)
        _check(load().qpc_lgwz_last_run_ms(self._h, ctypes.byref(v)))
        return v.value

    def launch_count(self):
        return int(load().qpc_lgwz_launch_count(self._h))

    def enable_profiling(self, on=True):
        _check(load().qpc_lgwz_set_profiling(self._h, int(bool(on))))

    def tuning(self):
        """{"lookahead": K, "coupling": {bucket: G}, "fieldfree": {bucket: G}} (G = lanes per part, -1 = the
        segmented solver)."""
        out = np.zeros(65, np.int32)
        _check(load().qpc_lgwz_get_tuning(self._h, _ptr(out)))
        return {"lookahead": int(out[0]),
                "coupling": {b: int(out[1 + b]) for b in range(32) if out[1 + b]},
                "fieldfree": {b: int(out[33 + b]) for b in range(32) if out[33 + b]}}

    def kernel_times(self):
        """{kernel: (total ms, launches)} accumulated by run() while profiling is on."""
        ms = np.zeros(len(KERNELS))
        n = np.zeros(len(KERNELS), np.int64)
        _check(load().qpc_lgwz_kernel_times(self._h, _ptr(ms), _ptr(n)))
        return {k: (float(ms[i]), int(n[i])) for i, k in enumerate(KERNELS)}

    def norm(self):
        out = np.zeros(self.shape[0])
        _check(load().qpc_lgwz_norm(self._h, _ptr(out)))
        return out

    def mask(self, M):
        """absorber_mask::operator()(coef, s) on every wavefunction: c <- S^-1 (M c) per channel."""
        _check(load().qpc_lgwz_mask(self._h, _ptr(_f64(M))))

    def dipole(self, F):
        out = np.zeros(2 * self.shape[0])
        _check(load().qpc_lgwz_dipole(self._h, _ptr(_f64(F)), _ptr(out)))
        return out[0::2] + 1j * out[1::2]

    def projection(self, n_state, basis):
        """basis: list over l = 0..lmax of arrays [n_state[l], n_r] (S v rows)."""
        n_state = np.ascontiguousarray(n_state, dtype=np.int32)
        packed = _f64(np.concatenate([np.asarray(b, np.float64).reshape(-1) for b in basis]))
        B, M, L, N = self.shape
        tot = 0
        for im in range(M):
            for il in range(L):
                tot += int(n_state[il + abs(self.dims.m0 + im)])
        out = np.zeros(B * tot, complex)
        _check(load().qpc_lgwz_projection(self._h, _ptr(n_state), _ptr(packed), _ptr(out)))
        return out


def run_many(props, ftabs, nt_field, nt_total=None):
    """propagator_cn_hc_lgwz.run on several handles at once (qpc_lgwz_run_many): one host
    thread per handle, so that batches on different grids share the GPU."""
    n = len(props)
    keep = []
    H = (ctypes.c_void_p * n)()
    F = (ctypes.c_void_p * n)()
    LD = np.zeros(n, np.int64)
    NF = (ctypes.c_void_p * n)()
    NT = (ctypes.c_void_p * n)()
    for i, pr in enumerate(props):
        B = pr.shape[0]
        nf = np.ascontiguousarray(np.broadcast_to(nt_field[i], (B,)), dtype=np.int64)
        ntt = nf.copy() if nt_total is None else np.ascontiguousarray(np.broadcast_to(nt_total[i], (B,)), dtype=np.int64)
        tab = _f64(np.atleast_2d(ftabs[i]))
        if tab.shape[0] != B:
            tab = _f64(np.broadcast_to(tab, (B, tab.shape[1])))
        keep += [nf, ntt, tab]
        H[i] = pr._h.value
        F[i] = tab.ctypes.data
        LD[i] = tab.shape[1]
        NF[i] = nf.ctypes.data
        NT[i] = ntt.ctypes.data
    failed = ctypes.c_int32(-1)
    _check(load().qpc_lgwz_run_many(n, H, F, _ptr(LD), NF, NT, ctypes.byref(failed)))


VGWR_COMPONENTS = ("x1", "x2", "y1", "y2")


def vgwr_angular(n_l, n_m, m0, comp):
    """(lam[N_ch], P[N_ch][N_ch] complex) of coupling component comp (0..3 = x1, x2, y1, y2)
    of propagator_cn_hc_vgwr: P Z P^H = diag(lam)."""
    N = n_l * n_m
    lam = np.zeros(N)
    P = np.zeros((N, N), complex)
    _check(load().qpc_vgwr_angular(n_l, n_m, m0, comp, _ptr(lam), _ptr(P)))
    return lam, P


def mask_band(n_r, p, knots, rmin, rmax, index=1.0 / 6.0):
    """absorber_mask::initialize (absorber.hpp:42-49): <B_i|m(r)|B_j>, m = |cos(pi/2 (r-rmin)/(rmax-rmin))|^index."""
    kn = _f64(knots)
    M = np.zeros((n_r, p + 1))
    _check(load().qpc_mask_band(n_r, p, _ptr(kn), rmin, rmax, index, _ptr(M)))
    return M


def cholesky_band(S, p):
    """S = L L^T, L(r+k, r) at [r, k] (operator_sc::cholesky(), operators/1e.hpp:1233-1244)."""
    S = _f64(S)
    n = S.size // (p + 1)
    L = np.zeros((n, p + 1))
    rc = load().qpc_cholesky_band(n, p, _ptr(S), _ptr(L))
    if rc:
        raise QpcError(4 if rc > 0 else 1, "cholesky_band: %d" % rc)
    return L


class propagator_hc_lgwz:
    """Batched GPU Arnoldi propagator, propagator_hc_lgwz of spherical/propagator/la_1e.hpp:390-444
    with propagate<1>(coef, dt) (propagator_arnoldi::propagate1, la_1e.hpp:312-335).

    propagator_hc_lgwz(kmax, emin, emax) mirrors the constructor (arnoldi_workspace,
    la_1e.hpp:54-62); initialize(...) takes the grid, the bands and dt; the field
    member ez of the reference class is given per instance to propagate(ez) or as a
    table to run().  H may be [lmax+1][n_r][p+1] (shared) or [n_inst][lmax+1][n_r][p+1]
    (one potential per wavefunction).  propagate() and run() return the criterion()
    codes (0: dt should be smaller, 1: keep, 2: dt may grow).
    """

    def __init__(self, kmax, emin, emax):
        if not (emin <= emax and emin > 0 and emax > 0):
            raise QpcError(1, "invalid parameters for arnoldi propagator")
        self.kmax, self.emin, self.emax = int(kmax), float(emin), float(emax)
        self._h = None
        self.ez = 0.0

    def initialize(self, n_r, p, n_l, S, R, H, y10, dt, n_m=1, m0=0, n_inst=1):
        lib = load()
        self.close()
        d = qpc_dims(n_r, p, n_l, n_m, m0, n_inst)
        lmax = max(abs(m0), abs(m0 + n_m - 1)) + n_l - 1
        H = _f64(H)
        per = H.ndim == 4
        H = _f64(H[:, :lmax + 1] if per else H[:lmax + 1])
        y10 = _f64(np.broadcast_to(np.asarray(y10, np.float64).reshape(-1, n_l), (n_m, n_l)))
        h = ctypes.c_void_p()
        _check(lib.qpc_arnoldi_create(ctypes.byref(d), _ptr(_f64(S)), _ptr(_f64(R)), _ptr(H), int(per), _ptr(y10),
                                      float(dt), self.kmax, self.emin, self.emax, ctypes.byref(h)))
        self._h = h
        self.dims = d
        self.dt = float(dt)
        self.shape = (n_inst, n_m, n_l, n_r)
        return self

    def close(self):
        if self._h is not None:
            load().qpc_arnoldi_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def put(self, coef):
        c = np.ascontiguousarray(coef, dtype=np.complex128).reshape(self.shape)
        _check(load().qpc_arnoldi_put(self._h, _ptr(c)))

    def get(self):
        c = np.zeros(self.shape, np.complex128)
        _check(load().qpc_arnoldi_get(self._h, _ptr(c)))
        return c

    def put_device(self, dev_ptr):
        _check(load().qpc_arnoldi_put_device(self._h, ctypes.c_void_p(dev_ptr)))

    def get_device(self, dev_ptr):
        _check(load().qpc_arnoldi_get_device(self._h, ctypes.c_void_p(dev_ptr)))

    def propagate(self, ez=None):
        ez = self.ez if ez is None else ez
        e = _f64(np.broadcast_to(ez, (self.shape[0],)))
        crit = np.zeros(self.shape[0], np.int8)
        _check(load().qpc_arnoldi_propagate(self._h, _ptr(e), _ptr(crit)))
        return crit

    def run(self, eztab, nt=None, want_msub=False):
        """eztab[inst, s] = ez during step s; nt[inst] steps (default: all columns).
        Returns crit[inst, s] (and msub[inst, s]); -1 where an instance took no step."""
        tab = _f64(np.atleast_2d(eztab))
        if tab.shape[0] != self.shape[0]:
            tab = _f64(np.broadcast_to(tab, (self.shape[0], tab.shape[1])))
        ld = tab.shape[1]
        nt = np.full(self.shape[0], ld, np.int64) if nt is None else np.ascontiguousarray(
            np.broadcast_to(nt, (self.shape[0],)), dtype=np.int64)
        crit = np.zeros((self.shape[0], ld), np.int8)
        ms = np.zeros((self.shape[0], ld), np.int8)
        _check(load().qpc_arnoldi_run(self._h, _ptr(tab), ld, _ptr(nt), _ptr(crit), _ptr(ms)))
        return (crit, ms) if want_msub else crit

    def norm(self):
        out = np.zeros(self.shape[0])
        _check(load().qpc_arnoldi_norm(self._h, _ptr(out)))
        return out

    def last_run(self):
        """(device ms of the last run, kernel launches it made)"""
        ms = ctypes.c_float(0)
        n = ctypes.c_int64(0)
        _check(load().qpc_arnoldi_last_run(self._h, ctypes.byref(ms), ctypes.byref(n)))
        return ms.value, n.value


class mlp_ensemble:
    """GPU-trained ensemble MLP (qpc_mlp): members x (n_in -> n_layers x n_hidden GELU -> n_out),
    bf16 operands with fp32 accumulation, Adam."""

    def __init__(self, n_in, n_out, n_hidden=256, n_layers=4, n_members=5, seed=0):
        self._h = None
        h = ctypes.c_void_p()
        _check(load().qpc_mlp_create(n_in, n_hidden, n_layers, n_out, n_members, ctypes.c_uint64(seed), ctypes.byref(h)))
        self._h = h
        self.n_in, self.n_out, self.n_hidden, self.n_layers, self.n_members = n_in, n_out, n_hidden, n_layers, n_members
        n = ctypes.c_int64(0)
        _check(load().qpc_mlp_param_count(h, ctypes.byref(n)))
        self.n_params = n.value

    def close(self):
        if self._h is not None:
            load().qpc_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def get_params(self, member):
        out = np.zeros(self.n_params, np.float32)
        _check(load().qpc_mlp_get_params(self._h, member, _ptr(out)))
        return out

    def set_params(self, member, flat):
        f = np.ascontiguousarray(flat, dtype=np.float32)
        assert f.size == self.n_params
        _check(load().qpc_mlp_set_params(self._h, member, _ptr(f)))

    def loss_grad(self, X, Y):
        X = np.ascontiguousarray(X, dtype=np.float32)
        Y = np.ascontiguousarray(Y, dtype=np.float32)
        loss = np.zeros(self.n_members, np.float32)
        grad = np.zeros((self.n_members, self.n_params), np.float32)
        _check(load().qpc_mlp_loss_grad(self._h, _ptr(X), _ptr(Y), X.shape[0], _ptr(loss), _ptr(grad)))
        return loss, grad

    def train(self, X, Y, epochs, batch=256, lr=1e-3, seed=1):
        X = np.ascontiguousarray(X, dtype=np.float32)
        Y = np.ascontiguousarray(Y, dtype=np.float32)
        hist = np.zeros((epochs, self.n_members), np.float32)
        _check(load().qpc_mlp_train(self._h, _ptr(X), _ptr(Y), X.shape[0], epochs, batch, ctypes.c_float(lr),
                                    ctypes.c_uint64(seed), _ptr(hist)))
        return hist

    def predict(self, X):
        """[members][n][n_out]"""
        X = np.ascontiguousarray(X, dtype=np.float32)
        out = np.zeros((self.n_members, X.shape[0], self.n_out), np.float32)
        _check(load().qpc_mlp_predict(self._h, _ptr(X), X.shape[0], _ptr(out)))
        return out


class propagator_cn_hc_vgwr:
    """Batched GPU propagator_cn_hc_vgwr (velocity gauge, elliptical; cn_1e.hpp:812-951).

    initialize(...) mirrors the reference's initialize (S, 1/r, D = <B|d/dr|B>, H_l per l);
    propagate(ax_ti, ax_tf, ay_ti, ay_tf) and propagate() the two overloads (cn_1e.hpp:903-950)
    for every instance; run(atab, nt_field, nt_total) the driver loop with atab[inst, s] =
    (A_x(t_s), A_y(t_s)).  State c[inst][m][l][r] complex128."""

    def __init__(self):
        self._h = None

    def initialize(self, n_r, p, n_l, n_m, m0, S, Rinv, D, H, dt, n_inst=1):
        lib = load()
        self.close()
        d = qpc_dims(n_r, p, n_l, n_m, m0, n_inst)
        lmax = max(abs(m0), abs(m0 + n_m - 1)) + n_l - 1
        H = _f64(H)
        if H.shape[0] < lmax + 1:
            raise QpcError(1, "H needs lmax+1 = %d blocks" % (lmax + 1))
        h = ctypes.c_void_p()
        _check(lib.qpc_vgwr_create(ctypes.byref(d), dt, _ptr(_f64(S)), _ptr(_f64(Rinv)), _ptr(_f64(D)), _ptr(_f64(H[:lmax + 1])),
                                   ctypes.byref(h)))
        self._h = h
        self.dims = d
        self.shape = (n_inst, n_m, n_l, n_r)
        return self

    def close(self):
        if self._h is not None:
            load().qpc_vgwr_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def put(self, coef):
        c = np.ascontiguousarray(coef, dtype=np.complex128).reshape(self.shape)
        _check(load().qpc_vgwr_put(self._h, _ptr(c)))

    def get(self):
        c = np.zeros(self.shape, np.complex128)
        _check(load().qpc_vgwr_get(self._h, _ptr(c)))
        return c

    def propagate(self, ax_ti=None, ax_tf=None, ay_ti=None, ay_tf=None):
        if ax_ti is None:
            _check(load().qpc_vgwr_propagate_free(self._h))
            return
        B = self.shape[0]
        a = [_f64(np.broadcast_to(v, (B,))) for v in (ax_ti, ax_tf, ay_ti, ay_tf)]
        _check(load().qpc_vgwr_propagate(self._h, *[_ptr(v) for v in a]))

    def run(self, atab, nt_field, nt_total=None):
        """atab [inst][steps+1][2] (A_x, A_y at t_s)"""
        B = self.shape[0]
        tab = _f64(np.asarray(atab, np.float64).reshape(-1 if np.ndim(atab) == 3 else 1, np.shape(atab)[-2], 2))
        if tab.shape[0] != B:
            tab = _f64(np.broadcast_to(tab, (B,) + tab.shape[1:]))
        nf = np.ascontiguousarray(np.broadcast_to(nt_field, (B,)), dtype=np.int64)
        ntt = nf.copy() if nt_total is None else np.ascontiguousarray(np.broadcast_to(nt_total, (B,)), dtype=np.int64)
        _check(load().qpc_vgwr_run(self._h, _ptr(tab), tab.shape[1], _ptr(nf), _ptr(ntt)))

    def run_dipole(self, atab, nt_field, nt_total, F):
        """run() that also returns (x, y)[inst, s] = <psi(t_s)| f(r) sin(theta) (cos, sin)(phi) |psi(t_s)>
        for s < nt_total[inst] (observable_r; F = <B|f|B>, f(r) = r for the dipole)."""
        B = self.shape[0]
        nf = np.ascontiguousarray(np.broadcast_to(nt_field, (B,)), dtype=np.int64)
        ntt = np.ascontiguousarray(np.broadcast_to(nt_total, (B,)), dtype=np.int64)
        ldz = int(max(1, ntt.max()))
        x = np.zeros((B, ldz))
        y = np.zeros((B, ldz))
        if atab is None:
            tab, ld = None, 1
        else:
            tab = _f64(np.asarray(atab, np.float64).reshape(-1 if np.ndim(atab) == 3 else 1, np.shape(atab)[-2], 2))
            if tab.shape[0] != B:
                tab = _f64(np.broadcast_to(tab, (B,) + tab.shape[1:]))
            ld = tab.shape[1]
        _check(load().qpc_vgwr_run_dipole(self._h, _ptr(tab), ld, _ptr(nf), _ptr(ntt), _ptr(_f64(F)), _ptr(x), _ptr(y), ldz))
        return x, y

    def norm(self):
        out = np.zeros(self.shape[0])
        _check(load().qpc_vgwr_norm(self._h, _ptr(out)))
        return out

    def last_run(self):
        ms = ctypes.c_float(0)
        n = ctypes.c_int64(0)
        _check(load().qpc_vgwr_last_run(self._h, ctypes.byref(ms), ctypes.byref(n)))
        return ms.value, n.value

    def enable_profiling(self, on=True):
        _check(load().qpc_vgwr_set_profiling(self._h, int(bool(on))))

    def kernel_times(self):
        """{"transform" | "coupling" | "fieldfree": (total ms, launch groups)} of run() while profiling is on."""
        ms = np.zeros(3)
        n = np.zeros(3, np.int64)
        _check(load().qpc_vgwr_kernel_times(self._h, _ptr(ms), _ptr(n)))
        return {k: (float(ms[i]), int(n[i])) for i, k in enumerate(("transform", "coupling", "fieldfree"))}



# ------------------------------------------------------------------ momentum spectra

def coulomb_f(eta, rho, lmax):
    """F_l(eta, rho) and dF_l/drho for l = 0..lmax (functions/coulomb.h, coulombfg)."""
    F, Fp = np.zeros(lmax + 1), np.zeros(lmax + 1)
    _check(load().qpc_coulomb_f(eta, rho, lmax, _ptr(F), _ptr(Fp)))
    return F, Fp


def coulomb_sigma(eta, lmax):
    """arg Gamma(l + 1 + i eta), l = 0..lmax (coulomb_sig_real)."""
    out = np.zeros(lmax + 1)
    _check(load().qpc_coulomb_sigma(eta, lmax, _ptr(out)))
    return out


def sph_legendre(lmax, x):
    """Y_lm(theta, 0) at x = cos(theta), array index l(l+1)/2 + m (legendre::cal, functions/basis_legendre.h)."""
    out = np.zeros((lmax + 1) * (lmax + 2) // 2)
    _check(load().qpc_sph_legendre(lmax, x, _ptr(out)))
    return out


def _kgrid(nkr, nkt, nkp, krmin, krmax, ktmin, ktmax, kpmin, kpmax, flag):
    return qpc_kgrid(nkr, nkt, nkp, krmin, krmax, ktmin, ktmax, kpmin, kpmax, flag)


def _lmax(n_l, n_m, m0):
    return max(abs(m0), abs(m0 + n_m - 1)) + n_l - 1


def pcs_tables(n_r, p, n_l, knots, nkr, nkt, nkp, krmin, krmax, ktmin, ktmax, kpmin, kpmax, zc, rb=0.0, flag=0, n_m=1, m0=0):
    """spectrum_c_pcs::initialize (analytic Coulomb waves; spherical/spectrum/momentum_1e.hpp:453-485):
    dict of kr, kt, kp, ijl [nkr][lmax+1][n_r], plm [nkt][n_m][n_l], exm [nkp][n_m], cps [nkr][lmax+1]."""
    d = qpc_dims(n_r, p, n_l, n_m, m0, 1)
    g = _kgrid(nkr, nkt, nkp, krmin, krmax, ktmin, ktmax, kpmin, kpmax, flag)
    nl = _lmax(n_l, n_m, m0) + 1
    t = {"kr": np.zeros(nkr), "kt": np.zeros(nkt), "kp": np.zeros(nkp), "ijl": np.zeros((nkr, nl, n_r)),
         "plm": np.zeros((nkt, n_m, n_l)), "exm": np.zeros((nkp, n_m), complex), "cps": np.zeros((nkr, nl), complex)}
    _check(load().qpc_pcs_tables(ctypes.byref(d), _ptr(_f64(knots)), ctypes.byref(g), zc, rb, *[_ptr(t[k]) for k in
                                 ("kr", "kt", "kp", "ijl", "plm", "exm", "cps")]))
    return t


def pcs_tables_numeric(n_r, p, n_l, knots, nkr, nkt, nkp, krmin, krmax, ktmin, ktmax, kpmin, kpmax, potential, flag=0, n_m=1, m0=0):
    """spectrum_c_pcs::initialize with numerical partial waves of V = -(zc + zs e^{-sigma r})/r
    (potential = (kind, zc, zs, sigma) as radial_setup takes it); same dict as pcs_tables."""
    d = qpc_dims(n_r, p, n_l, n_m, m0, 1)
    g = _kgrid(nkr, nkt, nkp, krmin, krmax, ktmin, ktmax, kpmin, kpmax, flag)
    pot = qpc_potential(*potential)
    nl = _lmax(n_l, n_m, m0) + 1
    t = {"kr": np.zeros(nkr), "kt": np.zeros(nkt), "kp": np.zeros(nkp), "ijl": np.zeros((nkr, nl, n_r)),
         "plm": np.zeros((nkt, n_m, n_l)), "exm": np.zeros((nkp, n_m), complex), "cps": np.zeros((nkr, nl), complex)}
    _check(load().qpc_pcs_tables_numeric(ctypes.byref(d), _ptr(_f64(knots)), ctypes.byref(g), ctypes.byref(pot),
                                         *[_ptr(t[k]) for k in ("kr", "kt", "kp", "ijl", "plm", "exm", "cps")]))
    return t


def tsurff_tables(n_r, p, n_l, knots, r0, zc, nkr, nkt, nkp, krmin, krmax, ktmin, ktmax, kpmin, kpmax, flag=0, n_m=1, m0=0):
    """spectrum_c_tsf::initialize (spherical/spectrum/momentum_1e.hpp:778-866): dict of kr, kt, kp,
    ib, b0, br (splines non-zero at r0), j0, jr [nkr][lmax+1], y0 [nkt][n_m][n_l], e0 [nkp][n_m],
    pmat [3][n_m][n_l]."""
    d = qpc_dims(n_r, p, n_l, n_m, m0, 1)
    g = _kgrid(nkr, nkt, nkp, krmin, krmax, ktmin, ktmax, kpmin, kpmax, flag)
    nl = _lmax(n_l, n_m, m0) + 1
    t = {"kr": np.zeros(nkr), "kt": np.zeros(nkt), "kp": np.zeros(nkp), "ib": np.zeros(p + 1, np.int32),
         "b0": np.zeros(p + 1), "br": np.zeros(p + 1), "j0": np.zeros((nkr, nl)), "jr": np.zeros((nkr, nl)),
         "y0": np.zeros((nkt, n_m, n_l)), "e0": np.zeros((nkp, n_m), complex), "pmat": np.zeros((3, n_m, n_l))}
    nb = ctypes.c_int32(0)
    _check(load().qpc_tsurff_tables(ctypes.byref(d), _ptr(_f64(knots)), ctypes.byref(g), r0, zc, _ptr(t["kr"]), _ptr(t["kt"]),
                                    _ptr(t["kp"]), ctypes.byref(nb), _ptr(t["ib"]), _ptr(t["b0"]), _ptr(t["br"]), _ptr(t["j0"]),
                                    _ptr(t["jr"]), _ptr(t["y0"]), _ptr(t["e0"]), _ptr(t["pmat"])))
    for k in ("ib", "b0", "br"):
        t[k] = t[k][:nb.value].copy()
    return t


class spectrum_c_pcs:
    """Photoelectron momentum spectra by projection onto Coulomb partial waves on the GPU
    (spectrum_c_pcs<dims_t, nkr, nkt, nkp>, spherical/spectrum/momentum_1e.hpp:443-514).

    initialize(...) builds the tables (pcs_tables; the grid is given by its knots instead of an
    integrator_radi) and uploads them; measure_lmd / measure_prj / measure_pad(coef) mirror the
    reference's members for a batch coef[inst][m][l][r] (host array, or a propagator_cn_hc_lgwz
    whose resident state is measured)."""

    def __init__(self, nkr, nkt, nkp):
        self.nkr, self.nkt, self.nkp = nkr, nkt, nkp
        self._h = None

    def initialize(self, n_r, p, n_l, knots, krmin, krmax, thmin, thmax, phmin, phmax, zc, rb=0.0, flag=0, n_m=1, m0=0, tables=None,
                   potential=None):
        """potential = (kind, zc, zs, sigma) selects the numerical partial waves of that potential
        (pcs_tables_numeric, the reference's numerical PCS); otherwise analytic Coulomb waves of charge
        zc with the cut-off rb (pcs_tables)."""
        lib = load()
        self.close()
        if tables is not None:
            t = tables
        elif potential is not None:
            t = pcs_tables_numeric(n_r, p, n_l, knots, self.nkr, self.nkt, self.nkp, krmin, krmax, thmin, thmax, phmin, phmax, potential,
                                   flag, n_m, m0)
        else:
            t = pcs_tables(n_r, p, n_l, knots, self.nkr, self.nkt, self.nkp, krmin, krmax, thmin, thmax, phmin, phmax, zc, rb, flag, n_m, m0)
        d = qpc_dims(n_r, p, n_l, n_m, m0, 1)
        g = _kgrid(self.nkr, self.nkt, self.nkp, krmin, krmax, thmin, thmax, phmin, phmax, flag)
        h = ctypes.c_void_p()
        _check(lib.qpc_pcs_create(ctypes.byref(d), ctypes.byref(g), _ptr(_f64(t["kr"])), _ptr(_f64(t["ijl"])), _ptr(_f64(t["plm"])),
                                  _ptr(np.ascontiguousarray(t["exm"], np.complex128)), _ptr(np.ascontiguousarray(t["cps"], np.complex128)),
                                  ctypes.byref(h)))
        self._h, self.tables, self.shape = h, t, (n_m, n_l, n_r)
        self.kr, self.kt, self.kp = t["kr"], t["kt"], t["kp"]
        return self

    def close(self):
        if self._h is not None:
            load().qpc_pcs_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _measure(self, kind, coef):
        n_m, n_l, _ = self.shape
        shapes = {SPEC_LMD: (self.nkr, n_m, n_l), SPEC_PMD: (self.nkr, self.nkt, self.nkp), SPEC_PAD: (self.nkr, self.nkt)}
        if isinstance(coef, propagator_cn_hc_lgwz):
            out = np.zeros((coef.shape[0],) + shapes[kind], np.complex128)
            _check(load().qpc_lgwz_pcs(coef._h, self._h, kind, _ptr(out)))
            return out
        c = np.ascontiguousarray(coef, dtype=np.complex128).reshape((-1,) + self.shape)
        out = np.zeros((c.shape[0],) + shapes[kind], np.complex128)
        _check(load().qpc_pcs_measure(self._h, kind, _ptr(c), 0, c.shape[0], _ptr(out)))
        return out

    def measure_lmd(self, coef):
        """[inst][kr][m][l] partial-wave amplitudes (measure_lmd, momentum_1e.hpp:386-403)"""
        return self._measure(SPEC_LMD, coef)

    def measure_prj(self, coef):
        """[inst][kr][kt][kp] momentum amplitudes (measure_prj, momentum_1e.hpp:337-355)"""
        return self._measure(SPEC_PMD, coef)

    def measure_pad(self, coef):
        """[inst][kr][kt] (measure_pad, momentum_1e.hpp:358-383)"""
        return self._measure(SPEC_PAD, coef)

    def last_run_ms(self):
        """device time of the last measurement's kernels"""
        ms = ctypes.c_float(0)
        _check(load().qpc_pcs_last_run(self._h, ctypes.byref(ms)))
        return ms.value


class spectrum_c_tsf:
    """t-SURFF momentum spectra on the GPU (spectrum_c_tsf, spherical/spectrum/momentum_1e.hpp:516-1072)
    for n_inst wavefunctions: initialize(...) at the surface r0; accumulate(coef, dt, a) after every
    step with a = None (field-free), a[inst][2] = (A_z(t_i), A_z(t_i+1)) or a[inst][4] =
    (A_x(t_i), A_x(t_i+1), A_y(t_i), A_y(t_i+1)); coef is a host array [inst][m][l][r] or a
    propagator handle (propagator_cn_hc_lgwz, propagator_cn_hc_vgwr) whose resident state is used."""

    def __init__(self, nkr, nkt, nkp):
        self.nkr, self.nkt, self.nkp = nkr, nkt, nkp
        self._h = None

    def initialize(self, n_r, p, n_l, knots, r0, zc, krmin, krmax, thmin, thmax, phmin, phmax, flag=0, n_m=1, m0=0, n_inst=1, tables=None):
        lib = load()
        self.close()
        t = tables or tsurff_tables(n_r, p, n_l, knots, r0, zc, self.nkr, self.nkt, self.nkp, krmin, krmax, thmin, thmax, phmin, phmax,
                                    flag, n_m, m0)
        d = qpc_dims(n_r, p, n_l, n_m, m0, n_inst)
        g = _kgrid(self.nkr, self.nkt, self.nkp, krmin, krmax, thmin, thmax, phmin, phmax, flag)
        h = ctypes.c_void_p()
        ib = np.ascontiguousarray(t["ib"], np.int32)
        _check(lib.qpc_tsurff_create(ctypes.byref(d), ctypes.byref(g), _ptr(_f64(t["kr"])), _ptr(_f64(t["kt"])), _ptr(_f64(t["kp"])),
                                     len(ib), _ptr(ib), _ptr(_f64(t["b0"])), _ptr(_f64(t["br"])), _ptr(_f64(t["j0"])), _ptr(_f64(t["jr"])),
                                     _ptr(_f64(t["y0"])), _ptr(np.ascontiguousarray(t["e0"], np.complex128)), _ptr(_f64(t["pmat"])),
                                     ctypes.byref(h)))
        self._h, self.tables, self.shape = h, t, (n_inst, n_m, n_l, n_r)
        self.kr, self.kt, self.kp = t["kr"], t["kt"], t["kp"]
        return self

    def close(self):
        if self._h is not None:
            load().qpc_tsurff_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def clearwork(self):
        _check(load().qpc_tsurff_clear(self._h))

    def accumulate(self, coef, dt, a=None):
        B = self.shape[0]
        if a is None:
            mode, av = TSURFF_FREE, None
        else:
            av = _f64(np.asarray(a, np.float64).reshape(B, -1) if np.ndim(a) > 1 else np.broadcast_to(np.asarray(a, np.float64), (B, len(a))))
            if av.shape[1] not in (2, 4):
                raise QpcError(1, "a needs 2 (z) or 4 (xy) values per instance")
            mode = TSURFF_Z if av.shape[1] == 2 else TSURFF_XY
        lib = load()
        if isinstance(coef, propagator_cn_hc_lgwz):
            _check(lib.qpc_lgwz_tsurff(coef._h, self._h, mode, _ptr(av), dt))
        elif isinstance(coef, propagator_cn_hc_vgwr):
            _check(lib.qpc_vgwr_tsurff(coef._h, self._h, mode, _ptr(av), dt))
        else:
            c = np.ascontiguousarray(coef, dtype=np.complex128).reshape(self.shape)
            _check(lib.qpc_tsurff_accumulate(self._h, mode, _ptr(av), dt, _ptr(c), 0))

    def last_run_ms(self):
        """device time of the last accumulate's kernels"""
        ms = ctypes.c_float(0)
        _check(load().qpc_tsurff_last_run(self._h, ctypes.byref(ms)))
        return ms.value

    def get(self):
        """(work [inst][kr][kt][kp] complex, clock [inst][4] = time, disx, disy, disz)"""
        w = np.zeros((self.shape[0], self.nkr, self.nkt, self.nkp), np.complex128)
        ck = np.zeros((self.shape[0], 4))
        _check(load().qpc_tsurff_get(self._h, _ptr(w), _ptr(ck)))
        return w, ck
