"""Generate the golden fixtures in tests/golden/ by running the reference's own
propagator (QPC-TDSE headers compiled by oracle/ref/Makefile into oracle/_ref/).

Run on the development machine, where the reference checkout exists:
    python tests/golden/make_golden.py <reference checkout>/include [--arnoldi] [--vgwr] [--mask] [--multim] [--momentum]
(or with the environment variable QPC_REFERENCE_DIR naming the checkout instead of the argument)
(those flags regenerate only the named fixtures.)
The fixtures are committed; the tests only read them.

Cases (hydrogen unless stated; r in [0, rmax], uniform knots, m = 0):
  small_setup.npz   N_r=64, p=6, n_l=6, rmax=30, dt=0.05: S, R, Rinv, D, H_l,
                    CN bands upper/lower (lu_zsb), Y10 eigensystem, knots, ground state
  small_yukawa.npz  same grid, V = -(1 + 17 e^{-2r})/r: H_l and ground state
  small_prop.npz    seeded random initial state, 50 field steps f_i = 0.05 sin(0.1 i),
                    then 5 field-free steps: final coefficients, S-norm, <z>, per-step <z>
  c0_field.npz      f(t_i) of the C0 pulse: 800 nm (w0 = 45.5633525/800),
                    1e14 W/cm^2 (E0 = sqrt(1e14/3.50944758e16)), sin^2, 4 cycles, dt = 0.05
  mid_pulse.npz     N_r=160, p=6, n_l=12, rmax=80: ground state through 1 cycle of
                    800 nm at 2e14 W/cm^2, CEP 0.5 pi, then 200 field-free steps; the
                    driver's per-step <z> (z_list) included
  c0_final.npz      the C0 workload: N_r=400, p=6, n_l=21, rmax=200, ground state,
                    the full c0 pulse (8826 steps): final coefficients, norm, <z>,
                    projections onto field-free states with E < 2
  arnoldi_small.npz the Arnoldi propagator propagator_hc_lgwz (la_1e.hpp) on the small
                    grid, kmax = 12, emin = 1e-14, emax = 1e-8, with the reference's
                    Cholesky factor of S: ground state through 3000 steps of dt = 0.01
                    under ez(t) = 0.05 sin(0.057 t) sin^2(pi t/30) ("conv"); from that
                    state 1 and 3 steps of dt = 0.1 at ez = 0.05 ("step1", "step3") and
                    1 step with the Yukawa Hamiltonian ("ystep1"); the ground state
                    through 10 field-free steps of dt = 0.1 (Krylov breakdown, "bd")
  arnoldi_mid.npz   the same propagator on the mid grid from the mid_pulse final state:
                    1 and 2 steps of dt = 0.1 at ez = 0.03, kmax = 12
  ep_prop.npz       the length-gauge propagator on a multi-m grid (N_r=40, p=5, n_l=4,
                    m = -2..2, r in [0, 20], dt = 0.05): the reference's S, R, H_l,
                    a seeded random state through 20 field steps f_i = 0.04 sin(0.2 i + 0.3)
                    and 2 field-free steps
  small_mask.npz    absorber_mask (absorber.hpp:40-63) on the small grid, [20, 30] with index 1/6,
                    applied once to a seeded random state: the mask band and the result
  vgwr_ep.npz       the velocity-gauge elliptical propagator propagator_cn_hc_vgwr
  vgwr_ep6.npz      (cn_1e.hpp:812-951) on two multi-m grids: N_r=40, p=5, n_l=4, m=-2..2
                    (odd n_m: zero-eigenvalue channels) and N_r=48, p=6, n_l=5, m=-3..2,
                    r in [0, 20], dt = 0.05; seeded random initial state, 20 steps under
                    A_x = 0.3 sin(0.5 t + 0.1), A_y = 0.2 cos(0.5 t), then 2 field-free
                    steps: the reference's S, 1/r, D, H_l, the couplings' eigenvalues, the
                    final coefficients and S-norm
  pcs_small.npz     spectrum_c_pcs (spectrum/momentum_1e.hpp:443-514) on the small grid (rmax = 30)
  pcs_ep.npz        and on the multi-m grid (N_r=40, p=5, n_l=4, m=-2..2, rmax = 20): a seeded
                    random state, nkr = 24, nkt = 5, nkp = 4, theta in [0, 3], phi in [0, 6];
                    "coul": Coulomb waves zc = 1, |k| uniform in [0.1, 2]; "plane": plane waves
                    with the cut-off at rb = 10, k^2/2 uniform for |k| in [0.2, 1.5]; the tables
                    (kr, kt, kp, ijl, plm, exm, cps) and measure_lmd / measure_prj / measure_pad
  pcsnum_small.npz  spectrum_c_pcs with numerical partial waves of V = -(1 + 17 e^{-2r})/r (the
                    driver's choice for screened potentials) on the small grid, "coul" axes:
                    ijl, cps, measure_lmd and measure_prj of a seeded random state
  tsurff_small.npz  spectrum_c_tsf (momentum_1e.hpp:516-1072) in the driver loop of the
                    length-gauge propagator on the small grid: a seeded random state, 60 steps
                    with f_i = 0.3 sin(0.4 t_i) sin^2(pi t_i / t_60) passed to accumulate(f_i,
                    f_i+1, dt, coef), then 20 field-free steps with accumulate(dt, coef);
                    surface r0 = 20, zc = 0, nkr = 24 (|k| in [0.2, 1.6]), nkt = 5 (theta in
                    [0.1, 3]), nkp = 4 (phi in [0, 4.5]): tables, work, clock, final state
  tsurff_ep.npz     the same with the velocity-gauge elliptical propagator on the multi-m grid
                    and accumulate(ax_i, ax_i+1, ay_i, ay_i+1, dt, coef) under the vgwr_ep
                    field, surface r0 = 12, zc = 1
"""
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.path.join(ROOT, "oracle", "_ref")


def build(ref_include):
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle", "ref"), "-j4", "REF_INCLUDE=" + ref_include], check=True)


def run(binary, *args, record_z=False):
    env = dict(os.environ, OPENBLAS_NUM_THREADS="1", OMP_NUM_THREADS="1")
    if record_z:
        env["QPC_REF_RECORD_Z"] = "1"
    out = subprocess.run([os.path.join(REF, binary)] + [str(a) for a in args], check=True, env=env,
                         stdout=subprocess.PIPE, text=True)
    return out.stdout


def load(d, name, shape=None, cplx=False):
    a = np.fromfile(os.path.join(d, name + ".bin"))
    if cplx:
        a = a.view(np.complex128)
    return a.reshape(shape) if shape is not None else a


def c0_field():
    e0 = float(np.sqrt(1e14 / 3.50944758e16))
    w0 = 45.5633525 / 800.0
    return e0, w0, 4.0, 0.0, 0.0, 0.05


def arnoldi(d):
    """Arnoldi fixtures (see the module docstring)."""
    NR, P, NL, RMAX = 64, 6, 6, 30.0
    K, EMIN, EMAX = 12, 1e-14, 1e-8
    run("ref_small", "setup", d, RMAX, 0.1, 1, 0, 0)
    chol = load(d, "chol", (NR, P + 1))
    out = {"kmax": K, "emin": EMIN, "emax": EMAX, "chol": chol}

    def arn(binary, init, ez, dt, tag, rmax=RMAX, pot=(1, 0, 0), shape=(NL, NR)):
        ez = np.asarray(ez, np.float64)
        ez.tofile(os.path.join(d, "ez.bin"))
        if not isinstance(init, str):
            np.asarray(init, np.complex128).tofile(os.path.join(d, "ainit.bin"))
            init = os.path.join(d, "ainit.bin")
        run(binary, "arnoldi", d, rmax, dt, pot[0], pot[1], pot[2], init, os.path.join(d, "ez.bin"), ez.size, K, EMIN, EMAX)
        out[tag + "_ez"] = ez
        out[tag + "_dt"] = dt
        out[tag + "_coef"] = load(d, "coef", shape, True)
        out[tag + "_crit"] = load(d, "crit").astype(np.int8)
        return out[tag + "_coef"]

    t = 0.01 * np.arange(3000)
    conv = arn("ref_small", "gs", 0.05 * np.sin(0.057 * t) * np.sin(np.pi * t / 30.0) ** 2, 0.01, "conv")
    arn("ref_small", conv, [0.05], 0.1, "step1")
    arn("ref_small", conv, [0.05] * 3, 0.1, "step3")
    arn("ref_small", conv, [0.05], 0.1, "ystep1", pot=(1, 17, 2))
    arn("ref_small", "gs", np.zeros(10), 0.1, "bd")
    np.savez(os.path.join(HERE, "arnoldi_small.npz"), **out)
    # mid grid, from the CN mid-pulse final state
    out = {"kmax": K, "emin": EMIN, "emax": EMAX}
    mid = np.load(os.path.join(HERE, "mid_pulse.npz"))["coef"]
    out["init"] = mid
    arn("ref_mid", mid, [0.03], 0.1, "step1", rmax=80.0, shape=(12, 160))
    arn("ref_mid", mid, [0.03] * 2, 0.1, "step2", rmax=80.0, shape=(12, 160))
    np.savez(os.path.join(HERE, "arnoldi_mid.npz"), **out)


def multi_m(d):
    NR, P, NL, NM, M0, RMAX, DT = 40, 5, 4, 5, -2, 20.0, 0.05
    run("ref_ep", "setup", d, RMAX, DT, 1, 0, 0)
    nlh = abs(M0) + NL
    rng = np.random.default_rng(12)
    n = NR * NL * NM
    c0 = (rng.standard_normal(n) + 1j * rng.standard_normal(n)) * np.exp(-np.tile(np.arange(NR), NL * NM) / 8.0)
    c0.tofile(os.path.join(d, "einit.bin"))
    nt, nfree = 20, 2
    f = 0.04 * np.sin(0.2 * np.arange(nt + 1) + 0.3)
    f.tofile(os.path.join(d, "efield.bin"))
    S, R, H = load(d, "S", (NR, P + 1)), load(d, "R", (NR, P + 1)), load(d, "H", (nlh, NR, P + 1))
    run("ref_ep", "propagate", d, RMAX, DT, 1, 0, 0, os.path.join(d, "einit.bin"), os.path.join(d, "efield.bin"), nt, nfree, 1)
    np.savez(os.path.join(HERE, "ep_prop.npz"), n_r=NR, p=P, n_l=NL, n_m=NM, m0=M0, dt=DT, S=S, R=R, H=H,
             init=c0.reshape(NM, NL, NR), f=f, nt=nt, nfree=nfree, coef=load(d, "coef", (NM, NL, NR), True), norm=load(d, "norm"))


def mask(d):
    NR, P, NL, RMAX = 64, 6, 6, 30.0
    rng = np.random.default_rng(8)
    c0 = rng.standard_normal(NL * NR) + 1j * rng.standard_normal(NL * NR)
    c0.tofile(os.path.join(d, "minit.bin"))
    run("ref_small", "mask", d, RMAX, 0.05, 1, 0, 0, os.path.join(d, "minit.bin"), 20.0, 30.0, 1.0 / 6.0)
    np.savez(os.path.join(HERE, "small_mask.npz"), rmin=20.0, rmax_mask=30.0, index=1.0 / 6.0, init=c0.reshape(NL, NR),
             band=load(d, "maskband", (NR, P + 1)), coef=load(d, "coef", (NL, NR), True))


def vgwr(d):
    """Velocity-gauge elliptical fixtures (see the module docstring)."""
    for binary, tag, NR, P, NL, NM, M0 in (("ref_ep", "vgwr_ep", 40, 5, 4, 5, -2), ("ref_ep6", "vgwr_ep6", 48, 6, 5, 6, -3)):
        RMAX, DT, nt, nfree = 20.0, 0.05, 20, 2
        run(binary, "setup", d, RMAX, DT, 1, 0, 0)
        nlh = max(abs(M0), abs(M0 + NM - 1)) + NL
        out = {"n_r": NR, "p": P, "n_l": NL, "n_m": NM, "m0": M0, "rmax": RMAX, "dt": DT, "nt": nt, "nfree": nfree,
               "S": load(d, "S", (NR, P + 1)), "RINV": load(d, "RINV", (NR, P + 1)), "D": load(d, "D", (NR, P + 1)),
               "H": load(d, "H", (nlh, NR, P + 1))}
        rng = np.random.default_rng(4)
        n = NR * NL * NM
        c0 = (rng.standard_normal(n) + 1j * rng.standard_normal(n)) * np.exp(-np.tile(np.arange(NR), NL * NM) / 8.0)
        c0.tofile(os.path.join(d, "vinit.bin"))
        t = DT * np.arange(nt + 1)
        a = np.stack([0.3 * np.sin(0.5 * t + 0.1), 0.2 * np.cos(0.5 * t)], 1)
        a.tofile(os.path.join(d, "vfield.bin"))
        run(binary, "vgwr", d, RMAX, DT, 1, 0, 0, os.path.join(d, "vinit.bin"), os.path.join(d, "vfield.bin"), nt, nfree)
        out.update(init=c0.reshape(NM, NL, NR), atab=a, coef=load(d, "coef", (NM, NL, NR), True), norm=load(d, "norm"),
                   zeig=np.stack([load(d, "zeig_" + c) for c in ("x1", "x2", "y1", "y2")]),
                   xlist=load(d, "xlist"), ylist=load(d, "ylist"))
        np.savez(os.path.join(HERE, tag + ".npz"), **out)


def momentum(d):
    """Momentum-spectrum fixtures (see the module docstring); the harness's momentum grids are
    compile-time: nkr = 24, nkt = 5, nkp = 4."""
    nk = (24, 5, 4)
    # ---- PCS on the small grid (m = 0) and on the multi-m grid
    for binary, tag, NR, P, NL, NM, M0, RMAX in (("ref_small", "pcs_small", 64, 6, 6, 1, 0, 30.0), ("ref_ep", "pcs_ep", 40, 5, 4, 5, -2, 20.0)):
        rng = np.random.default_rng(21)
        n = NR * NL * NM
        c = (rng.standard_normal(n) + 1j * rng.standard_normal(n)) * np.exp(-np.tile(np.arange(NR), NL * NM) / 12.0)
        c.tofile(os.path.join(d, "pcoef.bin"))
        out = {"n_r": NR, "p": P, "n_l": NL, "n_m": NM, "m0": M0, "rmax": RMAX, "nkr": nk[0], "nkt": nk[1], "nkp": nk[2],
               "coef": c.reshape(NM, NL, NR)}
        lmax = max(abs(M0), abs(M0 + NM - 1)) + NL - 1
        for case, krng, pzc, rb, flag in (("coul", (0.1, 2.0), 1.0, 0.0, 0), ("plane", (0.2, 1.5), 0.0, 10.0, 1)):
            ang = (0.0, 3.0, 0.0, 6.0)
            run(binary, "pcs", d, RMAX, 0.05, 1, 0, 0, os.path.join(d, "pcoef.bin"), krng[0], krng[1], *ang, pzc, rb, flag)
            out.update({case + "_grid": np.array([krng[0], krng[1], *ang, pzc, rb, flag]),
                        case + "_kr": load(d, "kr"), case + "_kt": load(d, "kt"), case + "_kp": load(d, "kp"),
                        case + "_ijl": load(d, "ijl", (nk[0], lmax + 1, NR)), case + "_plm": load(d, "plm", (nk[1], NM, NL)),
                        case + "_exm": load(d, "exm", (nk[2], NM), True), case + "_cps": load(d, "cps", (nk[0], lmax + 1), True),
                        case + "_lmd": load(d, "lmd", (nk[0], NM, NL), True), case + "_pmd": load(d, "pmd", nk, True),
                        case + "_pad": load(d, "pad", None, True)[:nk[0] * nk[1]].reshape(nk[0], nk[1])})
        np.savez(os.path.join(HERE, tag + ".npz"), **out)
    # ---- numerical partial waves of a screened potential (the driver's PCS for hydrogenic_yukawa)
    NR, P, NL, RMAX = 64, 6, 6, 30.0
    rng = np.random.default_rng(23)
    c = (rng.standard_normal(NR * NL) + 1j * rng.standard_normal(NR * NL)) * np.exp(-np.tile(np.arange(NR), NL) / 12.0)
    c.tofile(os.path.join(d, "pcoef.bin"))
    ZC, ZS, SG = 1.0, 17.0, 2.0
    run("ref_small", "pcsnum", d, RMAX, 0.05, ZC, ZS, SG, os.path.join(d, "pcoef.bin"), 0.1, 2.0, 0.0, 3.0, 0.0, 6.0, 0)
    np.savez(os.path.join(HERE, "pcsnum_small.npz"), n_r=NR, p=P, n_l=NL, rmax=RMAX, zc=ZC, zs=ZS, sigma=SG, nkr=nk[0], nkt=nk[1],
             nkp=nk[2], grid=np.array([0.1, 2.0, 0.0, 3.0, 0.0, 6.0, 0]), coef=c.reshape(1, NL, NR),
             kr=load(d, "kr"), ijl=load(d, "ijl", (nk[0], NL, NR)), cps=load(d, "cps", (nk[0], NL), True),
             lmd=load(d, "lmd", (nk[0], 1, NL), True), pmd=load(d, "pmd", nk, True))
    # ---- t-SURFF in the driver loops
    for binary, tag, NR, P, NL, NM, M0, RMAX, mode, r0, tzc in (("ref_small", "tsurff_small", 64, 6, 6, 1, 0, 30.0, "z", 20.0, 0.0),
                                                                 ("ref_ep", "tsurff_ep", 40, 5, 4, 5, -2, 20.0, "xy", 12.0, 1.0)):
        DT, nt, nfree = 0.05, 60, 20
        run(binary, "setup", d, RMAX, DT, 1, 0, 0)
        nlh = max(abs(M0), abs(M0 + NM - 1)) + NL
        rng = np.random.default_rng(22)
        n = NR * NL * NM
        c0 = (rng.standard_normal(n) + 1j * rng.standard_normal(n)) * np.exp(-np.tile(np.arange(NR), NL * NM) / 10.0)
        c0.tofile(os.path.join(d, "tinit.bin"))
        t = DT * np.arange(nt + 1)
        if mode == "z":
            f = 0.3 * np.sin(0.4 * t) * np.sin(np.pi * t / t[-1]) ** 2
        else:
            f = np.stack([0.3 * np.sin(0.5 * t + 0.1), 0.2 * np.cos(0.5 * t)], 1)
        f.tofile(os.path.join(d, "tfield.bin"))
        krng, ang = (0.2, 1.6), (0.1, 3.0, 0.0, 4.5)
        run(binary, "tsurff", d, RMAX, DT, 1, 0, 0, os.path.join(d, "tinit.bin"), os.path.join(d, "tfield.bin"), nt, nfree, mode, r0, tzc,
            krng[0], krng[1], *ang, 0)
        lmax = nlh - 1
        out = {"n_r": NR, "p": P, "n_l": NL, "n_m": NM, "m0": M0, "rmax": RMAX, "dt": DT, "nt": nt, "nfree": nfree, "mode": mode,
               "r0": r0, "tzc": tzc, "grid": np.array([krng[0], krng[1], *ang, 0]), "nkr": nk[0], "nkt": nk[1], "nkp": nk[2],
               "S": load(d, "S", (NR, P + 1)), "R": load(d, "R", (NR, P + 1)), "RINV": load(d, "RINV", (NR, P + 1)),
               "D": load(d, "D", (NR, P + 1)), "H": load(d, "H", (nlh, NR, P + 1)), "knots": load(d, "knots"),
               "init": c0.reshape(NM, NL, NR), "field": f,
               "kr": load(d, "kr"), "kt": load(d, "kt"), "kp": load(d, "kp"), "ib": load(d, "ib").astype(np.int32),
               "b0": load(d, "b0"), "br": load(d, "br"), "j0": load(d, "j0", (nk[0], lmax + 1)), "jr": load(d, "jr", (nk[0], lmax + 1)),
               "y0": load(d, "y0", (nk[1], NM, NL)), "e0": load(d, "e0", (nk[2], NM), True),
               "pmat": np.stack([load(d, "pmat%d" % i, (NM, NL)) for i in range(3)]),
               "work": load(d, "work", nk, True), "clock": load(d, "clock"), "coef": load(d, "coef", (NM, NL, NR), True)}
        np.savez(os.path.join(HERE, tag + ".npz"), **out)


def main():
    if len(sys.argv) > 1 and not sys.argv[1].startswith("--"):
        ref_include = sys.argv[1]
    elif os.environ.get("QPC_REFERENCE_DIR"):
        ref_include = os.path.join(os.environ["QPC_REFERENCE_DIR"], "include")
    else:
        sys.exit("usage: make_golden.py <reference checkout>/include [--flags] (or set QPC_REFERENCE_DIR)")
    build(ref_include)
    if any(a in sys.argv for a in ("--arnoldi", "--vgwr", "--mask", "--multim", "--momentum")):
        with tempfile.TemporaryDirectory() as d:
            if "--arnoldi" in sys.argv:
                arnoldi(d)
            if "--vgwr" in sys.argv:
                vgwr(d)
            if "--mask" in sys.argv:
                mask(d)
            if "--multim" in sys.argv:
                multi_m(d)
            if "--momentum" in sys.argv:
                momentum(d)
        return
    meta = {}
    with tempfile.TemporaryDirectory() as d:
        # ---- small grid setup
        NR, P, NL, RMAX, DT = 64, 6, 6, 30.0, 0.05
        run("ref_small", "setup", d, RMAX, DT, 1, 0, 0)
        np.savez(os.path.join(HERE, "small_setup.npz"),
                 n_r=NR, p=P, n_l=NL, rmax=RMAX, dt=DT,
                 S=load(d, "S", (NR, P + 1)), R=load(d, "R", (NR, P + 1)), RINV=load(d, "RINV", (NR, P + 1)),
                 D=load(d, "D", (NR, P + 1)), H=load(d, "H", (NL, NR, P + 1)),
                 upper=load(d, "upper", (NL, NR, P + 1), True), lower=load(d, "lower", (NL, NR, P + 1), True),
                 yeig=load(d, "yeig"), yprj=load(d, "yprj", (NL, NL)), y10=load(d, "y10"),
                 knots=load(d, "knots"), gs_energy=load(d, "gs_energy"), gs_coef=load(d, "gs_coef", (NL, NR), True))
        run("ref_small", "setup", d, RMAX, DT, 1, 17, 2)
        np.savez(os.path.join(HERE, "small_yukawa.npz"), zc=1.0, zs=17.0, sigma=2.0,
                 H=load(d, "H", (NL, NR, P + 1)), gs_energy=load(d, "gs_energy"), gs_coef=load(d, "gs_coef", (NL, NR), True))
        # ---- small propagation
        rng = np.random.default_rng(1)
        c0 = rng.standard_normal(NL * NR) + 1j * rng.standard_normal(NL * NR)
        c0.tofile(os.path.join(d, "init.bin"))
        nt, nfree = 50, 5
        f = 0.05 * np.sin(0.1 * np.arange(nt + 1))
        f.tofile(os.path.join(d, "field.bin"))
        run("ref_small", "propagate", d, RMAX, DT, 1, 0, 0, os.path.join(d, "init.bin"), os.path.join(d, "field.bin"), nt, nfree, 1,
            record_z=True)
        np.savez(os.path.join(HERE, "small_prop.npz"), init=c0.reshape(NL, NR), f=f, nt=nt, nfree=nfree,
                 coef=load(d, "coef", (NL, NR), True), norm=load(d, "norm"), dipole=load(d, "dipole"),
                 zlist=load(d, "zlist"))
        # ---- C0 field
        e0, w0, nc, n0, cep, dt = c0_field()
        run("ref_small", "field", d, e0, w0, nc, n0, cep, dt)
        np.savez(os.path.join(HERE, "c0_field.npz"), e0=e0, w0=w0, nc=nc, n0=n0, cep=cep, dt=dt,
                 nt=int(load(d, "nt")[0]), f=load(d, "f"))
        # ---- mid grid: one cycle of 800 nm at 2e14 W/cm^2, CEP 0.5 pi
        e0m = float(np.sqrt(2e14 / 3.50944758e16))
        run("ref_mid", "field", d, e0m, w0, 1.0, 0.0, 0.5, 0.05)
        fm = load(d, "f")
        ntm = int(load(d, "nt")[0])
        fm.tofile(os.path.join(d, "fieldm.bin"))
        out = run("ref_mid", "propagate", d, 80.0, 0.05, 1, 0, 0, "gs", os.path.join(d, "fieldm.bin"), ntm, 200, 1, record_z=True)
        meta["mid_pulse"] = out.strip()
        np.savez(os.path.join(HERE, "mid_pulse.npz"), n_r=160, p=6, n_l=12, rmax=80.0, dt=0.05,
                 e0=e0m, w0=w0, nc=1.0, n0=0.0, cep=0.5, nt=ntm, nfree=200, f=fm,
                 coef=load(d, "coef", (12, 160), True), norm=load(d, "norm"), dipole=load(d, "dipole"),
                 zlist=load(d, "zlist"))
        # ---- C0 full pulse
        fc = np.load(os.path.join(HERE, "c0_field.npz"))["f"]
        ntc = fc.size - 1
        fc.tofile(os.path.join(d, "fieldc.bin"))
        out = run("ref_c0", "propagate", d, 200.0, 0.05, 1, 0, 0, "gs", os.path.join(d, "fieldc.bin"), ntc, 0, 1)
        meta["c0_final"] = out.strip()
        coef = load(d, "coef", (21, 400), True)
        norm, dip = load(d, "norm"), load(d, "dipole")
        coef.tofile(os.path.join(d, "c0coef.bin"))
        run("ref_c0", "proj", d, 200.0, 0.05, 1, 0, 0, os.path.join(d, "c0coef.bin"), 2.0)
        np.savez(os.path.join(HERE, "c0_final.npz"), n_r=400, p=6, n_l=21, rmax=200.0, dt=0.05, nt=ntc,
                 coef=coef, norm=norm, dipole=dip, proj=load(d, "proj", None, True),
                 proj_nnz=load(d, "proj_nnz").astype(np.int64), proj_energy=load(d, "proj_energy"))
        arnoldi(d)
        vgwr(d)
        mask(d)
        multi_m(d)
        momentum(d)
    # what was run, on stdout (kept out of the fixtures directory)
    print(json.dumps(meta, indent=1))


if __name__ == "__main__":
    main()
