"""Learned surrogate for the laser scan: laser parameters -> photoelectron and harmonic
spectra, with the batched TDSE engine as the label generator and the fallback.

No counterpart in the reference.  Pieces:
  * draw_params      the batched laser scan's parameter distribution: peak intensity
                     log-uniform in [5e13, 5e14] W/cm^2, wavelength uniform in
                     [400, 2000] nm, CEP uniform in [0, 2 pi), integer sin^2 cycles 2..10,
                     ellipticity 0 (the length-gauge engine is z-linear).
  * features         network inputs.  "sym" (default, 10 inputs): log10(I / 1e14 W/cm^2),
                     (lambda - 1200)/800, sin 2 CEP, cos 2 CEP (the spectra are invariant under
                     CEP -> CEP + pi), (cycles - 6)/4, ellipticity, and four derived ones (cutoff
                     order, w/U_p, Ip/U_p, pulse length); "base" (6 inputs): the first six with
                     sin CEP, cos CEP.
  * tdse_spectra     runs the batched Crank-Nicolson engine (hydrogen, B-splines of
                     degree 6, N_r = 800 on [0, 400], l < 41, dt = 0.05) from the ground
                     state through each pulse, recording <z>(t) in the loop, then projects
                     on the field-free eigenstates.  Labels:
                       PES  256 bins on [0, 3.17 U_p): sum |<E_n|psi>|^2 g(E - E_n) with a
                            Gaussian g of width max(3.17 U_p / 32, 0.003 a.u.) (the box's
                            discrete continuum broadened beyond its level spacing), times
                            U_p, log10, floored 6 decades below the spectrum's maximum;
                       HHG  harmonic orders 1..128: mean of S(w) (plot_hhs.m restated,
                            sin^2 window over the pulse, evaluated on the GPU by qpc_hhg_spectra)
                            over w / w0 in [q - 1/2, q + 1/2),
                            log10, floored 8 decades below the maximum (a detector's
                            dynamic range; below it the spectrum is window leakage).
  * tdse_spectra_elliptical
                     the fallback for ellipticity != 0 (outside the z-linear training set): the
                     velocity-gauge elliptical engine (propagator_cn_hc_vgwr) on ELL_GRID from the
                     ground state, A(t) = A0/sqrt(1 + eps^2) sin^2(pi t/tau) (cos, eps sin)(w t + cep)
                     with A0 = E0/w; <x>, <y> recorded in the loop (observable_r) and the final state
                     projected on the field-free eigenstates of every (m, l).  Labels as above, the
                     harmonic spectrum being S_x + S_y.
  * Surrogate        a 5-member ensemble of 6 -> 4 x 256 GELU -> 384 MLPs trained on the GPU
                     (qpc_mlp: bfloat16 operands, fp32 accumulation, Adam) on standardised
                     targets; query() answers from the ensemble mean when the members agree
                     (mean over outputs of the standard deviation, in standardised units,
                     below the threshold) and the ellipticity is 0; every other query is
                     answered by the TDSE: z-linear queries by the batched length-gauge engine,
                     elliptical ones always by the velocity-gauge engine.
"""
import importlib
import time

import numpy as np

C2_GRID = dict(n_r=800, p=6, n_l=41, rmax=400.0, dt=0.05)
# the elliptical fallback's grid: the scan's radial grid, l <= 20 for |m| <= 20 (the reference's
# rectangular channel set, 41 x 21 channels)
ELL_GRID = dict(n_r=800, p=6, l_max=20, rmax=400.0, dt=0.05)
N_PES, N_HHG = 256, 128
PES_DECADES, HHG_DECADES = 6.0, 8.0


def _q():
    return importlib.import_module(__name__.rsplit(".", 1)[0])


def draw_params(n, seed):
    rng = np.random.default_rng(seed)
    return {
        "intensity": 10 ** rng.uniform(np.log10(5e13), np.log10(5e14), n),
        "wavelength": rng.uniform(400.0, 2000.0, n),
        "cep": rng.uniform(0.0, 2 * np.pi, n),
        "cycles": rng.integers(2, 11, n).astype(np.float64),
        "ellipticity": np.zeros(n),
    }


FEATURES = ("base", "sym")
IP_H = 0.5   # ionization potential of the scan's atom (hydrogen), a.u.


def features(p, kind="sym"):
    """network inputs.  base: log10(I / 1e14 W/cm^2), (lambda - 1200)/800, sin CEP, cos CEP,
    (cycles - 6)/4, ellipticity.  sym: the CEP enters as sin 2 CEP, cos 2 CEP -- the spectra are
    exactly invariant under CEP -> CEP + pi (the field changes sign; the atom is symmetric under
    r -> -r, so |<E|psi>|^2 and |FFT <z>|^2 are unchanged) -- and four derived inputs are added:
    log of the cutoff order (Ip + 3.17 U_p)/w, log(w/U_p), log(Ip/U_p) and the pulse length in
    wavelength-cycles, each scaled to about [-1, 1]."""
    x = np.stack([np.log10(p["intensity"] / 1e14), (p["wavelength"] - 1200.0) / 800.0, np.sin(p["cep"]), np.cos(p["cep"]),
                  (p["cycles"] - 6.0) / 4.0, p["ellipticity"]], axis=1)
    if kind == "base":
        return x.astype(np.float32)
    if kind != "sym":
        raise ValueError("unknown feature set %r" % (kind,))
    x[:, 2], x[:, 3] = np.sin(2 * p["cep"]), np.cos(2 * p["cep"])
    q = _q()
    u = up(p)
    w0 = np.array([q.wavelength_to_w0(l) for l in p["wavelength"]])
    extra = np.stack([(np.log((IP_H + 3.17 * u) / w0) - 4.0) / 2.0, (np.log(w0 / u) + 2.0) / 3.0, np.log(IP_H / u) / 3.0,
                      (p["cycles"] * p["wavelength"] / 1000.0 - 8.0) / 6.0], axis=1)
    return np.concatenate([x, extra], axis=1).astype(np.float32)


def up(p):
    """Ponderomotive energy E0^2 / (4 w^2) per parameter set [a.u.]"""
    q = _q()
    e0 = np.array([q.intensity_to_e0(i) for i in p["intensity"]])
    w0 = np.array([q.wavelength_to_w0(l) for l in p["wavelength"]])
    return e0 ** 2 / (4 * w0 ** 2)


class _Setup:
    """Grid, matrices, ground state and field-free eigenbasis of one TDSE grid."""

    def __init__(self, grid, emax):
        q = _q()
        g = dict(grid)
        self.g = g
        kn = q.linear_knots(g["n_r"], g["p"], 0.0, g["rmax"])
        self.S, self.R, _, _, self.H = q.radial_setup(g["n_r"], g["p"], g["n_l"], kn)
        self.c0, self.e0 = q.ground_state(self.S, self.H, g["n_l"])
        self.n_state, self.basis, self.energies = q.left_eigenbasis(self.S, self.H, g["n_l"] - 1, emax)
        self.energy = np.concatenate(self.energies)


def _pes_label(proj, energy, u):
    """Gaussian-broadened PES on [0, 3.17 U_p), 256 bins, in units of 1/U_p, log10, floored."""
    emax = 3.17 * u
    edges = np.linspace(0.0, emax, N_PES + 1)
    centres = 0.5 * (edges[1:] + edges[:-1])
    w = np.abs(proj) ** 2
    sig = max(emax / 32.0, 0.003)
    keep = (energy > -6 * sig) & (energy < emax + 6 * sig)
    d = (centres[:, None] - energy[keep][None, :]) / sig
    dens = (np.exp(-0.5 * d * d) / (sig * np.sqrt(2 * np.pi))) @ w[keep]
    y = np.log10(np.maximum(dens * u, 1e-300))
    return np.maximum(y, y.max() - PES_DECADES)


def _hhg_bin(om, s, w0):
    """mean spectrum over harmonic orders q in [k + 1/2, k + 3/2), log10, floored"""
    h = om / w0
    out = np.full(N_HHG, 1e-300)
    for k in range(N_HHG):
        sel = (h >= k + 0.5) & (h < k + 1.5)
        if sel.any():
            out[k] = max(float(s[sel].mean()), 1e-300)
    y = np.log10(out)
    return np.maximum(y, y.max() - HHG_DECADES)


def _hhg_labels(z, n, dt, w0, z2=None):
    """harmonic labels of a batch from its dipole lists z [B][ld] (n[i] samples each; for elliptical
    pulses z2 holds the second component and the spectrum is the sum of both), with the spectra
    evaluated on the GPU (qpc_hhg_spectra) up to the frequencies the 128 orders need."""
    q = _q()
    n = np.asarray(n, np.int64)
    w0 = np.asarray(w0, float)
    kneed = np.minimum((n + 1) // 2, np.floor((N_HHG + 0.5) * w0 * n * dt / (2 * np.pi)).astype(np.int64) + 2)
    kmax = int(max(1, kneed.max()))
    s = q.hhg_spectra(z, n, dt, kmax)
    if z2 is not None:
        s = s + q.hhg_spectra(z2, n, dt, kmax)
    out = np.zeros((n.size, N_HHG), np.float32)
    for i in range(n.size):
        om = 2 * np.pi / (n[i] * dt) * np.arange(kmax)
        out[i] = _hhg_bin(om, s[i], w0[i])
    return out


def tdse_spectra(p, grid=C2_GRID, batch=256, setup=None, log=None):
    """PES and HHG labels [n][256], [n][128] for parameter sets p (ellipticity must be 0),
    from the batched engine in batches of `batch`.  Returns (pes, hhg, info)."""
    q = _q()
    n = len(p["intensity"])
    if np.any(p["ellipticity"] != 0):
        raise ValueError("the TDSE engine here is z-linear: ellipticity must be 0")
    u = up(p)
    if setup is None:
        setup = _Setup(grid, emax=max(3.17 * float(u.max()) * 1.5, 1.0))
    g = setup.g
    pes = np.zeros((n, N_PES), np.float32)
    hhg = np.zeros((n, N_HHG), np.float32)
    wf_steps, t_run = 0, 0.0
    prop = None
    for b0 in range(0, n, batch):
        idx = np.arange(b0, min(n, b0 + batch))
        B = idx.size
        tabs = [q.field_sinen(q.intensity_to_e0(p["intensity"][i]), q.wavelength_to_w0(p["wavelength"][i]), p["cycles"][i], 0.0,
                              p["cep"][i] / np.pi, g["dt"]) for i in idx]
        nt = np.array([t.size - 1 for t in tabs], np.int64)
        ftab = np.zeros((B, int(nt.max()) + 1))
        for k, t in enumerate(tabs):
            ftab[k, :t.size] = t
        if prop is None or prop.shape[0] != B:
            prop = q.propagator_cn_hc_lgwz().initialize(g["n_r"], g["p"], g["n_l"], setup.S, setup.R, setup.H, g["dt"], n_inst=B)
        prop.put(np.broadcast_to(setup.c0, (B,) + setup.c0.shape))
        t0 = time.time()
        z = prop.run_dipole(ftab, nt, nt, setup.R)
        t_run += time.time() - t0
        wf_steps += int(nt.sum())
        proj = prop.projection(setup.n_state, setup.basis).reshape(B, -1)
        for k, i in enumerate(idx):
            pes[i] = _pes_label(proj[k], setup.energy, u[i])
        hhg[idx] = _hhg_labels(z, nt, g["dt"], [q.wavelength_to_w0(p["wavelength"][i]) for i in idx])
        if log:
            log("batch %d-%d: %d wf-steps, %.1f s" % (idx[0], idx[-1], int(nt.sum()), time.time() - t0))
    return pes, hhg, {"wf_steps": wf_steps, "run_s": t_run}


def elliptic_vector_potential(intensity, wavelength, cycles, cep, ellipticity, dt):
    """(nt, A[nt+1][2]): A(t_i) = A0/sqrt(1 + eps^2) sin^2(pi t/tau) (cos, eps sin)(w t + cep) at
    t_i = i dt, tau = cycles 2 pi / w, A0 = E0 / w, nt = floor(tau / dt)."""
    q = _q()
    w0 = q.wavelength_to_w0(wavelength)
    a0 = q.intensity_to_e0(intensity) / w0
    tau = cycles * 2 * np.pi / w0
    nt = int(np.floor(tau / dt + 1e-9))
    t = dt * np.arange(nt + 1)
    env = np.sin(np.pi * t / tau) ** 2 / np.sqrt(1.0 + ellipticity ** 2)
    return nt, np.stack([a0 * env * np.cos(w0 * t + cep), a0 * ellipticity * env * np.sin(w0 * t + cep)], 1)


class _EllSetup:
    """Grid, matrices, ground state (1s in the m = 0, l = 0 channel) and field-free eigenbasis of the
    elliptical fallback's grid."""

    def __init__(self, grid, emax):
        q = _q()
        g = dict(grid)
        self.g = g
        L = g["l_max"]
        self.n_m, self.n_l, self.m0 = 2 * L + 1, L + 1, -L
        self.lmax = abs(self.m0) + self.n_l - 1
        kn = q.linear_knots(g["n_r"], g["p"], 0.0, g["rmax"])
        self.S, self.R, self.Ri, self.D, self.H = q.radial_setup(g["n_r"], g["p"], self.lmax + 1, kn)
        c, self.e0 = q.ground_state(self.S, self.H, self.n_l, self.n_m, -self.m0, 0, 0, self.m0)
        self.c0 = c
        self.n_state, self.basis, self.energies = q.left_eigenbasis(self.S, self.H, self.lmax, emax)


def tdse_spectra_elliptical(p, grid=ELL_GRID, batch=16, setup=None, log=None):
    """PES and HHG labels [n][256], [n][128] for parameter sets p with any ellipticity, from the
    velocity-gauge elliptical engine in batches of `batch`.  Returns (pes, hhg, info)."""
    q = _q()
    n = len(p["intensity"])
    u = up(p)
    if setup is None:
        setup = _EllSetup(grid, emax=max(3.17 * float(u.max()) * 1.5, 1.0))
    g = setup.g
    pes = np.zeros((n, N_PES), np.float32)
    hhg = np.zeros((n, N_HHG), np.float32)
    wf_steps, t_run = 0, 0.0
    prop = None
    for b0 in range(0, n, batch):
        idx = np.arange(b0, min(n, b0 + batch))
        B = idx.size
        tabs = [elliptic_vector_potential(p["intensity"][i], p["wavelength"][i], p["cycles"][i], p["cep"][i], p["ellipticity"][i],
                                          g["dt"]) for i in idx]
        nt = np.array([t[0] for t in tabs], np.int64)
        atab = np.zeros((B, int(nt.max()) + 1, 2))
        for k, (m, a) in enumerate(tabs):
            atab[k, :m + 1] = a
        if prop is None or prop.shape[0] != B:
            prop = q.propagator_cn_hc_vgwr().initialize(g["n_r"], g["p"], setup.n_l, setup.n_m, setup.m0, setup.S, setup.Ri, setup.D,
                                                        setup.H, g["dt"], n_inst=B)
        prop.put(np.broadcast_to(setup.c0, (B,) + setup.c0.shape))
        t0 = time.time()
        x, y = prop.run_dipole(atab, nt, nt, setup.R)
        t_run += time.time() - t0
        wf_steps += int(nt.sum())
        c = prop.get()
        for k, i in enumerate(idx):
            proj, energy = [], []
            for im in range(setup.n_m):
                for il in range(setup.n_l):
                    l = il + abs(setup.m0 + im)
                    if setup.n_state[l]:
                        proj.append(setup.basis[l] @ c[k, im, il])
                        energy.append(setup.energies[l])
            pes[i] = _pes_label(np.concatenate(proj), np.concatenate(energy), u[i])
        hhg[idx] = _hhg_labels(x, nt, g["dt"], [q.wavelength_to_w0(p["wavelength"][i]) for i in idx], y)
        if log:
            log("elliptical batch %d-%d: %d wf-steps, %.1f s" % (idx[0], idx[-1], int(nt.sum()), time.time() - t0))
    return pes, hhg, {"wf_steps": wf_steps, "run_s": t_run}


class Surrogate:
    """Ensemble MLP surrogate with TDSE fallback."""

    def __init__(self, n_members=5, n_hidden=256, n_layers=4, seed=0, features="sym"):
        self.n_members, self.n_hidden, self.n_layers, self.seed = n_members, n_hidden, n_layers, seed
        self.features = features
        self.net = None

    def fit(self, p, pes, hhg, epochs=400, batch=256, lr=1e-3, stages=1):
        """Adam on standardised targets; with stages > 1 the epochs are split into stages whose
        learning rate falls by 3x each (the optimiser state carries over).  Returns the loss
        history [epochs][members]."""
        q = _q()
        X = features(p, self.features)
        Y = np.concatenate([pes, hhg], axis=1).astype(np.float64)
        self.mu = Y.mean(axis=0)
        self.sd = np.maximum(Y.std(axis=0), 1e-3)
        Yn = ((Y - self.mu) / self.sd).astype(np.float32)
        self.net = q.mlp_ensemble(X.shape[1], Y.shape[1], self.n_hidden, self.n_layers, self.n_members, self.seed)
        hist = []
        per = max(1, epochs // stages)
        for st in range(stages):
            ep = per if st < stages - 1 else epochs - per * (stages - 1)
            hist.append(self.net.train(X, Yn, ep, batch, lr / 3.0 ** st, seed=self.seed + 1 + st))
        return np.concatenate(hist, axis=0)

    def predict(self, p):
        """(mean [n][384], disagreement [n]) in label units; disagreement is the mean over
        outputs of the members' standard deviation in standardised units."""
        y = self.net.predict(features(p, self.features)).astype(np.float64)
        mean = y.mean(axis=0) * self.sd + self.mu
        dis = y.std(axis=0).mean(axis=1)
        return mean, dis

    def calibrate(self, p_val, y_val, quantile=0.9):
        """Threshold on the disagreement: the given quantile over a validation set."""
        _, dis = self.predict(p_val)
        self.threshold = float(np.quantile(dis, quantile))
        return self.threshold

    def query(self, p, threshold=None, setup=None, ell_grid=ELL_GRID, ell_setup=None):
        """Spectra [n][384] for parameter sets p, and the mask of queries the TDSE answered.
        Out-of-trust queries go to the TDSE: those with ellipticity 0 whose disagreement is above
        the threshold to the batched z-linear engine, and every query with ellipticity != 0 (the
        network was trained on z-linear pulses only) to the velocity-gauge elliptical engine on
        ell_grid."""
        thr = self.threshold if threshold is None else threshold
        mean, dis = self.predict(p)
        ell = p["ellipticity"] != 0
        fall = (dis > thr) | ell
        lin = fall & ~ell
        if lin.any():
            sub = {k: v[lin] for k, v in p.items()}
            pes, hhg, _ = tdse_spectra(sub, setup=setup)
            mean[lin] = np.concatenate([pes, hhg], axis=1)
        if ell.any():
            sub = {k: v[ell] for k, v in p.items()}
            pes, hhg, _ = tdse_spectra_elliptical(sub, grid=ell_grid, setup=ell_setup)
            mean[ell] = np.concatenate([pes, hhg], axis=1)
        return mean, fall


def rel_l2(pred, ref):
    """per-row relative L2 error of log-scaled spectra"""
    return np.linalg.norm(pred - ref, axis=1) / np.linalg.norm(ref, axis=1)
