"""CPU oracle of the momentum spectra (test infrastructure only: imported by tests/, never by the
product).  A numpy restatement, in the reference's loop order, of

  spectrum_c::measure_prj / measure_pad / measure_lmd   spherical/spectrum/momentum_1e.hpp:337-403
  spectrum_c_tsf::prepare + accumulate (ff, z, xy)      spherical/spectrum/momentum_1e.hpp:594-777

on tables of the layouts qpc_pcs_tables / qpc_tsurff_tables produce (and the reference's harness
dumps).  Pinned against the reference itself by tests/golden/pcs_*.npz and tsurff_*.npz.
"""
import numpy as np

SQRT_2_OVER_PI = 0.797884560802865
POWER_OF_MINUS_I = np.array([-1j, -1.0, 1j, 1.0])	# (-i)^(l+1) indexed by l % 4 (momentum_1e.hpp:535-538)


def _l_of(n_l, n_m, m0):
    return np.array([[abs(m0 + im) + il for il in range(n_l)] for im in range(n_m)])


def pcs_measure(t, coef, m0):
    """(lmd [kr][m][l], pmd [kr][kt][kp], pad [kr][kt]) of one wavefunction coef[m][l][r] from the
    tables t (kr, ijl [kr][l][r], plm [kt][m][l], exm [kp][m], cps [kr][l])."""
    n_m, n_l, n_r = coef.shape
    L = _l_of(n_l, n_m, m0)
    ijl, plm, exm, cps, kr = t["ijl"], t["plm"], t["exm"], t["cps"], t["kr"]
    # proj[kr][m][l] = sum_r ijl(kr, l, r) c(m, l, r)   (vecd_proj_vecd, blas1.hpp:396-409)
    proj = np.einsum("kmlr,mlr->kml", ijl[:, L, :], coef)
    cp = cps[:, L]                                   # [kr][m][l]
    lmd = proj * (cp * SQRT_2_OVER_PI)
    pmd = np.einsum("tml,pm,kml->ktp", plm, exm, cp * proj) * SQRT_2_OVER_PI
    pad = np.einsum("tml,kml->kt", plm, cp * proj) * (np.sqrt(kr) * 2.0)[:, None]
    return lmd, pmd, pad


class Tsurff:
    """spectrum_c_tsf for one wavefunction: the clock (time, disx, disy, disz) and work[kr][kt][kp]."""

    def __init__(self, t, n_l, n_m, m0):
        self.t, self.n_l, self.n_m, self.m0 = t, n_l, n_m, m0
        self.L = _l_of(n_l, n_m, m0)
        self.clock = np.zeros(4)
        self.work = np.zeros((t["kr"].size, t["kt"].size, t["kp"].size), complex)

    def accumulate(self, coef, dt, a=None):
        """accumulate(dt, coef), accumulate(az0, az1, dt, coef) with a = (az0, az1), or
        accumulate(ax0, ax1, ay0, ay1, dt, coef) with a = (ax0, ax1, ay0, ay1)."""
        t, n_l, n_m, m0, L = self.t, self.n_l, self.n_m, self.m0, self.L
        ib, b0, br = t["ib"], t["b0"], t["br"]
        temp = coef[:, :, ib] @ b0        # prepare(coef), 606-619
        temq = coef[:, :, ib] @ br
        mode = 0 if a is None else len(a) // 2
        ax = ay = az = 0.0
        if mode == 1:
            az = 0.5 * (a[0] + a[1])
        elif mode == 2:
            ax, ay = 0.5 * (a[0] + a[1]), 0.5 * (a[2] + a[3])
        ck = self.clock                   # prepare(ax, ay, az, dt), 620-626
        ck[0] += dt
        ck[1] += ax * dt
        ck[2] += ay * dt
        ck[3] += az * dt
        j0, jr = t["j0"][:, L], t["jr"][:, L]          # [kr][m][l]
        jdb = -0.5 * (j0 * temq[None] - jr * temp[None])
        if mode == 1:
            iaz = a[1] * 1j
            pm0 = t["pmat"][0]
            prev = np.zeros_like(temp)
            nxt = np.zeros_like(temp)
            prev[:, 1:] = temp[:, :-1] * pm0[:, :-1]
            nxt[:, :-1] = temp[:, 1:] * pm0[:, :-1]
            u = jdb - iaz * j0 * prev[None] - iaz * j0 * nxt[None]
        elif mode == 2:
            iap = (a[1] + a[3] * 1j) * 1j * 0.5
            ias = (a[1] - a[3] * 1j) * 1j * 0.5
            pm1, pm2 = t["pmat"][1], t["pmat"][2]
            u = jdb.copy()
            for im in range(n_m):
                for il in range(n_l):
                    l = L[im, il]
                    # in_check<msh, lsh> (spherical/dimension/1e.hpp:97-100) and 737-752
                    for dm, dl, coefm, pe in ((-1, -1, ias, "jj1"), (-1, 1, ias, "jj2"), (1, -1, iap, "ii2"), (1, 1, iap, "ii1")):
                        jm = im + dm
                        if jm < 0 or jm >= n_m:
                            continue
                        jl = l + dl - abs(m0 + jm)
                        if jl < 0 or jl >= n_l:
                            continue
                        p = {"jj1": pm1[jm, jl], "jj2": pm2[jm, jl], "ii2": pm2[im, il], "ii1": pm1[im, il]}[pe]
                        u[:, im, il] -= coefm * j0[:, im, il] * temp[jm, jl] * p
        else:
            u = jdb
        y = t["y0"][:, None, :, :] * t["e0"][None, :, :, None] * POWER_OF_MINUS_I[L % 4][None, None]   # [kt][kp][m][l]
        s = np.einsum("tpml,kml->ktp", y, u)
        kr, kt, kp = t["kr"], t["kt"], t["kp"]
        K, ST, CT, SP, CP = kr[:, None, None], np.sin(kt)[None, :, None], np.cos(kt)[None, :, None], np.sin(kp)[None, None, :], np.cos(kp)[None, None, :]
        ph = 0.5 * K * K * ck[0]
        if mode != 1:
            ph = ph + K * ST * CP * ck[1] + K * ST * SP * ck[2]
        if mode != 2:
            ph = ph + K * CT * ck[3]
        self.work += s * np.exp(1j * ph) * dt * SQRT_2_OVER_PI
