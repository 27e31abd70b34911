"""Benchmark of the batched GB300 propagation engine.

Workload (default): the batched laser scan -- 256 hydrogen wavefunctions,
B-splines order 7 (p = 6), N_r = 800 on [0, 400] a.u. with uniform knots,
l_max = 40 (n_l = 41), z-linear length gauge, dt = 0.05, sharing one H0
factorisation; per wavefunction, seeded draws (numpy default_rng(2025)) of the
peak intensity (log-uniform 5e13..5e14 W/cm^2), wavelength (uniform
400..2000 nm), CEP (uniform [0, 2 pi)) and sin^2 cycles (integer 2..10).

One bench step = one time step of every wavefunction in the batch (all 256
are inside their pulse for the first 2207 steps, which is where the timed
window sits).  Metric: wavefunction-steps/s.

  value      device time (CUDA events on the engine's stream) of
             qpc_lgwz_run over the timed steps, states resident in HBM
  e2e        the same steps through the public C ABI with host buffers:
             qpc_lgwz_put (host -> device) + qpc_lgwz_run + qpc_lgwz_get
             (device -> host) per timed step, wall clock
  plain_1wf  the plain one-wavefunction-at-a-time GPU path (n_inst = 1, same
             kernels) on the same grid and fields, device time
  roofline   the dominant kernel (the coupling sweeps), FP64 flops per launch
             over its CUDA-event duration, against the measured FP64 peak
  cpu_baseline  the CPU oracle (a port of the reference's propagator) on the
             host cores, a bounded sample of the same workload

--impl reference times the reference's CPU implementation of the path (the
oracle port: the reference itself needs x86 and MKL) on all host cores.

--workload c2scan runs the whole uneven scan (every wavefunction over its full pulse, 5.46 M
wavefunction-steps, a few minutes) with the plain one-wavefunction path on a sample of the same pulses.
--workload c0 times the reference's own CPU case (one hydrogen atom, N_r = 400, l_max = 20, the whole
4-cycle 800 nm pulse) on the GPU, with the CPU oracle beside it.
--workload c3 runs 64 wavefunctions on mixed grids (one handle each, qpc_lgwz_run_many) for a window;
--workload c3arn the same grids with the Arnoldi propagator (one handle and host thread each).
--workload c3a times the Arnoldi propagator (k_max = 12, dt = 0.1) on --batch wavefunctions
with their own screened potentials on the N_r = 800, n_l = 41 grid.
--workload pcs times the PCS momentum distribution (measure_prj) of 256 resident wavefunctions
(500 |k| x 181 theta, Coulomb waves); --workload tsurff the t-SURFF accumulation after each step
for the same batch and momenta.
--workload c1 measures the single large velocity-gauge elliptical instance over a
window of steps around the pulse peak (a whole 6-cycle pulse at 1800 nm is ~24k steps):
screened Coulomb V = -(1 + 17 e^{-2r})/r, B-splines order 8 (p = 7), N_r = 2000 on
[0, 1000] with quadratic-then-linear knots, l <= 60 for |m| <= 60 in the reference's
rectangular layout (n_m = 121, m0 = -60, n_l = 61: 7381 channels), 1800 nm, ellipticity
0.5, 8e13 W/cm^2, sin^2 envelope of 6 cycles, dt = 0.05.
"""
import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

_FP64_PEAK = {}


def fp64_peak():
    """The FP64 roofline denominator, measured in this run on this GPU: the engine's DFMA
    throughput probe (qpc_fp64_peak, independent FMA chains, best of 5 launches, FMA = 2 flops).
    The HBM and bf16 peaks of MEASURED_PEAKS.json have no FP64 counterpart."""
    if not _FP64_PEAK:
        import importlib
        q = importlib.import_module("qpc-tdse-cpc_gb300")
        _FP64_PEAK["tflops"] = q.fp64_peak()
        _FP64_PEAK["source"] = "measured in this run: DFMA throughput probe qpc_fp64_peak (CUDA events, best of 5)"
    return _FP64_PEAK


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return json.load(fh)
    except Exception:
        return {}


def c2_workload(n_inst=256, seed=2025):
    rng = np.random.default_rng(seed)
    inten = 10 ** rng.uniform(np.log10(5e13), np.log10(5e14), n_inst)
    lam_nm = rng.uniform(400.0, 2000.0, n_inst)
    cep = rng.uniform(0.0, 2 * np.pi, n_inst)
    cyc = rng.integers(2, 11, n_inst)
    return inten, lam_nm, cep, cyc


def c2_config(B, n_r, p, n_l, dt):
    """The config of the batched-scan line, shared by both arms."""
    return {"workload": "batched laser scan: 256 H atoms, N_r=800, p=6, l_max=40, z-linear length gauge, dt=0.05",
            "n_inst": B, "n_r": n_r, "p": p, "n_l": n_l, "dt": dt, "parallelism": "replicas only",
            "l2": "working set %.1f GB > 129 MB L2 (no flush needed)" % ((B * n_l * n_r * 16 * 4 + 8 * B * (n_l // 2) * n_r * 7 * 16) / 1e9)}


def field_tables(q, inten, lam_nm, cep, cyc, dt=0.05):
    tabs = [q.field_sinen(q.intensity_to_e0(I), q.wavelength_to_w0(l), float(c), 0.0, float(p / np.pi), dt)
            for I, l, p, c in zip(inten, lam_nm, cep, cyc)]
    nt = np.array([t.size - 1 for t in tabs], dtype=np.int64)
    return tabs, nt


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self):
        self.p = None
        import tempfile
        self.path = os.environ.get("QPC_CLOCKS_CSV") or os.path.join(tempfile.gettempdir(), "qpc_clocks_%d.csv" % os.getpid())

    def __enter__(self):
        try:
            self.fh = open(self.path, "w")
            self.p = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p is not None:
            self.p.terminate()
            try:
                self.p.wait(5)
            except Exception:
                self.p.kill()
            self.fh.close()

    def summary(self):
        try:
            rows = [l.split(",") for l in open(self.path).read().strip().splitlines() if l.strip()]
        except Exception:
            return None
        if not rows:
            return None
        sm = [float(r[1]) for r in rows]
        mx = float(rows[0][2])
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in rows for n, v in zip(names, r[5:9]) if v.strip() == "Active"})
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": reasons, "samples": len(rows)}


def setup_grid(q, n_r=800, p=6, n_l=41, rmax=400.0):
    t = q.linear_knots(n_r, p, 0.0, rmax)
    S, R, _, _, H = q.radial_setup(n_r, p, n_l, t)
    c0, e = q.ground_state(S, H, n_l)
    return S, R, H, c0


def chain_flops(n_r, p, chains, power):
    """FP64 flops of one chain-kernel launch as implemented (FMA = 2 flops): per
    chain, row and application, both parts do S z ((2p+1) FMA), the forward and
    backward recurrences (2p FMA each), D^-1 y (1 MUL + 1 FMA) and 2x - z (1 FMA)."""
    per_part = 2 * (2 * p + 1) + 2 * (2 * p) + 2 * (2 * p) + 3 + 2
    return chains * n_r * power * 2 * per_part


def path_flops(n_r, p, n_l, power=2):
    """FP64 flops of one wavefunction-step of the batched run (FMA = 2): coupling
    chains (n_l - n_l%2 chains, M^2), field-free chains (n_l), the complex-symmetric
    LDL^T of each channel pair (~217 flops per row) and both l-space transforms."""
    npair = n_l // 2
    chains_c = chain_flops(n_r, p, 2 * npair, power)
    chains_f = chain_flops(n_r, p, n_l, 1)
    factor = npair * n_r * (4 * p * (p + 1) // 2 * 2 + 6 * p + 13)
    even, odd = (n_l + 1) // 2, n_l // 2
    fwd = npair * (2 * 2 * (even + odd) + 4) + (n_l % 2) * 2 * 2 * even
    bwd = even * 2 * 2 * (npair + n_l % 2) + odd * 2 * 2 * npair
    return chains_c + chains_f + factor + n_r * (fwd + bwd)


# DRAM bytes per chain-row of the coupling chain kernel (both applications): one ncu capture
# of a coupling-chain launch at G = 3 (64 instances x 40 chains x 800 rows, two applications),
# dram__bytes_read.sum + dram__bytes_write.sum divided by the chain-rows the launch processed
TRAFFIC_PER_CHAIN_ROW = 252.0


def aggregate_over_ranks(line, batch, device=None):
    """Replicas only: every rank advances its own batch of `batch` wavefunctions.  The whole job's
    value is all ranks' wavefunction-steps over the slowest rank's time (MAX over ranks of the
    per-step time); e2e likewise from the slowest rank.  Needs an initialised process group."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size()
    t = torch.tensor([line["ms_per_step"], -(line.get("e2e") or {}).get("value", 0.0)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    out = dict(line)
    out["n_gpus"] = world
    out["ms_per_step"] = float(t[0].item())
    out["value"] = world * batch * 1e3 / out["ms_per_step"]
    if line.get("e2e"):
        out["e2e"] = dict(line["e2e"], value=world * float(-t[1].item()))
    return out


def run_engine(args, sync=None):
    """sync (optional): called right before and right after the timed steps (a barrier across ranks)"""
    import importlib
    q = importlib.import_module("qpc-tdse-cpc_gb300")
    B, n_r, p, n_l, dt = args.batch, 800, 6, 41, 0.05
    S, R, H, c0 = setup_grid(q, n_r, p, n_l)
    inten, lam_nm, cep, cyc = c2_workload(B)
    tabs, nt = field_tables(q, inten, lam_nm, cep, cyc, dt)
    K, W = args.steps, args.warmup
    assert W + K <= nt.min(), "timed window must stay inside every pulse"
    ftab = np.stack([t[:W + K + 1] for t in tabs])
    state0 = np.repeat(c0[None], B, 0)

    prop = q.propagator_cn_hc_lgwz().initialize(n_r, p, n_l, S, R, H, dt, n_inst=B)
    launches0 = prop.launch_count()
    prop.put(state0)
    # warm-up: W steps (untimed)
    prop.run(ftab[:, :W + 1], np.full(B, W))
    # timed: K steps continuing from t_W (inputs resident, working set > L2)
    q.load()
    with Clocks() as clk:
        launches1 = prop.launch_count()
        prop.enable_profiling(True)
        if sync:
            sync()
        prop.run(ftab[:, W:W + K + 1], np.full(B, K))
        if sync:
            sync()
        dev_ms = prop.last_run_ms()
        ktimes = prop.kernel_times()
        prop.enable_profiling(False)
        gpu_launches = prop.launch_count() - launches1
        # e2e through the C ABI with host buffers, copies inside the timed region
        host_in = np.ascontiguousarray(state0)
        t0 = time.perf_counter()
        prop.put(host_in)
        prop.run(ftab[:, W:W + K + 1], np.full(B, K))
        out = prop.get()
        e2e_s = time.perf_counter() - t0
    clocks = clk.summary()
    # the drop-in adapter's per-step path (propagate(coef, f_ti, f_tf) of the C++ binding): the
    # whole batch state copied to the device and back around every single step, as a caller
    # that keeps the reference's host-side driver loop sees it
    Kpp = min(K, 5)
    t0 = time.perf_counter()
    for i in range(Kpp):
        prop.put(host_in)
        prop.propagate(ftab[:, W + i], ftab[:, W + i + 1])
        out = prop.get()
    pp_s = time.perf_counter() - t0
    value = B * K / (dev_ms * 1e-3)
    e2e = B * K / e2e_s
    state_bytes = state0.nbytes
    h2d = (state_bytes + ftab[:, W:W + K + 1].nbytes) / K
    d2h = state_bytes / K
    # dominant kernel: the coupling chains.  Its launches in the timed region cover
    # all live instances once per step (split over the instance-group streams), so
    # the flops of one launch are the step's coupling flops over the launches per step.
    sw_ms, sw_n = ktimes.get("sweep", (0.0, 0))
    live_pairs = B * (n_l // 2)
    launches_per_step = max(sw_n / max(K, 1), 1.0)
    fl_step = chain_flops(n_r, p, 2 * live_pairs, 2)
    fl = fl_step / launches_per_step
    launch_ms = sw_ms / max(sw_n, 1) if sw_n else None
    achieved = fl / (launch_ms * 1e-3) / 1e12 if sw_n else None
    peaks = load_peaks()
    # algorithmic bytes of the coupling chains per step: each pair's factors (p+1
    # complex per row) read twice per application, each chain's eigen-basis vector
    # read and written once per application, its work vector through the five passes
    sweep_bytes = live_pairs * n_r * 2 * ((p + 1) * 16 * 2 + 2 * 16 * 2 + 2 * 16 * 5) / launches_per_step
    # the whole step: every kernel's FP64 flops per wavefunction-step (path_flops)
    step_flops = path_flops(n_r, p, n_l) * B
    path_tflops = step_flops / (dev_ms / K * 1e-3) / 1e12
    roof = {"bound": "fp64", "kernel": "k_chain<6,G,coupling> (coupling CN chains)", "achieved": achieved,
            "peak": fp64_peak()["tflops"], "unit": "TFLOP/s", "frac": (achieved / fp64_peak()["tflops"]) if achieved else None,
            "peak_source": fp64_peak()["source"],
            "flops_per_launch": fl, "launch_ms": launch_ms, "concurrent_streams": launches_per_step,
            "traffic": (TRAFFIC_PER_CHAIN_ROW * 2 * live_pairs * n_r / launches_per_step) if TRAFFIC_PER_CHAIN_ROW else None,
            "traffic_source": "ncu dram__bytes_read+write of one k_chain coupling launch, scaled by chain-rows",
            "hbm": {"achieved_gbs": sweep_bytes / (launch_ms * 1e-3) / 1e9 if sw_n else None,
                    "peak_gbs": peaks.get("hbm_gbs"), "bytes_per_launch": sweep_bytes},
            "path": {"flops_per_wf_step": path_flops(n_r, p, n_l), "achieved_tflops": path_tflops,
                     "frac": path_tflops / fp64_peak()["tflops"]}}
    if roof["hbm"]["achieved_gbs"] and peaks.get("hbm_gbs"):
        roof["hbm"]["frac"] = roof["hbm"]["achieved_gbs"] / peaks["hbm_gbs"]
    kt = {k: {"ms_total": v[0], "launches": v[1]} for k, v in ktimes.items()}
    tuning = prop.tuning()
    prop.close()

    # plain one-wavefunction GPU path, same kernels, same grid, fields of instance 0
    Kp = min(K, 60)
    pl = q.propagator_cn_hc_lgwz().initialize(n_r, p, n_l, S, R, H, dt, n_inst=1)
    pl.put(c0[None])
    pl.run(ftab[:1, :W + 1], [W])
    pl.run(ftab[:1, W:W + Kp + 1], [Kp])
    plain = Kp / (pl.last_run_ms() * 1e-3)
    tuning_plain = pl.tuning()
    gpu_launches += 0
    pl.close()

    # the CPU sample may run up to the shortest pulse, so that it lasts its time budget
    ftab_cpu = np.stack([t[:int(nt.min()) + 1] for t in tabs])
    cpu = cpu_baseline(q, S, R, H, c0, ftab_cpu, dt, n_l, budget_s=args.cpu_seconds) if not args.no_cpu else None
    line = {
        "metric": "wavefunction-steps/s (batched, 256 wavefunctions)",
        "value": value, "unit": "wf-steps/s", "n_gpus": 1, "steps": K, "warmup": W,
        "ms_per_step": dev_ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c128 (complex FP64)", "data": "synthetic (seeded laser parameters, numpy default_rng(2025))",
        "config": c2_config(B, n_r, p, n_l, dt),
        "e2e": {"value": e2e, "unit": "wf-steps/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "e2e_per_step_propagate": {"value": B * Kpp / pp_s, "unit": "wf-steps/s", "steps": Kpp,
                                   "h2d_bytes_per_step": state_bytes + 2 * B * 8, "d2h_bytes_per_step": state_bytes,
                                   "path": "put + propagate(f_ti, f_tf) + get per step, host buffers (wall clock)"},
        "plain_1wf": {"value": plain, "unit": "wf-steps/s", "ratio_batched_over_plain": value / plain},
        "gpu_launches": gpu_launches,
        "kernels": kt,
        "tuning": {"batched": tuning, "plain": tuning_plain},
        "roofline": roof,
        "cpu_baseline": cpu,
        "clocks": clocks,
    }
    return line


def run_c2scan(args):
    """The whole uneven batched scan: 256 wavefunctions, each over its full pulse (2,253 to
    54,961 steps, 5.46 M wavefunction-steps), device time of one qpc_lgwz_run; beside it the plain
    one-wavefunction path on the same pulses (a sample of instances across the scan, each over a
    window of its pulse: the per-step cost of one wavefunction does not depend on its pulse)."""
    import importlib
    q = importlib.import_module("qpc-tdse-cpc_gb300")
    B, n_r, p, n_l, dt = args.batch, 800, 6, 41, 0.05
    S, R, H, c0 = setup_grid(q, n_r, p, n_l)
    inten, lam_nm, cep, cyc = c2_workload(B)
    tabs, nt = field_tables(q, inten, lam_nm, cep, cyc, dt)
    ld = int(nt.max()) + 1
    ftab = np.zeros((B, ld))
    for k, t in enumerate(tabs):
        ftab[k, :t.size] = t
    prop = q.propagator_cn_hc_lgwz().initialize(n_r, p, n_l, S, R, H, dt, n_inst=B)
    # warm-up (tuning) on a short window, then the whole scan from the ground state
    prop.put(np.repeat(c0[None], B, 0))
    prop.run(ftab[:, :11], np.full(B, 10))
    prop.put(np.repeat(c0[None], B, 0))
    n0 = prop.norm()
    with Clocks() as clk:
        l0 = prop.launch_count()
        prop.run(ftab, nt)
        dev_ms = prop.last_run_ms()
        launches = prop.launch_count() - l0
    clocks = clk.summary()
    drift = float(np.abs(np.sqrt(prop.norm() / n0) - 1.0).max())
    tuning = prop.tuning()
    prop.close()
    value = float(nt.sum()) / (dev_ms * 1e-3)
    # plain path: every 32nd instance of the pulse-length order, 400 steps around its pulse middle
    order = np.argsort(nt)
    sample = [int(k) for k in order[::32]]
    Kp = 400
    pl = q.propagator_cn_hc_lgwz().initialize(n_r, p, n_l, S, R, H, dt, n_inst=1)
    pl.put(c0[None])
    pl.run(ftab[:1, :11], [10])
    ms = 0.0
    for k in sample:
        s0 = int(nt[k]) // 2 - Kp // 2
        pl.put(c0[None])
        pl.run(ftab[k:k + 1, s0:s0 + Kp + 1], [Kp])
        ms += pl.last_run_ms()
    pl.close()
    plain = len(sample) * Kp / (ms * 1e-3)
    return {
        "metric": "wavefunction-steps/s (whole uneven batched scan, 256 wavefunctions)",
        "value": value, "unit": "wf-steps/s", "n_gpus": 1, "steps": int(nt.max()), "warmup": 10,
        "ms_per_step": dev_ms / int(nt.max()), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c128 (complex FP64)", "data": "synthetic (seeded laser parameters, numpy default_rng(2025))",
        "config": dict(c2_config(B, n_r, p, n_l, dt), window="every instance over its whole pulse",
                       wf_steps=int(nt.sum()), pulse_steps_min=int(nt.min()), pulse_steps_max=int(nt.max())),
        "scan_seconds": dev_ms * 1e-3,
        "plain_1wf": {"value": plain, "unit": "wf-steps/s", "ratio_scan_over_plain": value / plain,
                      "sample": "%d instances across the scan, %d steps each around the pulse middle" % (len(sample), Kp)},
        "norm_drift_max": drift, "gpu_launches": int(launches), "tuning": tuning, "clocks": clocks,
    }


def c1_knots(n_r, p, rmax, frac=0.1):
    """Quadratic-then-linear knots (the reference has no such knot generator, functions/basis_bsplines.h:450-526
    offers linear, sine^2, piecewise and exponential ones): the first `frac` of the
    n_r + 2 - p intervals grow quadratically, the rest are uniform with the matching slope."""
    M = n_r + 2 - p
    Mq = max(1, int(round(frac * M)))
    rq = rmax / (1.0 + 2.0 * (M - Mq) / Mq)
    i = np.arange(M + 1, dtype=np.float64)
    r = np.where(i <= Mq, rq * (i / Mq) ** 2, rq + 2.0 * rq / Mq * (i - Mq))
    r[-1] = rmax
    return np.concatenate([np.zeros(p), r, np.full(p, rmax)])


def run_c1(args):
    import importlib
    q = importlib.import_module("qpc-tdse-cpc_gb300")
    n_r, p, n_l, n_m, m0, rmax, dt = 2000, 7, 61, 121, -60, 1000.0, 0.05
    if args.c1_nm:	# a reduced channel set (for profiling runs); the default is the full C1 grid
        n_m, n_l = args.c1_nm, args.c1_nl or n_l
        m0 = -(n_m // 2)
    lam_nm, inten, eps, ncyc = 1800.0, 8e13, 0.5, 6
    kn = c1_knots(n_r, p, rmax)
    nlh = abs(m0) + n_l
    t0 = time.perf_counter()
    S, R, Ri, D, H = q.radial_setup(n_r, p, nlh, kn, (q.POTENTIAL_YUKAWA, 1.0, 17.0, 2.0))
    c_gs, e_gs = q.ground_state(S, H, n_l, n_m, im=-m0, il=0, ir=0, m0=m0)
    prop = q.propagator_cn_hc_vgwr().initialize(n_r, p, n_l, n_m, m0, S, Ri, D, H, dt)
    setup_s = time.perf_counter() - t0
    w0 = q.wavelength_to_w0(lam_nm)
    a0 = q.intensity_to_e0(inten) / w0
    T = ncyc * 2 * np.pi / w0
    K, W = args.steps, args.warmup
    s0 = int(T / dt / 2) - W            # window centred on the pulse peak
    t = dt * (s0 + np.arange(W + K + 1))
    env = np.sin(np.pi * t / T) ** 2
    atab = np.stack([a0 / np.sqrt(1 + eps ** 2) * env * np.cos(w0 * t), a0 * eps / np.sqrt(1 + eps ** 2) * env * np.sin(w0 * t)], 1)
    prop.put(c_gs[None])
    prop.run(atab[None, :W + 1], [W])
    n0 = prop.norm()[0]
    with Clocks() as clk:
        prop.enable_profiling(True)
        prop.run(atab[None, W:W + K + 1], [K])
        dev_ms, launches = prop.last_run()
        ktimes = prop.kernel_times()
        prop.enable_profiling(False)
    clocks = clk.summary()
    n1 = prop.norm()[0]
    nch = n_l * n_m
    # the transforms act per il-parity block and m-parity set (csrc/qpc_vgwr.cu): a transform is one
    # real GEMM per set, n_set x n_set on 2 N_r reals per channel; 10 transforms per step
    sq = 0
    for par in range(2):
        for mpar in range(2):
            n_set = sum(1 for im in range(n_m) if im % 2 == mpar) * sum(1 for il in range(n_l) if il % 2 == par)
            sq += n_set * n_set
    gemm_flops = 10 * 2.0 * (2 * n_r) * sq
    tr_ms, tr_n = ktimes["transform"]
    tfl = gemm_flops * K / (tr_ms * 1e-3) / 1e12 if tr_n else None
    peak = fp64_peak()
    line = {
        "metric": "wavefunction-steps/s (single large elliptical instance, window at the pulse peak)",
        "value": K / (dev_ms * 1e-3), "unit": "wf-steps/s", "n_gpus": 1, "steps": K, "warmup": W,
        "ms_per_step": dev_ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c128 (complex FP64)", "data": "synthetic (ground state of the screened potential, analytic pulse)",
        "config": {"workload": "C1: V=-(1+17e^-2r)/r, p=7, N_r=2000 on [0,1000] quadratic-then-linear knots, n_m=121 (m0=-60), "
                               "n_l=61 (7381 channels), 1800 nm, eps=0.5, 8e13 W/cm^2, 6 cycles, velocity gauge, dt=0.05",
                   "n_m": n_m, "m0": m0, "n_l": n_l, "channels": n_m * n_l,
                   "window_start_step": int(s0 + W), "pulse_steps": int(T / dt), "ground_state_energy": float(e_gs)},
        "gpu_launches": int(launches),
        "roofline": c1_roofline(gemm_flops, tr_ms, tr_n, K, dev_ms, peak),
        "kernels": {k: {"ms_total": v[0], "launch_groups": v[1]} for k, v in ktimes.items()},
        "norm_drift_over_window": abs(n1 - n0) / n0,
        "setup_s": setup_s,
        "clocks": clocks,
    }
    return line


def c1_roofline(gemm_flops, tr_ms, tr_n, K, dev_ms, peak):
    """Roofline of the C1 transforms.  With the slice-product GEMM (the default) every FP64 product
    is 45 bf16 digit-pair products on the tensor cores: the bound is the tensor pipe, achieved =
    45 x the FP64 flops / transform time against the measured bf16 peak, and the FP64-equivalent
    rate is reported beside it against the FP64 (DFMA) peak.  With QPC_VG_GEMM=dfma the bound is
    the FP64 pipe."""
    tfl = gemm_flops * K / (tr_ms * 1e-3) / 1e12 if tr_n else None
    common = {"transform_ms_per_step": tr_ms / K, "share_of_step": tr_ms / dev_ms, "fp64_flops_per_step": gemm_flops}
    if os.environ.get("QPC_VG_GEMM", "slices") == "dfma":
        return {"bound": "fp64", "kernel": "k_dgemm (m,l) transforms with their pairing steps (CUDA events around each transform)",
                "achieved": tfl, "peak": peak["tflops"], "peak_source": peak["source"], "unit": "TFLOP/s",
                "frac": tfl / peak["tflops"] if tfl else None, **common}
    bf = load_peaks().get("bf16_tflops")
    ach = 45 * tfl if tfl else None
    if os.environ.get("QPC_OZ_TC", "1") == "0":
        kname = "k_oz_gemm (mma.sync)"
    else:
        kname = {"0": "k_oz_gemm_tc (tcgen05, cp.async operands)", "1": "k_oz_gemm_tma (tcgen05, TMA from one thread)"}.get(
            os.environ.get("QPC_OZ_TMA", "2"), "k_oz_gemm_ws (tcgen05, TMA producer / MMA / epilogue warps)")
    return {"bound": "tensor", "kernel": kname + ": slice products (9 x 7-bit digits, 45 bf16 pair products per FP64 product) "
                                         "with splitting and pairing steps (CUDA events around each transform)",
            "achieved": ach, "peak": bf, "peak_source": "MEASURED_PEAKS.json bf16_tflops (burst, cuBLAS)", "unit": "TFLOP/s",
            "frac": ach / bf if (ach and bf) else None, "traffic": None,
            "fp64_equivalent": {"achieved": tfl, "peak": peak["tflops"], "peak_source": peak["source"],
                                "ratio_to_fp64_peak": tfl / peak["tflops"] if tfl else None},
            **common}


def arnoldi_flops(n_r, p, n_l, kmax):
    """FP64 flops per complex element and step of the Arnoldi engine (csrc/qpc_arnoldi.cu):
    S-norms (kmax launches) 2(2p+1)+2 FMAs, expansion 3(2p+1) FMA pairs + projections 4(k+1)
    FMAs, S^-1 2(p+1) per real part, Gram-Schmidt 4(k+1), the final combination 4 kmax."""
    fma = 0.0
    for k in range(kmax):
        fma += 2 * (2 * p + 1) + 2                     # S-norm
        fma += 6 * (2 * p + 1) + 4 * (k + 1) + 6       # expand
        if k < kmax - 1:
            fma += 2 * 2 * (p + 1) + 4 * (k + 1)       # S^-1 (re, im) + Gram-Schmidt
    fma += 4 * kmax
    return 2.0 * fma * n_r * n_l


def run_c3arn(args):
    """Arnoldi propagator (k_max = 12, dt = 0.1) on the mixed grids of run_c3.  Wavefunctions on the same
    radial grid and l range share one handle, each with its own screened-Coulomb Hamiltonian (the engine
    takes one H per instance); the handles run together, each driven from its own host thread."""
    import importlib
    import threading
    q = importlib.import_module("qpc-tdse-cpc_gb300")
    rng = np.random.default_rng(2025)
    n_inst, p, dt = args.batch if args.batch != 256 else 64, 6, 0.1
    K, W = args.steps, args.warmup
    groups, flops = {}, 0.0
    for k in range(n_inst):
        n_r = int(rng.choice([400, 800, 1200, 1600, 2000]))
        n_l = int(rng.choice([21, 41, 61, 81]))
        a, b = rng.uniform(0, 17), rng.uniform(1, 3)
        groups.setdefault((n_r, n_l), []).append((a, b))
        flops += arnoldi_flops(n_r, p, n_l, 12)
    props = []
    for (n_r, n_l), pots in sorted(groups.items()):
        kn = q.linear_knots(n_r, p, 0.0, n_r / 2.0)
        Hs = []
        for a, b in pots:
            S, R, _, _, H = q.radial_setup(n_r, p, n_l, kn, (q.POTENTIAL_YUKAWA, 1.0, a, b))
            Hs.append(H)
        c0 = np.zeros((len(pots), 1, n_l, n_r), complex)
        r = np.arange(n_r) * 0.5
        c0[:, 0, 0] = np.exp(-((r - 3.0) / 1.5) ** 2)
        pr = q.propagator_hc_lgwz(12, 1e-14, 1e-8).initialize(n_r, p, n_l, S, R, np.stack(Hs), q.y10_coupling(n_l), dt,
                                                              n_inst=len(pots))
        pr.put(c0)
        props.append(pr)
    ez = 0.03 * np.sin(0.057 * dt * np.arange(W + K))

    def go(tab):
        th = [threading.Thread(target=pr.run, args=(np.repeat(tab[None, :], pr.shape[0], 0),)) for pr in props]
        for t in th:
            t.start()
        for t in th:
            t.join()
    go(ez[:W])
    with Clocks() as clk:
        t0 = time.perf_counter()
        go(ez[W:])
        wall = time.perf_counter() - t0
    tfl = flops * K / wall / 1e12
    return {
        "metric": "wavefunction-steps/s (Arnoldi, mixed grids, one handle per grid, run together)",
        "value": n_inst * K / wall, "unit": "wf-steps/s", "n_gpus": 1, "steps": K, "warmup": W,
        "ms_per_step": wall / K * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c128 (complex FP64)", "data": "synthetic (seeded grids and potentials)",
        "config": {"workload": "C3 (Arnoldi): %d wavefunctions, N_r in {400..2000}, l_max in {20,40,60,80}, "
                               "V=-(1+a e^-br)/r, k_max=12, dt=0.1" % n_inst, "handles": len(props)},
        "timing": "host wall clock around the concurrent runs",
        "roofline": {"bound": "fp64", "kernel": "whole Arnoldi step", "achieved": tfl, "peak": fp64_peak()["tflops"], "unit": "TFLOP/s",
                     "frac": tfl / fp64_peak()["tflops"]},
        "clocks": clk.summary(),
    }


def run_c3a(args):
    """Arnoldi propagator on a batch of wavefunctions with their own screened potentials."""
    import importlib
    q = importlib.import_module("qpc-tdse-cpc_gb300")
    B, n_r, p, n_l, dt, kmax = args.batch, 800, 6, 41, 0.1, 12
    rng = np.random.default_rng(2025)
    kn = q.linear_knots(n_r, p, 0.0, n_r / 2.0)
    Hs = []
    for _ in range(B):
        S, R, _, _, H = q.radial_setup(n_r, p, n_l, kn, (q.POTENTIAL_YUKAWA, 1.0, rng.uniform(0, 17), rng.uniform(1, 3)))
        Hs.append(H)
    c0 = np.stack([q.ground_state(S, H, n_l)[0] for H in Hs])
    prop = q.propagator_hc_lgwz(kmax, 1e-14, 1e-8).initialize(n_r, p, n_l, S, R, np.stack(Hs), q.y10_coupling(n_l), dt, n_inst=B)
    K, W = args.steps, args.warmup
    ez = 0.03 * np.sin(0.057 * dt * np.arange(W + K))[None, :] * np.ones((B, 1))
    prop.put(c0)
    prop.run(ez[:, :W])
    with Clocks() as clk:
        prop.run(ez[:, W:])
        dev_ms, launches = prop.last_run()
    fl = arnoldi_flops(n_r, p, n_l, kmax)
    tfl = fl * B / (dev_ms / K * 1e-3) / 1e12
    return {
        "metric": "wavefunction-steps/s (Arnoldi, k_max = 12, per-instance screened potentials)",
        "value": B * K / (dev_ms * 1e-3), "unit": "wf-steps/s", "n_gpus": 1, "steps": K, "warmup": W,
        "ms_per_step": dev_ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c128 (complex FP64)", "data": "synthetic (seeded screened potentials a in [0,17], b in [1,3])",
        "config": {"workload": "Arnoldi batch: %d wavefunctions, N_r=800 on [0,400], p=6, n_l=41, dt=0.1, k_max=12" % B},
        "gpu_launches": int(launches),
        "roofline": {"bound": "fp64", "kernel": "whole Arnoldi step", "achieved": tfl, "peak": fp64_peak()["tflops"], "unit": "TFLOP/s",
                     "frac": tfl / fp64_peak()["tflops"], "flops_per_wf_step": fl},
        "clocks": clk.summary(),
    }


def run_c0(args):
    """The single hydrogen atom of the reference's CPU case: N_r = 400 on [0, 200], p = 6, l_max = 20,
    800 nm, 1e14 W/cm^2, sin^2 4 cycles, dt = 0.05 (8826 steps), one wavefunction, the whole pulse."""
    import importlib
    q = importlib.import_module("qpc-tdse-cpc_gb300")
    n_r, p, n_l, dt = 400, 6, 21, 0.05
    S, R, H, c0 = setup_grid(q, n_r, p, n_l, 200.0)
    f = q.field_sinen(q.intensity_to_e0(1e14), q.wavelength_to_w0(800.0), 4.0, 0.0, 0.0, dt)
    nt = f.size - 1
    prop = q.propagator_cn_hc_lgwz().initialize(n_r, p, n_l, S, R, H, dt)
    prop.put(c0[None])
    prop.run(f[None, :11], [10])                  # warm-up (autotuner)
    prop.put(c0[None])
    with Clocks() as clk:
        l0 = prop.launch_count()
        t0 = time.perf_counter()
        prop.put(c0[None])
        prop.run(f[None, :], [nt])
        out = prop.get()
        e2e_s = time.perf_counter() - t0
        dev_ms = prop.last_run_ms()
        launches = prop.launch_count() - l0
    norm = prop.norm()[0]
    ktimes = None
    if args.kernel_times:
        # per-kernel device time (CUDA events around every launch) over 1000 steps of the same pulse
        prop.put(c0[None])
        prop.enable_profiling(True)
        prop.run(f[None, :1001], [1000])
        ktimes = {k: {"us_per_step": 1e3 * ms / 1000, "launches": n} for k, (ms, n) in prop.kernel_times().items()}
        ktimes["_step_us_with_events"] = 1e3 * prop.last_run_ms() / 1000
        prop.enable_profiling(False)
    tuning = prop.tuning()
    cpu = cpu_baseline(q, S, R, H, c0, f[None, :], dt, n_l, budget_s=args.cpu_seconds) if not args.no_cpu else None
    return {
        "metric": "wavefunction-steps/s (one hydrogen atom, whole 4-cycle pulse)",
        "value": nt / (dev_ms * 1e-3), "unit": "wf-steps/s", "n_gpus": 1, "steps": nt, "warmup": 10,
        "ms_per_step": dev_ms / nt, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c128 (complex FP64)", "data": "the reference's C0 case (analytic pulse)",
        "config": {"workload": "C0: H atom, N_r=400 on [0,200], p=6, l_max=20, 800 nm, 1e14 W/cm^2, 4 cycles, dt=0.05"},
        "e2e": {"value": nt / e2e_s, "unit": "wf-steps/s", "h2d_bytes_per_step": (c0.nbytes + f.nbytes) / nt,
                "d2h_bytes_per_step": out.nbytes / nt},
        "gpu_launches": int(launches), "final_norm": float(norm), "tuning": tuning, "kernel_times": ktimes,
        "roofline": {"bound": "fp64 (latency: one wavefunction's recurrences are sequential in r)",
                     "kernel": "whole step", "achieved": path_flops(n_r, p, n_l) * nt / (dev_ms * 1e-3) / 1e12,
                     "peak": fp64_peak()["tflops"], "unit": "TFLOP/s",
                     "frac": path_flops(n_r, p, n_l) * nt / (dev_ms * 1e-3) / 1e12 / fp64_peak()["tflops"],
                     "flops_per_step": path_flops(n_r, p, n_l)},
        "cpu_baseline": cpu, "clocks": clk.summary(),
    }


def run_c3(args):
    """Mixed grids: 64 wavefunctions with N_r in {400,...,2000}, l_max in {20,40,60,80} and their own
    screened potential, run together for a window of steps inside their pulses (fields drawn like the
    batched scan).  Wavefunctions on the same grid share one length-gauge handle, each with its own
    potential (qpc_lgwz_create_ex); the handles run together through qpc_lgwz_run_many.  The initial
    state is a normalised Gaussian in the l = 0 channel: the throughput does not depend on it."""
    import importlib
    q = importlib.import_module("qpc-tdse-cpc_gb300")
    rng = np.random.default_rng(2025)
    n_inst, p, dt = args.batch if args.batch != 256 else 64, 6, 0.05
    K, W = args.steps, args.warmup
    inten, lam_nm, cep, cyc = c2_workload(n_inst, seed=7)
    ft, nt = field_tables(q, inten, lam_nm, cep, cyc, dt)
    groups, work = {}, 0
    for k in range(n_inst):
        n_r = int(rng.choice([400, 800, 1200, 1600, 2000]))
        n_l = int(rng.choice([21, 41, 61, 81]))
        a, b = rng.uniform(0, 17), rng.uniform(1, 3)
        groups.setdefault((n_r, n_l), []).append((a, b, k))
        work += n_r * n_l
    props, tabs = [], []
    for (n_r, n_l), members in sorted(groups.items()):
        kn = q.linear_knots(n_r, p, 0.0, n_r / 2.0)
        Hs = []
        for a, b, _ in members:
            S, R, _, _, H = q.radial_setup(n_r, p, n_l, kn, (q.POTENTIAL_YUKAWA, 1.0, a, b))
            Hs.append(H)
        c0 = np.zeros((len(members), 1, n_l, n_r), complex)
        r = np.arange(n_r) * 0.5
        c0[:, 0, 0] = np.exp(-((r - 3.0) / 1.5) ** 2)
        pr = q.propagator_cn_hc_lgwz().initialize(n_r, p, n_l, S, R, np.stack(Hs), dt, n_inst=len(members))
        pr.put(c0)
        props.append(pr)
        tabs.append(np.stack([ft[k][:W + K + 1] for _, _, k in members]))
    q.run_many(props, [t[:, :W + 1] for t in tabs], [np.full(t.shape[0], W) for t in tabs])
    with Clocks() as clk:
        t0 = time.perf_counter()
        q.run_many(props, [t[:, W:] for t in tabs], [np.full(t.shape[0], K) for t in tabs])
        wall = time.perf_counter() - t0
    return {
        "metric": "wavefunction-steps/s (mixed grids, one handle per grid with per-wavefunction potentials, run together)",
        "value": n_inst * K / wall, "unit": "wf-steps/s", "n_gpus": 1, "steps": K, "warmup": W,
        "ms_per_step": wall / K * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c128 (complex FP64)", "data": "synthetic (seeded grids, potentials and fields)",
        "config": {"workload": "C3 (CN): %d wavefunctions, N_r in {400..2000}, l_max in {20,40,60,80}, "
                               "V=-(1+a e^-br)/r, dt=0.05" % n_inst, "channel_rows": int(work), "handles": len(props)},
        "timing": "host wall clock around qpc_lgwz_run_many (%d concurrent handles)" % len(props),
        "clocks": clk.summary(),
    }


def _random_states(B, n_l, n_r, seed):
    """seeded wavefunctions with a decaying radial envelope, S-norm irrelevant to the spectra's cost"""
    rng = np.random.default_rng(seed)
    env = np.exp(-np.arange(n_r) / 200.0)
    return (rng.standard_normal((B, 1, n_l, n_r)) + 1j * rng.standard_normal((B, 1, n_l, n_r))) * env


def _pcs_cpu_baseline(tables, states, budget_s):
    """CPU baseline leg: the oracle's measure_prj, one wavefunction at a time, for about budget_s"""
    from oracle import momentum_oracle as mo
    o = {k: tables[k] for k in ("kr", "ijl", "plm", "exm", "cps")}
    t0 = time.perf_counter()
    n = 0
    while time.perf_counter() - t0 < budget_s or n == 0:
        mo.pcs_measure(o, states[n % len(states)], 0)
        n += 1
    return n / (time.perf_counter() - t0), n


def _tsurff_cpu_baseline(tables, state, dt, budget_s):
    """CPU baseline leg: the oracle's accumulate(az0, az1, dt, coef) on one wavefunction for about budget_s"""
    from oracle import momentum_oracle as mo
    ors = mo.Tsurff(tables, state.shape[1], state.shape[0], 0)
    t0 = time.perf_counter()
    n = 0
    while time.perf_counter() - t0 < budget_s or n == 0:
        ors.accumulate(state, dt, (0.01, 0.011))
        n += 1
    return n / (time.perf_counter() - t0), n


def run_pcs(args):
    """PCS momentum distribution (spectrum_c_pcs::measure_prj) of a resident batch: 256 wavefunctions of
    the batched-scan grid (N_r = 800 on [0, 400], p = 6, l < 41), hydrogenic Coulomb waves, |k| in
    [0.005, 2.5] (500 points), theta_k in [0, pi] (181 points), one phi_k."""
    import importlib
    q = importlib.import_module("qpc-tdse-cpc_gb300")
    B, n_r, p, n_l = args.batch, 800, 6, 41
    nkr, nkt, nkp = 500, 181, 1
    t = q.linear_knots(n_r, p, 0.0, 400.0)
    S, R, _, _, H = q.radial_setup(n_r, p, n_l, t)
    t0 = time.perf_counter()
    pcs = q.spectrum_c_pcs(nkr, nkt, nkp).initialize(n_r, p, n_l, t, 0.005, 2.5, 0.0, np.pi, 0.0, 0.0, 1.0)
    setup_s = time.perf_counter() - t0
    states = _random_states(B, n_l, n_r, 11)
    prop = q.propagator_cn_hc_lgwz().initialize(n_r, p, n_l, S, R, H, 0.05, n_inst=B)
    prop.put(states)
    K, W = min(args.steps, 10), args.warmup
    for _ in range(W):
        pcs.measure_prj(prop)
    with Clocks() as clk:
        dev = []
        for _ in range(K):
            pcs.measure_prj(prop)
            dev.append(pcs.last_run_ms())
        t0 = time.perf_counter()
        for _ in range(K):
            out = pcs.measure_prj(states)          # host buffers in and out, copies inside
        e2e_s = (time.perf_counter() - t0) / K
    dev_ms = float(np.mean(dev))
    nch = n_l
    fl_proj = 4.0 * nkr * B * nch * n_r
    fl_out = B * nkr * nkt * nkp * (4.0 * nch + 8.0)
    tfl = (fl_proj + fl_out) / (dev_ms * 1e-3) / 1e12
    cpu_rate, n_cpu = _pcs_cpu_baseline(pcs.tables, states, min(args.cpu_seconds, 10.0))
    return {
        "metric": "wavefunctions/s (PCS momentum distribution measure_prj, 500 x 181 momenta)",
        "value": B / (dev_ms * 1e-3), "unit": "wavefunctions/s", "n_gpus": 1, "steps": K, "warmup": W,
        "ms_per_step": dev_ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c128 (complex FP64)", "data": "synthetic (seeded wavefunctions, numpy default_rng(11))",
        "config": {"workload": "PCS: %d wavefunctions, N_r=800 on [0,400], p=6, l<41, zc=1, |k| in [0.005,2.5] x 500, "
                               "theta in [0,pi] x 181, one phi" % B, "inputs": "resident batch (134 MB) > L2"},
        "e2e": {"value": B / e2e_s, "unit": "wavefunctions/s", "h2d_bytes_per_step": int(states.nbytes),
                "d2h_bytes_per_step": int(out.nbytes)},
        "gpu_launches": 2 * K,
        "roofline": {"bound": "fp64", "kernel": "k_pcs_proj + k_pcs_out (one measurement)", "achieved": tfl,
                     "peak": fp64_peak()["tflops"], "unit": "TFLOP/s", "frac": tfl / fp64_peak()["tflops"],
                     "flops_per_launch": fl_proj + fl_out, "flops_projection": fl_proj},
        "cpu_baseline": {"value": cpu_rate, "unit": "wavefunctions/s", "cores": os.cpu_count(), "kind": "port",
                         "sample": "%d wavefunctions through the numpy oracle of measure_prj (numpy's BLAS may use every host core)" % n_cpu},
        "tables_setup_s": setup_s, "clocks": clk.summary(),
    }


def run_tsurff(args):
    """t-SURFF accumulation after every step (spectrum_c_tsf::accumulate(az0, az1, dt, coef), the
    driver's call at sphTDSE.cpp:800) for 256 wavefunctions of the batched-scan grid: surface r0 = 200,
    zc = 0, |k| in [0.005, 2.5] (500 points), theta_k in [0, pi] (181 points), one phi_k."""
    import importlib
    q = importlib.import_module("qpc-tdse-cpc_gb300")
    B, n_r, p, n_l, dt = args.batch, 800, 6, 41, 0.05
    nkr, nkt, nkp = 500, 181, 1
    kn = q.linear_knots(n_r, p, 0.0, 400.0)
    S, R, H, c0 = setup_grid(q, n_r, p, n_l)
    inten, lam_nm, cep, cyc = c2_workload(B)
    tabs, nt = field_tables(q, inten, lam_nm, cep, cyc, dt)
    K, W = min(args.steps, 100), args.warmup
    ftab = np.stack([tb[:W + K + 1] for tb in tabs])
    tsf = q.spectrum_c_tsf(nkr, nkt, nkp).initialize(n_r, p, n_l, kn, 200.0, 0.0, 0.005, 2.5, 0.0, np.pi, 0.0, 0.0, n_inst=B)
    prop = q.propagator_cn_hc_lgwz().initialize(n_r, p, n_l, S, R, H, dt, n_inst=B)
    prop.put(_random_states(B, n_l, n_r, 12))
    for i in range(W):
        prop.propagate(ftab[:, i], ftab[:, i + 1])
        tsf.accumulate(prop, dt, np.stack([ftab[:, i], ftab[:, i + 1]], 1))
    with Clocks() as clk:
        acc_ms = []
        t0 = time.perf_counter()
        for i in range(W, W + K):
            prop.propagate(ftab[:, i], ftab[:, i + 1])
            tsf.accumulate(prop, dt, np.stack([ftab[:, i], ftab[:, i + 1]], 1))
            acc_ms.append(tsf.last_run_ms())
        loop_s = (time.perf_counter() - t0) / K
    ms = float(np.mean(acc_ms))
    fl_w = 4.0 * B * nkr * nkt * n_l
    fl = fl_w + B * nkr * n_l * 30.0 + B * nkr * nkt * nkp * 30.0
    tfl = fl / (ms * 1e-3) / 1e12
    w, _ = tsf.get()
    cpu_rate, n_cpu = _tsurff_cpu_baseline(tsf.tables, _random_states(1, n_l, n_r, 13)[0], dt, min(args.cpu_seconds, 10.0))
    return {
        "metric": "wf-steps/s (t-SURFF accumulate, 500 x 181 momenta per wavefunction)",
        "value": B / (ms * 1e-3), "unit": "wf-steps/s", "n_gpus": 1, "steps": K, "warmup": W,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c128 (complex FP64)", "data": "synthetic (seeded wavefunctions and laser parameters)",
        "config": {"workload": "t-SURFF: %d wavefunctions, N_r=800 on [0,400], p=6, l<41, r0=200, zc=0, |k| in [0.005,2.5] x 500, "
                               "theta in [0,pi] x 181, one phi, length-gauge propagator step + accumulate per step" % B,
                   "inputs": "resident batch (134 MB) and spectra (370 MB) > L2"},
        "with_propagation": {"value": B / loop_s, "unit": "wf-steps/s",
                             "note": "host loop of propagate(f_i, f_i+1) + accumulate per step, wall clock"},
        "gpu_launches": 5 * K,
        "roofline": {"bound": "fp64", "kernel": "k_ts_w (l-sum against Y_lm) + k_ts_u + k_ts_acc", "achieved": tfl,
                     "peak": fp64_peak()["tflops"], "unit": "TFLOP/s", "frac": tfl / fp64_peak()["tflops"],
                     "flops_per_launch": fl, "flops_l_sum": fl_w},
        "cpu_baseline": {"value": cpu_rate, "unit": "wf-steps/s", "cores": os.cpu_count(), "kind": "port",
                         "sample": "%d accumulates of one wavefunction through the numpy oracle (numpy's BLAS may use every host core)" % n_cpu},
        "finite": bool(np.isfinite(w).all()), "clocks": clk.summary(),
    }


def cpu_baseline(q, S, R, H, c0, ftab, dt, n_l, budget_s=15.0, threads=None):
    """The CPU oracle (port of the reference's propagator_cn_hc_lgwz), one
    wavefunction per host thread, on a bounded number of steps of the same workload."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from conftest import Oracle
    threads = threads or os.cpu_count()
    o = Oracle()
    # calibrate on one instance
    g1 = o.grid(S, R, H, dt, n_l, n_inst=1)
    t0 = time.perf_counter()
    o.run(g1, c0[None], ftab[:1, :4], [3], [3], threads=1)
    per_step = (time.perf_counter() - t0) / 3
    steps = int(max(3, min(ftab.shape[1] - 1, budget_s / per_step)))
    g = o.grid(S, R, H, dt, n_l, n_inst=threads)
    st = np.repeat(c0[None], threads, 0)
    tab = ftab[:threads, :steps + 1] if ftab.shape[0] >= threads else np.repeat(ftab[:1, :steps + 1], threads, 0)
    t0 = time.perf_counter()
    o.run(g, st, tab, [steps] * threads, [steps] * threads, threads=threads)
    el = time.perf_counter() - t0
    return {"value": threads * steps / el, "unit": "wf-steps/s", "cores": threads, "kind": "port",
            "sample": "%d wavefunctions x %d steps of the same workload, one per host thread (%.1f s)" % (threads, steps, el)}


def run_reference(args):
    import importlib
    q = importlib.import_module("qpc-tdse-cpc_gb300")
    B, n_r, p, n_l, dt = args.batch, 800, 6, 41, 0.05
    S, R, H, c0 = setup_grid(q, n_r, p, n_l)
    inten, lam_nm, cep, cyc = c2_workload(B)
    tabs, nt = field_tables(q, inten, lam_nm, cep, cyc, dt)
    # every sample may run as many steps as its time budget allows (up to the shortest pulse)
    ftab = np.stack([t[:int(nt.min()) + 1] for t in tabs])
    vals = []
    budget = max(2.0, 60.0 / max(args.steps + args.warmup, 1))
    for i in range(args.warmup + args.steps):
        r = cpu_baseline(q, S, R, H, c0, ftab, dt, n_l, budget_s=budget)
        if i >= args.warmup:
            vals.append(r["value"])
    v = float(np.median(vals))
    r["value"] = v
    return {"impl": "reference", "metric": "wavefunction-steps/s (batched, 256 wavefunctions)", "value": v,
            "unit": "wf-steps/s", "n_gpus": 0, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128 (complex FP64)",
            "data": "synthetic (seeded laser parameters, numpy default_rng(2025))",
            "config": c2_config(B, n_r, p, n_l, dt),
            "cpu_baseline": r, "e2e": {"value": v, "unit": "wf-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--batch", type=int, default=256)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--kernel-times", action="store_true", help="c0: per-kernel device times over 1000 steps")
    ap.add_argument("--c1-nm", type=int, default=0, help="c1: number of m channels (default: the full 121)")
    ap.add_argument("--c1-nl", type=int, default=0, help="c1: number of l channels per m (default: the full 61)")
    ap.add_argument("--workload", default="c2", choices=["c2", "c2scan", "c0", "c1", "c3", "c3a", "c3arn", "pcs", "tsurff"])
    args = ap.parse_args()
    if args.workload == "c2scan":
        print(json.dumps(run_c2scan(args)))
        return
    if args.workload == "c0":
        print(json.dumps(run_c0(args)))
        return
    if args.workload == "c3":
        print(json.dumps(run_c3(args)))
        return
    if args.workload == "c1":
        print(json.dumps(run_c1(args)))
        return
    if args.workload == "c3a":
        print(json.dumps(run_c3a(args)))
        return
    if args.workload == "c3arn":
        print(json.dumps(run_c3arn(args)))
        return
    if args.workload == "pcs":
        print(json.dumps(run_pcs(args)))
        return
    if args.workload == "tsurff":
        print(json.dumps(run_tsurff(args)))
        return
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        if rank != 0:
            return
        print(json.dumps(run_reference(args)))
        return
    if world > 1:
        # replicas only: every rank runs its own batch; value = sum over ranks.  The CPU baseline is
        # a 1-GPU figure (rank 0 at N = 1), so no rank takes it here.
        args.no_cpu = True
        import torch
        import torch.distributed as dist
        dist.init_process_group("nccl")
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.barrier()

        def sync():
            torch.cuda.synchronize()
            dist.barrier()
            torch.cuda.synchronize()
        line = aggregate_over_ranks(run_engine(args, sync), args.batch, device="cuda")
        if rank == 0:
            print(json.dumps(line))
        dist.destroy_process_group()
        return
    print(json.dumps(run_engine(args)))


if __name__ == "__main__":
    main()
