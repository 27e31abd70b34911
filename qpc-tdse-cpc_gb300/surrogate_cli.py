"""Command line for the spectra surrogate (surrogate.py).

  python qpc-tdse-cpc_gb300/surrogate_cli.py generate --n 1024 --seed 11 --out data_11.npz
      TDSE labels for n parameter sets drawn with the seed (batched engine, GPU).
  python qpc-tdse-cpc_gb300/surrogate_cli.py fit --data data_*.npz --holdout 512 --out report.json
      trains the 5-member ensemble on all but the last `holdout` rows (a validation tenth of
      them held back to calibrate the trust threshold), reports the held-out error, the fallback
      rate at the calibrated threshold, the error of the combined answer (surrogate when trusted,
      TDSE otherwise), and the surrogate's queries/s against the TDSE runs/s measured while
      generating the data; --curve adds the held-out error after fitting a quarter and a half
      of the rows.
"""
import argparse
import glob
import importlib
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
q = importlib.import_module(os.path.basename(HERE))
sg = importlib.import_module(os.path.basename(HERE) + ".surrogate")


def generate(a):
    p = sg.draw_params(a.n, a.seed)
    t0 = time.time()
    pes, hhg, info = sg.tdse_spectra(p, batch=a.batch, log=lambda s: print(s, flush=True))
    info["wall_s"] = time.time() - t0
    np.savez(a.out, pes=pes, hhg=hhg, seed=a.seed, **{k: v for k, v in p.items()},
             wf_steps=info["wf_steps"], run_s=info["run_s"], wall_s=info["wall_s"])
    print(json.dumps({"n": a.n, **info}))


def _errors(sg, s, p, pes, hhg):
    mean, dis = s.predict(p)
    ref = np.concatenate([pes, hhg], axis=1)
    return (sg.rel_l2(mean, ref), sg.rel_l2(mean[:, :sg.N_PES], pes), sg.rel_l2(mean[:, sg.N_PES:], hhg),
            np.sqrt(((mean - ref) ** 2).mean(axis=1)), dis)


def fit(a):
    files = sorted(sum([glob.glob(f) for f in a.data], []))
    parts = [np.load(f) for f in files]
    keys = ["intensity", "wavelength", "cep", "cycles", "ellipticity"]
    p = {k: np.concatenate([d[k] for d in parts]) for k in keys}
    pes = np.concatenate([d["pes"] for d in parts])
    hhg = np.concatenate([d["hhg"] for d in parts])
    tdse_runs = sum(len(d["pes"]) for d in parts)
    tdse_s = sum(float(d["wall_s"]) for d in parts)
    n = len(pes)
    ntr = n - a.holdout
    nval = int(round(ntr * a.val_frac))
    nfit = ntr - nval
    sub = lambda lo, hi: {k: v[lo:hi] for k, v in p.items()}
    tr, va, te = sub(0, nfit), sub(nfit, ntr), sub(ntr, n)
    # learning curve: the same ensemble on the first quarter, half and all of the fitting rows
    curve = []
    if a.curve:
        for frac in (0.25, 0.5):
            m = int(nfit * frac)
            s = sg.Surrogate(seed=a.seed, features=a.features)
            s.fit(sub(0, m), pes[:m], hhg[:m], epochs=int(a.epochs / frac), batch=a.batch, lr=a.lr, stages=a.stages)
            curve.append({"n_fit": m, "holdout_rel_l2_mean": float(_errors(sg, s, te, pes[ntr:], hhg[ntr:])[0].mean())})
    s = sg.Surrogate(seed=a.seed, features=a.features)
    t0 = time.time()
    hist = s.fit(tr, pes[:nfit], hhg[:nfit], epochs=a.epochs, batch=a.batch, lr=a.lr, stages=a.stages)
    train_s = time.time() - t0
    # trust threshold: a quantile of the ensemble's disagreement on validation rows it was not fitted on
    thr = s.calibrate(va, None, a.quantile)
    t0 = time.time()
    e_all, e_pes, e_hhg, rms_dec, dis = _errors(sg, s, te, pes[ntr:], hhg[ntr:])
    pred_s = time.time() - t0
    curve.append({"n_fit": nfit, "holdout_rel_l2_mean": float(e_all.mean())})
    trust = dis <= thr
    # the combined answer: the surrogate for trusted queries, the TDSE (exact labels) for the rest
    combined = np.where(trust, e_all, 0.0)
    # queries/s of the ensemble on a large batch (steady state)
    big = sg.draw_params(65536, 12345)
    s.predict(big)
    t0 = time.time()
    s.predict(big)
    qps = 65536 / (time.time() - t0)
    rep = {
        "files": [os.path.basename(f) for f in files], "n_fit": int(nfit), "n_validation": int(nval), "n_holdout": int(a.holdout),
        "features": a.features, "epochs": a.epochs, "batch": a.batch, "lr": a.lr, "lr_stages": a.stages, "train_s": train_s,
        "final_train_loss": [float(x) for x in hist[-1]],
        "holdout_rel_l2_mean": float(e_all.mean()), "holdout_rel_l2_median": float(np.median(e_all)),
        "holdout_rel_l2_p90": float(np.quantile(e_all, 0.9)),
        "holdout_rel_l2_pes_mean": float(e_pes.mean()), "holdout_rel_l2_hhg_mean": float(e_hhg.mean()),
        "holdout_rms_decades_mean": float(rms_dec.mean()),
        "learning_curve": curve,
        "threshold": thr, "threshold_quantile_on_validation": a.quantile, "trusted_fraction": float(trust.mean()),
        "holdout_rel_l2_trusted_mean": float(e_all[trust].mean()) if trust.any() else None,
        "holdout_rel_l2_untrusted_mean": float(e_all[~trust].mean()) if (~trust).any() else None,
        "corr_disagreement_error": float(np.corrcoef(dis, e_all)[0, 1]),
        "holdout_rel_l2_with_fallback_mean": float(combined.mean()),
        "surrogate_queries_per_s": qps, "tdse_runs_per_s": tdse_runs / tdse_s,
        "holdout_predict_s": pred_s,
    }
    print(json.dumps(rep, indent=1))
    if a.out:
        with open(a.out, "w") as f:
            json.dump(rep, f, indent=1)


def main():
    ap = argparse.ArgumentParser()
    sub = ap.add_subparsers(dest="cmd", required=True)
    g = sub.add_parser("generate")
    g.add_argument("--n", type=int, default=256)
    g.add_argument("--seed", type=int, default=0)
    g.add_argument("--batch", type=int, default=256)
    g.add_argument("--out", required=True)
    f = sub.add_parser("fit")
    f.add_argument("--data", nargs="+", required=True)
    f.add_argument("--holdout", type=int, default=512)
    f.add_argument("--epochs", type=int, default=400)
    f.add_argument("--val-frac", type=float, default=0.1)
    f.add_argument("--curve", action="store_true")
    f.add_argument("--batch", type=int, default=256)
    f.add_argument("--lr", type=float, default=1e-3)
    f.add_argument("--stages", type=int, default=3)
    f.add_argument("--quantile", type=float, default=0.9)
    f.add_argument("--seed", type=int, default=0)
    f.add_argument("--features", default="sym", choices=sg.FEATURES)
    f.add_argument("--out", default=None)
    a = ap.parse_args()
    generate(a) if a.cmd == "generate" else fit(a)


if __name__ == "__main__":
    main()
