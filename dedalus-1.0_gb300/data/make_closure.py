"""Make the learned LES closure: run the FP64 DNS, sample filtered snapshots,
train the MLP on the GPU, choose the closure-term band and gain on a
validation seed, save the weights and evaluate the closed and unclosed 64^3
LES against the filtered DNS on a test seed.

    python dedalus-1.0_gb300/data/make_closure.py --seeds 50 --snaps 20 \
        --stride 50 --epochs 10 --band-target 10.5 21 --select-seed 11 \
        --eval-seed 7 --eval-steps 1000 --report closure_report.json

Seeds seed0 .. seed0 + seeds - 1 make the training data (the last
``--val-seeds`` of them held out for the validation loss); ``--select-seed``
chooses among the candidate closures, ``--eval-seed`` (used for neither)
measures the chosen one.  With ``--band-target lo hi`` a second network is
trained on the stress restricted to that spectral band (the part of tau the
banded closure term uses) and competes in the selection.

The stored closure (les_closure_256to64.npz) was made by the command above.

``--base FILE`` skips the dataset and the training and starts from a stored
network (any weights file written by this script).  ``--calibrate-seeds N``
fits per-shell closure-term weights on training seeds seed0 .. seed0 + N - 1:
the ratio of the exact to the network's subgrid energy transfer per
wavenumber shell, summed over the filtered DNS snapshots
(closure.calibrate_shells); the calibrated closure and its variants then
compete in the selection:

    python dedalus-1.0_gb300/data/make_closure.py --base weights.npz \
        --calibrate-seeds 4 --select-seed 11 --eval-seeds 7 13 17 \
        --eval-steps 1000 --out calibrated.npz --report calibrated.json

(On the stored network's all-mode sibling the calibrated weights lost to the
banded closure on the selection seed.)
"""
import argparse
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--seeds", type=int, default=50)
    ap.add_argument("--snaps", type=int, default=20)
    ap.add_argument("--stride", type=int, default=50)
    ap.add_argument("--seed0", type=int, default=1000)
    ap.add_argument("--val-seeds", type=int, default=5)
    ap.add_argument("--dns", type=int, default=256)
    ap.add_argument("--les", type=int, default=64)
    ap.add_argument("--nu", type=float, default=5e-3)
    ap.add_argument("--dt", type=float, default=2e-3)
    ap.add_argument("--epochs", type=int, default=10)
    ap.add_argument("--batch", type=int, default=65536)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--lr-min", type=float, default=2e-5)
    ap.add_argument("--init-seed", type=int, default=0)
    ap.add_argument("--band-target", type=float, nargs=2, default=None, metavar=("LO", "HI"))
    ap.add_argument("--select-seed", type=int, default=None)
    ap.add_argument("--eval-steps", type=int, default=0)
    ap.add_argument("--eval-every", type=int, default=100)
    ap.add_argument("--eval-seed", type=int, default=7)
    ap.add_argument("--eval-seeds", type=int, nargs="+", default=None, help="evaluate on each (overrides --eval-seed)")
    ap.add_argument("--base", default=None, help="start from this stored network (no dataset, no training)")
    ap.add_argument("--calibrate-seeds", type=int, default=0)
    ap.add_argument("--backscatter", type=float, nargs="+", default=None, metavar="B",
                    help="also select among shell tables gain * ramp(10.5, 21) - B below 10.5 (gain 2)")
    ap.add_argument("--fit-seeds", type=int, nargs="+", default=None,
                    help="with --base: fit the closure-term weight table a posteriori against the FP64 DNS of "
                         "these (training) seeds, then evaluate on --eval-seeds")
    ap.add_argument("--fit-knots", type=float, nargs="+", default=[0.0, 3.0, 6.0, 9.0, 12.0, 16.0, 21.0, 30.0])
    ap.add_argument("--fit-evals", type=int, default=300)
    ap.add_argument("--out", default=os.path.join(HERE, "les_closure_256to64.npz"))
    ap.add_argument("--report", default=None)
    ap.add_argument("--dump-samples", type=int, default=0, help="save this many random raw samples")
    ap.add_argument("--dump-path", default="samples.npy")
    a = ap.parse_args(argv)

    import numpy as np
    import torch
    import __graft_entry__
    dd = __graft_entry__.load_package()
    C = dd.closure
    torch.cuda.set_device(0)

    def log(msg):
        print(msg, flush=True)

    rep = {"args": vars(a)}

    def write_report():
        if a.report:
            with open(a.report, "w") as f:
                json.dump(rep, f)

    band = tuple(a.band_target) if a.band_target else None
    models = {}
    if a.base:
        models["stress"] = C.MLPClosure.load(a.base)
        rep["base"] = {"file": os.path.basename(a.base), "meta": models["stress"].meta}
        if a.fit_seeds:
            return fit_weights(a, C, rep, models["stress"], log, write_report)
        return finish(a, C, rep, models, band, log, write_report)
    raw, seeds, info = C.generate_dataset(a.seeds, a.snaps, a.stride, a.dns, a.les, a.nu, a.dt, a.seed0, log=log,
                                          band=band)
    raw_band = info.pop("raw_band", None)
    rep["data"] = info
    log("samples: %d (%.1f s of DNS, %d steps)" % (raw.shape[0], info["seconds"], info["dns_steps"]))
    if a.dump_samples:
        g = torch.Generator(device=raw.device)
        g.manual_seed(1)
        pick = torch.randperm(raw.shape[0], generator=g, device=raw.device)[:a.dump_samples]
        np.save(a.dump_path, raw[pick].cpu().numpy())
    npts = a.les ** 3
    nval = min(a.val_seeds, a.seeds - 1) * a.snaps * npts

    def fit(samples, name):
        cl = C.MLPClosure(info["delta"], seed=a.init_seed)
        cl.set_norm(*C.fit_norm(samples))
        X, T = C.normalise(cl, samples)
        ntr = X.shape[0] - nval
        tr = torch.arange(ntr, device=X.device, dtype=torch.int64)
        va = torch.arange(ntr, X.shape[0], device=X.device, dtype=torch.int64) if nval else None
        t0 = time.time()
        hist = C.train(cl, X, T, tr, va, epochs=a.epochs, batch=a.batch, lr=a.lr, lr_min=a.lr_min, log=log)
        torch.cuda.synchronize()
        tinfo = {"history": hist, "seconds": time.time() - t0, "adam_steps": cl.step,
                 "samples_per_s": a.epochs * (ntr // a.batch) * a.batch / (time.time() - t0)}
        if va is not None:
            tinfo["val_correlation"] = C.correlation(cl, X, T, va).tolist()
            log("%s: validation correlation per component %s" % (name, np.round(tinfo["val_correlation"], 3)))
        cl.meta = {"data": info, "train": {k: v for k, v in tinfo.items() if k != "history"},
                   "final": hist[-1] if hist else None, "target": name}
        del X, T
        torch.cuda.empty_cache()
        return cl, tinfo

    models["stress"], rep["train"] = fit(raw, "stress")
    del raw
    if raw_band is not None:
        models["band_stress"], rep["train_band"] = fit(raw_band, "band_stress [%g, %g]" % band)
        del raw_band
    torch.cuda.empty_cache()
    write_report()
    finish(a, C, rep, models, band, log, write_report)


def fit_weights(a, C, rep, base, log, write_report):
    """A-posteriori fit of the closure-term weight table (closure.fit_posteriori)
    on the training seeds a.fit_seeds, then evaluation of the fitted closure,
    the starting one and the unclosed LES on a.eval_seeds against the FP64 DNS;
    the fitted closure is saved to a.out."""
    import numpy as np
    knots = list(a.fit_knots)
    if base.shell_w is not None:
        start = np.interp(knots, np.arange(base.shell_w.numel()), base.shell_w.cpu().numpy())
    else:
        lo, hi = base.band
        start = np.clip((np.asarray(knots) - lo) / max(hi - lo, 1e-9), 0.0, 1.0) if hi > 0 else np.ones(len(knots))
    steps = a.eval_steps or 1000
    refs = []
    for s in a.fit_seeds:
        refs.append(C.dns_reference(s, a.dns, a.les, a.nu, a.dt, steps, a.eval_every))
        log("DNS reference seed %d: %.1f s" % (s, refs[-1]["seconds"]))
    w, info = C.fit_posteriori(base, refs, knots, start, max_evals=a.fit_evals, log=log)
    info["fit_seeds"] = list(a.fit_seeds)
    rep["fit"] = info
    log("fitted weights at %s: %s (score %.4f, start %.4f)" % (knots, np.round(w, 4).tolist(),
                                                               info["best"]["score"], info["start"]["score"]))
    write_report()
    fitted = base.with_shells(C.shell_table(knots, w, a.les))
    fitted.meta = dict(base.meta or {})
    fitted.meta["posteriori_fit"] = {"knots": knots, "weights": [float(v) for v in w], "seeds": list(a.fit_seeds),
                                     "score": info["best"]["score"], "steps": steps}
    cands = {"fitted": fitted, "start": base, "no_model": None}
    rep["eval"] = {}
    for seed in (a.eval_seeds or [a.eval_seed]):
        ref = C.dns_reference(seed, a.dns, a.les, a.nu, a.dt, steps, a.eval_every)
        rep["eval"][str(seed)] = {}
        for name, cl in cands.items():
            t = C.les_trajectory(cl, ref)
            rep["eval"][str(seed)][name] = {k: t[k] for k in ("steps", "err_half", "err_half_shells", "err_full",
                                                               "diss_err", "closure_input")}
            log("seed %d %s: max E(k) err k<=kmax/2 %.4f (final %.4f), max |diss err| %.4f (final %+.4f)" % (
                seed, name, max(t["err_half"]), t["err_half"][-1], max(abs(v) for v in t["diss_err"][1:]),
                t["diss_err"][-1]))
        write_report()
    fitted.meta["eval"] = {s: {"err_half_max": max(v["fitted"]["err_half"]),
                               "diss_err_max_abs": max(abs(x) for x in v["fitted"]["diss_err"][1:])}
                           for s, v in rep["eval"].items()}
    fitted.save(a.out)
    log("saved %s" % a.out)
    write_report()


def finish(a, C, rep, models, band, log, write_report):
    """Calibration, selection, storage and evaluation of the closure."""
    import numpy as np
    chosen = models["stress"]
    shells = None
    if a.calibrate_seeds:
        shells, cinfo = C.calibrate_shells(models["stress"], n_seeds=a.calibrate_seeds, n_snap=a.snaps,
                                           stride=a.stride, dns_n=a.dns, les_n=a.les, nu=a.nu, dt=a.dt,
                                           seed0=a.seed0, log=log)
        cinfo["weights"] = shells.tolist()
        rep["calibration"] = cinfo
        log("shell weights %s" % np.round(shells, 3).tolist())
        chosen = models["stress"].with_shells(shells)
        write_report()
    if a.select_seed is not None:
        cands = {"stress_all_modes": models["stress"]}
        for lo, hi, gn in [(10.5, 21.0, 1.0), (10.5, 21.0, 2.0), (10.5, 15.75, 1.5)]:
            cands["stress_band_%g_%g_x%g" % (lo, hi, gn)] = models["stress"].with_band(lo, hi, gn)
        if "band_stress" in models:
            for gn in (1.0, 1.5, 2.0, 3.0):
                cands["band_stress_x%g" % gn] = models["band_stress"].with_band(band[0], band[1], gn)
        if a.backscatter:
            kk = np.arange(C.shell_count(a.les), dtype=np.float64)
            ramp = 2.0 * np.clip((kk - 10.5) / 10.5, 0.0, 1.0)
            for b in a.backscatter:
                w = np.where(kk < 10.5, -b, ramp)
                w[0] = 0.0
                cands["stress_band_x2_backscatter_%g" % b] = models["stress"].with_shells(w)
        if shells is not None:
            cands["stress_shells"] = models["stress"].with_shells(shells)
            cands["stress_shells_no_backscatter"] = models["stress"].with_shells(np.maximum(shells, 0.0))
            for f in (0.8, 1.25):
                cands["stress_shells_x%g" % f] = models["stress"].with_shells(f * shells)
        cands["no_model"] = None
        ev = C.evaluate(cands, seed=a.select_seed, dns_n=a.dns, les_n=a.les, nu=a.nu, dt=a.dt,
                        nsteps=a.eval_steps or 1000, every=a.eval_every, log=log)
        score = {n: max(ev[n]["err_half"]) for n in ev["models"]}
        rep["selection"] = {"seed": a.select_seed, "max_err_k_le_kmax_half": score}
        best = min((n for n in score if n != "no_model"), key=lambda n: score[n])
        chosen = cands[best]
        rep["selection"]["chosen"] = {"name": best, "band": list(chosen.band), "gain": chosen.gain,
                                      "shells": None if chosen.shell_w is None else chosen.shell_w.cpu().tolist()}
        log("selected %s (%.4f) on seed %d" % (best, score[best], a.select_seed))
        write_report()

    chosen.meta["selection"] = rep.get("selection")
    if "calibration" in rep:
        chosen.meta["calibration"] = {k: v for k, v in rep["calibration"].items() if k in ("snapshots", "seed0")}
    chosen.save(a.out)
    log("saved %s" % a.out)
    if a.eval_steps:
        final = {"chosen": chosen, "stress_all_modes": models["stress"], "no_model": None}
        for seed in (a.eval_seeds or [a.eval_seed]):
            ev = C.evaluate(final, seed=seed, dns_n=a.dns, les_n=a.les, nu=a.nu, dt=a.dt, nsteps=a.eval_steps,
                            every=a.eval_every, log=log)
            rep["eval" if seed == (a.eval_seeds or [a.eval_seed])[0] else "eval_%d" % seed] = ev
            for name in ev["models"]:
                r = ev[name]
                log("seed %d %s: max E(k) err k<=kmax/2 %.4f, k<=kmax %.4f, final diss %.5f + sgs %.5f (DNS %.5f)" % (
                    seed, name, max(r["err_half"]), max(r["err_full"]), r["diss"][-1], r["diss_sgs"][-1],
                    ev["dns_diss"][-1]))
            write_report()
    write_report()


if __name__ == "__main__":
    main()
