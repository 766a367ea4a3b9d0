"""Make the learned LES closure: run the FP64 DNS, sample filtered snapshots,
train the MLP on the GPU, save the weights and (optionally) evaluate the closed
and unclosed 64^3 LES against the filtered DNS.

    python dedalus-1.0_gb300/data/make_closure.py --seeds 50 --snaps 20 \
        --stride 50 --epochs 6 --eval-steps 1000 --out les_closure_256to64.npz \
        --report closure_report.json

Seeds seed0 .. seed0 + seeds - 1 make the training data; the last
``--val-seeds`` of them are held out for validation; the evaluation run uses
``--eval-seed`` (not a training seed).
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
    ap.add_argument("--epochs", type=int, default=6)
    ap.add_argument("--batch", type=int, default=65536)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--lr-min", type=float, default=2e-5)
    ap.add_argument("--init-seed", type=int, default=0)
    ap.add_argument("--eval-steps", type=int, default=0)
    ap.add_argument("--eval-every", type=int, default=100)
    ap.add_argument("--eval-seed", type=int, default=7)
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
    raw, seeds, info = C.generate_dataset(a.seeds, a.snaps, a.stride, a.dns, a.les, a.nu, a.dt, a.seed0, log=log)
    rep["data"] = info
    log("samples: %d (%.1f s of DNS, %d steps)" % (raw.shape[0], info["seconds"], info["dns_steps"]))
    if a.dump_samples:
        g = torch.Generator(device=raw.device)
        g.manual_seed(1)
        pick = torch.randperm(raw.shape[0], generator=g, device=raw.device)[:a.dump_samples]
        np.save(a.dump_path, raw[pick].cpu().numpy())
    cl = C.MLPClosure(info["delta"], seed=a.init_seed)
    cl.set_norm(*C.fit_norm(raw))
    X, T = C.normalise(cl, raw)
    del raw
    torch.cuda.empty_cache()
    npts = (a.les ** 3)
    nval = min(a.val_seeds, a.seeds - 1) * a.snaps * npts
    ntr = X.shape[0] - nval
    tr = torch.arange(ntr, device=X.device, dtype=torch.int64)
    va = torch.arange(ntr, X.shape[0], device=X.device, dtype=torch.int64) if nval else None
    t0 = time.time()
    hist = C.train(cl, X, T, tr, va, epochs=a.epochs, batch=a.batch, lr=a.lr, lr_min=a.lr_min, log=log)
    torch.cuda.synchronize()
    rep["train"] = {"history": hist, "seconds": time.time() - t0, "adam_steps": cl.step,
                    "samples_per_s": a.epochs * (ntr // a.batch) * a.batch / (time.time() - t0)}
    if va is not None:
        rep["train"]["val_correlation"] = C.correlation(cl, X, T, va).tolist()
        log("validation correlation per component: %s" % np.round(rep["train"]["val_correlation"], 3))
    cl.meta = {"data": info, "train": {k: v for k, v in rep["train"].items() if k != "history"},
               "final": hist[-1] if hist else None}
    cl.save(a.out)
    log("saved %s" % a.out)
    if a.report:
        with open(a.report, "w") as f:
            json.dump(rep, f)
    del X, T
    torch.cuda.empty_cache()
    if a.eval_steps:
        ev = C.evaluate(cl, seed=a.eval_seed, dns_n=a.dns, les_n=a.les, nu=a.nu, dt=a.dt, nsteps=a.eval_steps,
                        every=a.eval_every, log=log)
        rep["eval"] = ev
        for name in ev["models"]:
            r = ev[name]
            log("%s: max E(k) err k<=kmax/2 %.4f, k<=kmax %.4f, final diss %.5f + sgs %.5f (DNS %.5f)" % (
                name, max(r["err_half"]), max(r["err_full"]), r["diss"][-1], r["diss_sgs"][-1], ev["dns_diss"][-1]))
    if a.report:
        with open(a.report, "w") as f:
            json.dump(rep, f)


if __name__ == "__main__":
    main()
