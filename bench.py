#!/usr/bin/env python
"""Benchmark: 3D incompressible hydro, 256^3, FP64, RK4 (dt = 2e-3, nu = 5e-3),
2/3 dealiasing, on one GB300 per rank.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload hydro3d-256-fp64|hydro3d-256-fp32|hydro3d-128-fp64]

A step is one RK4 step (4 fused right-hand sides + stage updates) of the
whole 256^3 state.  The state (3 x 135 MB complex128) and the transform
intermediates are larger than L2 (129 MB), so no L2 flush is needed between
steps.  Prints one JSON line (rank 0).  Multi-GPU runs are independent
replicas (weak scaling, no collective on the data path).

``--impl reference`` times the reference's CPU path (the oracle: the
reference's numpy-FFT algorithm with the C restatement of its Cython stage
kernels) on the host cores, on the same workload.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "256³ hydro steps/s: plain FP64 vs FP32 vs 64³+closure at matched E(k) error"
WORKLOADS = {
    "hydro3d-256-fp64": dict(shape=(256, 256, 256), nu=5e-3, dt=2e-3, precision="fp64"),
    "hydro3d-256-fp32": dict(shape=(256, 256, 256), nu=5e-3, dt=2e-3, precision="fp32"),
    "hydro3d-128-fp64": dict(shape=(128, 128, 128), nu=5e-3, dt=2e-3, precision="fp64"),
    "hydro3d-256-df64": dict(shape=(256, 256, 256), nu=5e-3, dt=2e-3, precision="df64"),
}


def algorithmic_bytes_per_step(N):
    """Canonical bytes of one 3D RK4 step: 4 RHS x 9 FFTs x (1 real + 1 complex
    field pass) + 4 stages x 3 components x 3 complex-array passes."""
    B3 = 8 * N ** 3 + 16 * N ** 2 * (N // 2 + 1)
    C3 = 16 * N ** 2 * (N // 2 + 1)
    return 4 * 9 * B3 + 4 * 3 * 3 * C3


def kernel_bytes(label, shape, precision):
    """Algorithmic bytes of one launch of a fused-hydro kernel (reads + writes
    of the pruned data it must move), keyed by the library's timing label."""
    Nz, Ny, Nx = shape
    Mx, My, Mz = (Nx - 1) // 3, (Ny - 1) // 3, (Nz - 1) // 3
    Kx, Ky, Kz = Mx + 1, 2 * My + 1, 2 * Mz + 1
    cs = 8 if precision == "fp32" else 16           # intermediate complex entry
    kc = Ky * Kz * Kx * 16                          # compact kept complex128 array
    w1 = Ky * Nz * Kx * cs
    w2 = Nz * Ny * Kx * cs
    if label.startswith("z_inv_curl"):
        return 3 * kc + 6 * w1
    if label.startswith("y_inv"):
        return 6 * w1 + 6 * w2
    if label.startswith("x_cross"):
        return 6 * w2 + 3 * w2
    if label.startswith("y_fwd"):
        return 3 * w2 + 3 * w1
    if label.startswith("z_fwd_compact"):
        return 3 * w1 + 3 * kc
    if label.startswith("rk4_stage3"):
        return 3 * kc * 5          # N, y, tot (read) + tot/ys (write), average stage
    return None


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms in the background."""

    FIELDS = ["index", "clocks.sm", "clocks.max.sm", "power.draw", "clocks_event_reasons.active",
              "clocks_event_reasons.hw_slowdown", "clocks_event_reasons.hw_thermal_slowdown",
              "clocks_event_reasons.sw_thermal_slowdown", "clocks_event_reasons.sw_power_cap"]

    def __init__(self, gpu_id=None):
        self.gpu_id = gpu_id
        self.lines = []
        self.proc = None

    def start(self):
        cmd = ["nvidia-smi", "--query-gpu=" + ",".join(self.FIELDS), "--format=csv,noheader,nounits", "-lms", "200"]
        if self.gpu_id:
            cmd += ["-i", self.gpu_id]
        try:
            self.proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=5)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < len(self.FIELDS):
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)), "reasons": sorted(reasons),
                "samples": len(sm)}


def gpu_uuid(torch, dev):
    try:
        u = torch.cuda.get_device_properties(dev).uuid
        return "GPU-" + str(u)
    except Exception:
        return None


def setup_dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def cpu_reference_steps(wl, seed, nsteps, workers, time_budget):
    """Time RK4 steps of the oracle (the reference's CPU algorithm) on the host."""
    import __graft_entry__
    dd = __graft_entry__.load_package()
    from oracle import physics as OP, time_step as OT, representation as OR
    OR.FFT_WORKERS = workers
    u0 = dd.init_cond.turbulence_3d(wl["shape"], seed=seed)
    rhs = OP.IncompressibleHydro(wl["shape"], OR.FourierRepresentation)
    rhs.parameters["nu"] = wl["nu"]
    data = rhs.create_fields(0.)
    for i in range(3):
        data["u"][i]["kspace"] = u0[i]
    ti = OT.RK4(rhs)
    times = []
    t_start = time.perf_counter()
    for s in range(nsteps):
        t0 = time.perf_counter()
        ti.do_advance(data, wl["dt"])
        times.append(time.perf_counter() - t0)
        if time.perf_counter() - t_start + times[-1] > time_budget:
            break
    return times


def run_reference(args, wl, ws, rank):
    if rank != 0:
        return 0
    cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()
    budget = 150.0
    times = cpu_reference_steps(wl, 0, args.warmup + args.steps, cores, budget)
    timed = times[min(args.warmup, len(times) - 1):] if len(times) > 1 else times
    v = len(timed) / sum(timed)
    sample = ("%d RK4 step(s) of the %s workload on the host (warm-up %d of %d requested; stopped at a %.0f s "
              "budget), numpy-FFT algorithm of the reference with pocketfft on %d threads"
              % (len(timed), args.workload, len(times) - len(timed), args.warmup, budget, cores))
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "steps/s", "n_gpus": ws,
            "steps": len(timed), "warmup": len(times) - len(timed), "ms_per_step": 1e3 / v,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded random-phase solenoidal field, E(k)~k^4 exp(-2(k/4)^2), unit energy)",
            "config": config_of(args, wl, ws),
            "cpu_baseline": {"value": v, "unit": "steps/s", "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def config_of(args, wl, ws):
    return {"workload": "%s: 3D incompressible hydro %dx%dx%d, RK4, dt=%g, nu=%g, 2/3 dealiasing, %s"
                        % (args.workload, *wl["shape"], wl["dt"], wl["nu"], wl["precision"]),
            "grid": list(wl["shape"]), "integrator": "RK4 (ETD stages)", "dt": wl["dt"], "nu": wl["nu"],
            "precision": wl["precision"], "parallelism": "replicas x%d" % ws,
            "l2": "inputs larger than L2 (state 406 MB + intermediates), no flush"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="hydro3d-256-fp64", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-variants", action="store_true")
    args = ap.parse_args()
    wl = WORKLOADS[args.workload]
    ws, rank, local = setup_dist()
    if args.impl == "reference":
        return run_reference(args, wl, ws, rank)

    import torch
    import __graft_entry__
    dd = __graft_entry__.load_package()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    dd.config.decfg.set("FFT", "precision", wl["precision"])
    M = dd.mods
    shape = wl["shape"]
    u0 = dd.init_cond.turbulence_3d(shape, seed=rank)
    rhs = M.IncompressibleHydro(shape, M.FourierRepresentation)
    rhs.parameters["nu"] = wl["nu"]
    data = rhs.create_fields(0.)
    for i in range(3):
        data["u"][i]["kspace"] = u0[i]
    ti = M.RK4(rhs)
    dt = wl["dt"]
    stream = torch.cuda.current_stream()
    for _ in range(max(args.warmup, 0)):
        ti.do_advance(data, dt)
    torch.cuda.synchronize()

    def barrier():
        if dist is not None:
            dist.barrier()

    sampler = ClockSampler(gpu_uuid(torch, local))
    sampler.start()
    dd._lib.timing_enable(True)
    dd._lib.timing_reset()
    n0 = dd._lib.launch_count()
    barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        ti.do_advance(data, dt)
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    launches = dd._lib.launch_count() - n0
    ms = e0.elapsed_time(e1)
    kt = dd._lib.timing_report()
    dd._lib.timing_enable(False)
    clocks = sampler.stop()
    if dist is not None:
        t = torch.tensor([ms], dtype=torch.float64, device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    ms_per_step = ms / args.steps
    value = ws * args.steps / (ms / 1e3)

    # dominant kernel roofline (device time from the events around each launch)
    peaks = {}
    pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.isfile(pk):
        peaks = json.load(open(pk))
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    top = max(kt.items(), key=lambda kv: kv[1][1]) if kt else None
    roofline = None
    kernels = {}
    for name, (cnt, tot) in sorted(kt.items(), key=lambda kv: -kv[1][1]):
        b = kernel_bytes(name, shape, wl["precision"])
        kernels[name] = {"launches": cnt, "ms_total": round(tot, 4), "share": round(tot / sum(v[1] for v in kt.values()), 4),
                         "gbs": (round(b / (tot / cnt / 1e3) / 1e9, 1) if b else None)}
    if top:
        name, (cnt, tot) = top
        b = kernel_bytes(name, shape, wl["precision"])
        avg = tot / cnt / 1e3
        ach = b / avg / 1e9 if b else None
        roofline = {"bound": "hbm", "kernel": name, "achieved": ach, "peak": hbm_peak, "unit": "GB/s",
                    "frac": (ach / hbm_peak) if ach else None, "traffic": None,
                    "peak_source": peak_src, "algorithmic_bytes_per_launch": b, "avg_launch_ms": avg * 1e3}
    B = algorithmic_bytes_per_step(shape[0])
    step_hbm = {"algorithmic_bytes_per_step": B, "t_roofline_ms": B / (hbm_peak * 1e9) * 1e3,
                "hbm_frac": (B / (hbm_peak * 1e9)) / (ms_per_step / 1e3),
                "grid_point_stages_per_s": float(np.prod(shape)) * 4 * value}

    # end to end through the public API with host buffers
    e2e = None
    if not args.no_e2e:
        host_in = [torch.from_numpy(c).pin_memory() for c in u0]
        host_out = [torch.empty_like(h).pin_memory() for h in host_in]
        ke = max(3, min(args.steps, 10))
        barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        for _ in range(ke):
            for i in range(3):
                data["u"][i].kdata.copy_(host_in[i], non_blocking=True)
                data["u"][i]._curr_space = "kspace"
                data["u"][i].data = data["u"][i].kdata
            ti.do_advance(data, dt)
            for i in range(3):
                host_out[i].copy_(data["u"][i].kdata, non_blocking=True)
        f1.record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        me = f0.elapsed_time(f1)
        if dist is not None:
            t = torch.tensor([me], dtype=torch.float64, device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            me = float(t.item())
        nb = sum(h.numel() * h.element_size() for h in host_in)
        e2e = {"value": ws * ke / (me / 1e3), "unit": "steps/s", "h2d_bytes_per_step": nb, "d2h_bytes_per_step": nb,
               "steps": ke, "host_wall_s": wall}

    # the same workload with the other transform arithmetics, from the same
    # initial state, with their difference from the FP64 state after the
    # same steps (FP64 native is the reference; it is the headline value)
    variants = None
    if not args.no_variants and wl["precision"] == "fp64":
        variants = {}
        kv = max(3, min(args.steps, 10))
        ref = None

        def run_prec(prec):
            dd.config.decfg.set("FFT", "precision", prec)
            try:
                r = M.IncompressibleHydro(shape, M.FourierRepresentation)
                r.parameters["nu"] = wl["nu"]
                d = r.create_fields(0.)
                for i in range(3):
                    d["u"][i]["kspace"] = u0[i]
                t = M.RK4(r)
                t.do_advance(d, dt)  # warm-up step, part of the compared trajectory
                torch.cuda.synchronize()
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                for _ in range(kv):
                    t.do_advance(d, dt)
                b.record(stream)
                torch.cuda.synchronize()
                out = [d["u"][i].kdata.clone() for i in range(3)]
                del r, d, t
                return a.elapsed_time(b) / kv, out
            finally:
                dd.config.decfg.set("FFT", "precision", "fp64")

        ms64, ref = run_prec("fp64")
        den = sum(float(torch.sum(torch.abs(x) ** 2)) for x in ref)
        for prec in ("df64", "fp32"):
            msv, outv = run_prec(prec)
            num = sum(float(torch.sum(torch.abs(x - y) ** 2)) for x, y in zip(outv, ref))
            variants[prec] = {"steps_per_s": ws * 1e3 / msv, "ms_per_step": msv,
                              "rel_l2_vs_fp64_after_%d_steps" % (kv + 1): (num / den) ** 0.5}
        variants["fp64_repeat"] = {"steps_per_s": ws * 1e3 / ms64, "ms_per_step": ms64}

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        times = cpu_reference_steps(wl, 0, 1, 1, 60.0)
        cpu = {"value": 1.0 / times[0], "unit": "steps/s", "cores": 1, "kind": "port",
               "sample": "1 RK4 step of the %s workload, oracle (reference numpy-FFT algorithm + C restatement "
                         "of its Cython stage kernels), single thread" % args.workload}

    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    if rank != 0:
        return 0
    vs = None
    line = {"metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": vs, "dtype": {"fp64": "f64", "df64": "df64", "fp32": "f32"}[wl["precision"]],
            "data": "synthetic (seeded random-phase solenoidal field, E(k)~k^4 exp(-2(k/4)^2), unit energy)",
            "config": config_of(args, wl, ws), "clocks": clocks, "e2e": e2e, "gpu_launches": launches,
            "roofline": roofline, "step_roofline": step_hbm, "kernels": kernels, "variants": variants,
            "cpu_baseline": cpu}
    print(json.dumps(line))
    return 0


if __name__ == "__main__":
    sys.exit(main())
