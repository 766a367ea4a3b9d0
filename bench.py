#!/usr/bin/env python
"""Benchmarks of the pseudospectral RHS / timestepping path on one GB300 per rank.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload NAME]

Default workload (the headline): 3D incompressible hydro, 256^3, FP64, RK4,
dt = 2e-3, nu = 5e-3, 2/3 dealiasing.  A step is one RK4 step (4 fused
right-hand sides and stage updates) of the whole state.  The state
(3 x 135 MB complex128) and the transform intermediates exceed L2 (129 MB),
so no L2 flush is needed between steps.  Other workloads (one per benchmark
configuration of the project):

    hydro3d-256-{fp64,df64,fp32}  3D hydro 256^3 RK4 with FP64 / double-float / FP32 transforms
    hydro3d-128-{fp64,df64}       the same at 128^3 (small cases for profiling)
    hydro3d-192-fp32              the same at 192^3, FP32 (profiling the x pass's store alignment)
    mhd3d-256-{fp32,fp64}         3D MHD 256^3 RK4, nu = eta = 5e-3, dt = 1e-3
    hydro2d-128                   2D hydro 128^2 RK2mid, nu = 1e-3, dt = 1e-3
    bouss2d-ensemble-512[-fp32]   512 2D Boussinesq runs, sizes uniform in {64,128,256,512}^2,
                                  nu = kappa = 2e-3, N^2 = 1, RK2mid, dt = 1e-2, one CUDA graph per step
                                  (FP64 or autotuned FP32 transforms; the FP32 line reports its
                                  difference from the FP64 ensemble)
    bouss2d-ensemble-64-fp32      64 runs in {256,512}^2, FP32 (small case for profiling)
    les64-closure                 64^3 LES with the learned subgrid closure (trained weights in
                                  dedalus-1.0_gb300/data), RK4, nu = 5e-3, dt = 2e-3, FP32 transforms,
                                  one CUDA graph per step; reports the FP64 256^3 DNS rate beside it

Prints one JSON line (rank 0).  Multi-GPU runs are independent replicas (weak
scaling, no collective on the data path).  ``--impl reference`` times the
reference's CPU algorithm (the oracle: numpy-FFT path with the C restatement of
the Cython stage kernels) on the host cores for the same workload.
"""
import argparse
import json
import os
import re
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

HEADLINE = "256³ hydro steps/s: plain FP64 vs FP32 vs 64³+closure at matched E(k) error"
DATA3 = "synthetic (seeded random-phase solenoidal field, E(k)~k^4 exp(-2(k/4)^2), unit energy)"
WORKLOADS = {
    "hydro3d-256-fp64": dict(kind="hydro3d", shape=(256,) * 3, nu=5e-3, dt=2e-3, precision="fp64"),
    "hydro3d-256-df64": dict(kind="hydro3d", shape=(256,) * 3, nu=5e-3, dt=2e-3, precision="df64"),
    "hydro3d-256-fp32": dict(kind="hydro3d", shape=(256,) * 3, nu=5e-3, dt=2e-3, precision="fp32"),
    "hydro3d-128-fp64": dict(kind="hydro3d", shape=(128,) * 3, nu=5e-3, dt=2e-3, precision="fp64"),
    # 256-point x rows on a grid small enough for a full ncu capture, larger than L2
    "hydro3d-128x128x256-fp64": dict(kind="hydro3d", shape=(128, 128, 256), nu=5e-3, dt=2e-3, precision="fp64"),
    "hydro3d-128-df64": dict(kind="hydro3d", shape=(128,) * 3, nu=5e-3, dt=2e-3, precision="df64"),
    # 192-point rows (64 kept kx: 512-byte FP32 rows, whole 32-byte sectors) beside the 256-point
    # ones (86 kept kx: 688-byte rows): the sector alignment of the x-pass stores
    "hydro3d-192-fp32": dict(kind="hydro3d", shape=(192,) * 3, nu=5e-3, dt=2e-3, precision="fp32"),
    "mhd3d-256-fp32": dict(kind="mhd3d", shape=(256,) * 3, nu=5e-3, dt=1e-3, precision="fp32"),
    "mhd3d-256-fp64": dict(kind="mhd3d", shape=(256,) * 3, nu=5e-3, dt=1e-3, precision="fp64"),
    "hydro2d-128": dict(kind="hydro2d", shape=(128, 128), nu=1e-3, dt=1e-3, precision="fp64"),
    "bouss2d-ensemble-512": dict(kind="ensemble", nrun=512, sizes=(64, 128, 256, 512), nu=2e-3, dt=1e-2,
                                 precision="fp64"),
    "bouss2d-ensemble-512-fp32": dict(kind="ensemble", nrun=512, sizes=(64, 128, 256, 512), nu=2e-3, dt=1e-2,
                                      precision="fp32"),
    "bouss2d-ensemble-64-fp32": dict(kind="ensemble", nrun=64, sizes=(256, 512), nu=2e-3, dt=1e-2,
                                     precision="fp32"),
    "les64-closure": dict(kind="les", shape=(64,) * 3, nu=5e-3, dt=2e-3, precision="fp32"),
}


# DRAM bytes per launch of a workload's dominant kernel from one ncu capture
# (dram__bytes_read.sum + dram__bytes_write.sum), scaled to the full launch by
# the units processed when the capture ran on a smaller grid.
TRAFFIC = {
    ("hydro3d-256-fp64", "x_cross_256_f64"): (
        8 * (67.76e6 + 18.20e6),
        "ncu capture of the same kernel on 128^3 FP64 (67.76 MB read + 18.20 MB written), x8 for 256^3"),
    ("hydro3d-256-fp64", "x_div_256_f64"): (
        4 * (67.81e6 + 50.79e6),
        "ncu capture of the same kernel on 128x128x256 FP64 (67.81 MB read + 50.79 MB written), x4 rows for 256^3"),
    ("hydro3d-256-fp32", "x_div_256_f32"): (
        135.41e6 + 166.06e6, "ncu capture at full size (135.41 MB read + 166.06 MB written)"),
    ("les64-closure", "les_mlp"): (
        9.48e6 + 0.0, "ncu capture at full size (9.48 MB read, stresses still in L2 at kernel end)"),
}


def B3(N):
    return 8 * N ** 3 + 16 * N ** 2 * (N // 2 + 1)


def C3(N):
    return 16 * N ** 2 * (N // 2 + 1)


def B3s(shape):
    nz, ny, nx = shape
    return 8 * nz * ny * nx + 16 * nz * ny * (nx // 2 + 1)


def C3s(shape):
    nz, ny, nx = shape
    return 16 * nz * ny * (nx // 2 + 1)


def B2(N):
    return 8 * N * N + 16 * N * (N // 2 + 1)


def C2(N):
    return 16 * N * (N // 2 + 1)


def bytes_2d(label, runs, cs, ni, no, nf, lo=False):
    """Algorithmic bytes of one launch of a 2D pass for size classes runs
    {N: number of runs in the launch}: compact intermediates W [y][kxc]
    (cs bytes per complex), kept-mode arrays Kx x Ky complex128.  lo: the
    low-storage FP32 step, whose products, stage derivative and stage state
    are complex64 (the state stays complex128)."""
    m = re.search(r"_(\d+)_f(32|64)$", label)
    sizes = [int(m.group(1))] if m else list(runs)
    tot = 0.0
    for N in sizes:
        nr = runs.get(N, 0)
        M = (N - 1) // 3
        Kx, Ky = M + 1, 2 * M + 1
        w, kc = N * Kx * cs, Kx * Ky * 16
        kp = Kx * Ky * 8 if lo else kc            # a compact product / stage region
        if label.startswith("x_prod") or label.startswith("x_div"):
            b = (ni + no) * w
        elif label.startswith("y_inv"):
            b = nf * (kc + kp) / 2 + ni * w        # the state (stage 1) or the stage state (stage 2)
        elif label.startswith("y_fwd_compact"):
            b = no * (w + kp)
        elif label.startswith("rk2mid_stage2d_lo"):
            # stage 1: products, state in, k1 and stage state out; stage 2: products,
            # T and u_dir of the stage state, state and k1 in, state out (mean of the two)
            s1 = no * 8 + nf * 16 + 2 * nf * 8
            s2 = no * 8 + (16 if nf == 3 else 0) + 2 * nf * 16 + nf * 8
            b = (s1 + s2) / 2 * Kx * Ky
        elif label.startswith("rk2mid_stage2d"):
            b = nf * 5 * kc
        else:
            return None
        tot += nr * b
    return tot if m else tot / max(len(sizes), 1)


def fft_flops(shape):
    """Canonical flops of one real transform of a grid: 2.5 n log2 n."""
    n = float(np.prod(shape))
    return 2.5 * n * np.log2(n)


def measured_gemm_tflops(torch, dtype, n=4096, reps=5):
    """FP64 / FP32 (no TF32) cuBLAS GEMM rate on this GPU, best of reps."""
    old = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    try:
        a = torch.randn(n, n, dtype=dtype, device="cuda")
        b = torch.randn(n, n, dtype=dtype, device="cuda")
        torch.matmul(a, b)
        torch.cuda.synchronize()
        best = 0.0
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            torch.matmul(a, b)
            e1.record()
            torch.cuda.synchronize()
            best = max(best, 2.0 * n ** 3 / (e0.elapsed_time(e1) / 1e3) / 1e12)
        return best
    finally:
        torch.backends.cuda.matmul.allow_tf32 = old


# ---------------------------------------------------------------- runners
class Hydro3Runner:
    """3D hydro (kind hydro3d) or MHD (kind mhd3d) with the fused RK4 step."""

    def __init__(self, dd, wl, rank):
        import torch
        self.torch, self.dd, self.wl = torch, dd, wl
        self.mhd = wl["kind"] == "mhd3d"
        shape = wl["shape"]
        dd.config.decfg.set("FFT", "precision", wl["precision"])
        M = dd.mods
        if self.mhd:
            u = dd.init_cond.turbulence_3d(shape, seed=rank, k0=3.0)
            b = dd.init_cond.turbulence_3d(shape, seed=rank + 1000, k0=3.0)
            self.host = u + b
            self.rhs = M.IncompressibleMHD(shape, M.FourierRepresentation)
            self.rhs.parameters.update({"nu": wl["nu"], "eta": wl["nu"]})
            self.names = [("u", 0), ("u", 1), ("u", 2), ("B", 0), ("B", 1), ("B", 2)]
        else:
            self.host = dd.init_cond.turbulence_3d(shape, seed=rank)
            self.rhs = M.IncompressibleHydro(shape, M.FourierRepresentation)
            self.rhs.parameters["nu"] = wl["nu"]
            self.names = [("u", 0), ("u", 1), ("u", 2)]
        self.data = self.rhs.create_fields(0.)
        for (f, c), a in zip(self.names, self.host):
            self.data[f][c]["kspace"] = a
        self.ti = M.RK4(self.rhs)
        self.launches_per_step = None

    def step(self):
        self.ti.do_advance(self.data, self.wl["dt"])

    def state(self):
        return [self.data[f][c].kdata for f, c in self.names]

    def touch(self):
        for f, c in self.names:
            self.data[f][c].touch()

    def divergence_form(self):
        """True when the fused steps ran the divergence form (hydro 3 + 5,
        MHD 6 + 8 transforms per RHS; chosen per step for a solenoidal state)."""
        return getattr(self.rhs, "last_phys3d", 0) in (2, 3)

    def transforms_per_rhs(self):
        if self.mhd:
            return 14 if self.divergence_form() else 18
        return 8 if self.divergence_form() else 9

    def canonical_transforms_per_rhs(self):
        return 18 if self.mhd else 9

    def bytes_per_step(self):
        """Algorithmic bytes: every transform reads and writes one real and one
        complex field (B3), every stage reads/writes three complex passes per
        component (C3); the divergence forms' stages read two more product
        fields."""
        sh = self.wl["shape"]
        nc = 6 if self.mhd else 3
        extra = 4 * 2 * C3s(sh) if self.divergence_form() else 0
        return 4 * self.transforms_per_rhs() * B3s(sh) + 4 * nc * 3 * C3s(sh) + extra

    def canonical_bytes_per_step(self):
        """The curl forms' count (4 RHS x 9 or 18 transforms) for comparison."""
        sh = self.wl["shape"]
        nc = 6 if self.mhd else 3
        return 4 * self.canonical_transforms_per_rhs() * B3s(sh) + 4 * nc * 3 * C3s(sh)

    def point_stages(self):
        return float(np.prod(self.wl["shape"])) * 4

    def flops_per_step(self):
        return 4 * self.transforms_per_rhs() * fft_flops(self.wl["shape"])

    def _nio(self):
        g = 2 if self.mhd else 1
        if self.divergence_form():
            return (6, 8) if self.mhd else (3, 5)
        return 6 * g, 3 * g

    def kernel_flops(self, label):
        """Canonical transform flops of one launch (5 L log2 L per complex
        pencil, 2.5 N log2 N per real row) plus the products."""
        Nz, Ny, Nx = self.wl["shape"]
        Mx, My, Mz = (Nx - 1) // 3, (Ny - 1) // 3, (Nz - 1) // 3
        Kx, Ky = Mx + 1, 2 * My + 1
        ni, no = self._nio()
        cf = lambda L: 5.0 * L * np.log2(L)
        if label.startswith("z_inv"):
            return ni * Kx * Ky * cf(Nz)
        if label.startswith("y_inv"):
            return ni * Kx * Nz * cf(Ny)
        if label.startswith("x_div"):
            return Nz * Ny * ((ni + no) * 0.5 * cf(Nx) + Nx * (24 if self.mhd else 7))
        if label.startswith("x_cross"):
            return Nz * Ny * ((ni + no) * 0.5 * cf(Nx) + Nx * (9 if not self.mhd else 30))
        if label.startswith("y_fwd"):
            return no * Kx * Nz * cf(Ny)
        if label.startswith("z_fwd_compact"):
            return no * Kx * Ky * cf(Nz)
        return None

    kernel_flops_pipe = property(lambda self: {"fp64": "fp64", "fp32": "fp32"}.get(self.wl["precision"]))

    def kernel_bytes(self, label):
        Nz, Ny, Nx = self.wl["shape"]
        Mx, My, Mz = (Nx - 1) // 3, (Ny - 1) // 3, (Nz - 1) // 3
        Kx, Ky, Kz = Mx + 1, 2 * My + 1, 2 * Mz + 1
        cs = 8 if self.wl["precision"] == "fp32" else 16
        kc = Ky * Kz * Kx * 16
        w1, w2 = Ky * Nz * Kx * cs, Nz * Ny * Kx * cs
        g = 2 if self.mhd else 1           # vector fields in the state
        ni, no = self._nio()
        if label.startswith("z_inv"):
            return 3 * g * kc + ni * w1
        if label.startswith("y_inv"):
            return ni * (w1 + w2)
        if label.startswith("x_cross") or label.startswith("x_div"):
            return (ni + no) * w2
        if label.startswith("y_fwd"):
            return no * (w2 + w1)
        if label.startswith("z_fwd_compact"):
            return no * (w1 + kc)
        if label.startswith("rk4_stage3_lo"):
            # FP32 step: complex64 products (no), increment (read + write) and stage state,
            # complex128 state read (a middle stage; the last writes the state instead)
            return no * kc // 2 + 3 * g * (3 * kc // 2 + kc)
        if label.startswith("rk4_stage3"):
            return 3 * g * kc * 5 + (2 * kc if self.divergence_form() else 0)
        if label.startswith("div_sums3"):
            return 3 * kc
        return None

    def config(self, ws):
        w = self.wl
        return {"workload": "%s %dx%dx%d, RK4 (ETD stages), dt=%g, nu=%g%s, 2/3 dealiasing, %s transforms"
                            % ("3D incompressible MHD" if self.mhd else "3D incompressible hydro", *w["shape"], w["dt"],
                               w["nu"], ", eta=%g" % w["nu"] if self.mhd else "", w["precision"]),
                "grid": list(w["shape"]), "integrator": "RK4", "dt": w["dt"], "precision": w["precision"],
                "parallelism": "replicas x%d" % ws, "l2": "inputs larger than L2 (state + intermediates), no flush",
                "nonlinear_form": ("divergence form, %s transforms per RHS (solenoidal state, checked every step)"
                                   % ("6 + 8" if self.mhd else "3 + 5") if self.divergence_form() else
                                   "curl forms, %s transforms per RHS" % ("12 + 6" if self.mhd else "6 + 3"))}

    def metric(self):
        if self.mhd:
            return "256³ MHD steps/s", "steps/s"
        return HEADLINE, "steps/s"


class Hydro2Runner:
    """2D hydro 128^2 with the fused RK2mid step."""

    def __init__(self, dd, wl, rank):
        import torch
        self.torch, self.dd, self.wl = torch, dd, wl
        dd.config.decfg.set("FFT", "precision", wl["precision"])
        M = dd.mods
        self.host = dd.init_cond.turbulence_2d(wl["shape"], seed=rank)
        self.rhs = M.IncompressibleHydro(wl["shape"], M.FourierRepresentation)
        self.rhs.parameters["nu"] = wl["nu"]
        self.data = self.rhs.create_fields(0.)
        for i in range(2):
            self.data["u"][i]["kspace"] = self.host[i]
        self.ti = M.RK2mid(self.rhs)
        # launch-bound at 128^2: one CUDA graph per step (the eager public-API
        # step is the e2e path)
        for _ in range(2):
            self.eager_step()
        torch.cuda.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        cap = torch.cuda.Stream()
        cap.wait_stream(torch.cuda.current_stream())
        n0 = dd._lib.launch_count()
        with torch.cuda.stream(cap):
            with torch.cuda.graph(self.graph, stream=cap):
                self.eager_step()
        torch.cuda.current_stream().wait_stream(cap)
        torch.cuda.synchronize()
        self.launches_per_step = dd._lib.launch_count() - n0
        for i in range(2):
            self.data["u"][i]["kspace"] = self.host[i]

    def step(self):
        self.graph.replay()

    def eager_step(self):
        self.ti.do_advance(self.data, self.wl["dt"])

    api_step = eager_step

    def state(self):
        return [self.data["u"][i].kdata for i in range(2)]

    def bytes_per_step(self):
        N = self.wl["shape"][0]
        return 2 * 5 * B2(N) + 2 * 2 * 3 * C2(N)

    def point_stages(self):
        return float(np.prod(self.wl["shape"])) * 2

    def flops_per_step(self):
        return 2 * 5 * fft_flops(self.wl["shape"])

    def kernel_bytes(self, label):
        cs = 16 if self.wl["precision"] == "fp64" else 8
        return bytes_2d(label, {self.wl["shape"][0]: 1}, cs, 3, 2, 2)

    def config(self, ws):
        w = self.wl
        return {"workload": "2D incompressible hydro %dx%d, RK2mid, dt=%g, nu=%g, 2/3 dealiasing" % (*w["shape"], w["dt"],
                                                                                                  w["nu"]),
                "grid": list(w["shape"]), "integrator": "RK2mid", "dt": w["dt"], "precision": w["precision"],
                "parallelism": "replicas x%d" % ws, "l2": "state fits in L2 (launch-bound workload)",
                "stepping": "one CUDA graph per RK2mid step (e2e: eager public API)"}

    def metric(self):
        return "128² 2D hydro steps/s", "steps/s"


class EnsembleRunner:
    """512 uneven-size 2D Boussinesq runs advanced together (CUDA graph per step)."""

    def __init__(self, dd, wl, rank):
        import torch
        self.torch, self.dd, self.wl = torch, dd, wl
        rng = np.random.Generator(np.random.PCG64(1234 + rank))
        self.sizes = [int(s) for s in rng.choice(wl["sizes"], wl["nrun"])]
        self.ens = dd.ensemble.BoussinesqEnsemble2D(self.sizes, nu=wl["nu"], kappa=wl["nu"],
                                                    precision=wl["precision"])
        self.ens.load_initial_conditions(seed=rank * 100000)
        self.sched = self.ens.autotune(wl["dt"])
        n0 = dd._lib.launch_count()
        self.ens.capture(wl["dt"])
        self.launches_per_step = (dd._lib.launch_count() - n0) // 2   # the eager warm-up + the captured step
        self.host = [c.slab.cpu() for c in self.ens.classes]

    def step(self):
        self.ens.step(self.wl["dt"])

    def eager_step(self):
        self.ens.step(self.wl["dt"], graph=False)

    def state(self):
        return [c.slab for c in self.ens.classes]

    def bytes_per_step(self):
        return self.ens.algorithmic_bytes_per_step()

    def point_stages(self):
        return float(self.ens.grid_point_stages())

    def flops_per_step(self):
        return sum(2 * self.ens.transforms_per_rhs(n) * fft_flops((n, n)) for n in self.sizes)

    def kernel_bytes(self, label):
        cs = 16 if self.wl["precision"] == "fp64" else 8
        div = all(c.phys == 3 for c in self.ens.classes)     # divergence form: 3 inverse, 4 forward fields
        ni, no = (3, 4) if div else (5, 3)
        lo = div and self.wl["precision"] == "fp32"          # the low-storage FP32 step
        b = bytes_2d(label, {n: self.sizes.count(n) for n in self.wl["sizes"]}, cs, ni, no, 3, lo)
        if b is not None and label.startswith("rk2mid_stage2d") and div and not lo:
            b *= 16.0 / 15.0                                  # one more product field read per stage
        return b

    def config(self, ws):
        w = self.wl
        counts = {n: self.sizes.count(n) for n in w["sizes"]}
        return {"workload": "%d independent 2D Boussinesq runs, sizes uniform (seeded) in %s^2 %s, nu=kappa=%g, "
                            "N^2=1, RK2mid, dt=%g, %s, one CUDA graph per ensemble step"
                            % (w["nrun"], list(w["sizes"]), counts, w["nu"], w["dt"], w["precision"]),
                "runs_per_size": counts, "schedule": self.sched, "dt": w["dt"], "precision": w["precision"],
                "parallelism": "replicas x%d" % ws, "l2": "ensemble state (> 1 GB) larger than L2, no flush",
                "nonlinear_form": "divergence form, 3 + 4 transforms per RHS (solenoidal u, checked at capture)"
                if all(c.phys == 3 for c in self.ens.classes) else "curl form, 5 + 3 transforms per RHS"}

    def metric(self):
        return "512-run 2D Boussinesq ensemble steps/s", "ensemble steps/s"


class LesRunner:
    """64^3 LES with the learned closure: the fused closed RK4 step
    (dd_les_rk4_step3d), replayed as one CUDA graph per step."""

    def __init__(self, dd, wl, rank):
        import torch
        self.torch, self.dd, self.wl = torch, dd, wl
        C = dd.closure
        if not os.path.isfile(C.DEFAULT_WEIGHTS):
            raise FileNotFoundError("trained closure weights missing: %s" % C.DEFAULT_WEIGHTS)
        self.cl = C.MLPClosure.load(C.DEFAULT_WEIGHTS)
        self.rhs, self.data, self.ti = C.les_problem(wl["shape"][0], wl["nu"], self.cl, wl["precision"])
        self.host = dd.init_cond.turbulence_3d(wl["shape"], seed=rank)
        for i in range(3):
            self.data["u"][i]["kspace"] = self.host[i]
        for _ in range(2):
            self.eager_step()
        torch.cuda.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        cap = torch.cuda.Stream()
        cap.wait_stream(torch.cuda.current_stream())
        n0 = dd._lib.launch_count()
        with torch.cuda.stream(cap):
            with torch.cuda.graph(self.graph, stream=cap):
                self.eager_step()
        torch.cuda.current_stream().wait_stream(cap)
        torch.cuda.synchronize()
        self.launches_per_step = dd._lib.launch_count() - n0
        for i in range(3):
            self.data["u"][i]["kspace"] = self.host[i]

    def step(self):
        self.graph.replay()

    def eager_step(self):
        self.ti.do_advance(self.data, self.wl["dt"])

    api_step = eager_step

    def state(self):
        return [self.data["u"][i].kdata for i in range(3)]

    def bytes_per_step(self):
        N = self.wl["shape"][0]
        # 4 RHS x 21 transforms (u 3, grad u 9, u x w 3, tau 6) + 4 stages x 3 components x 3 complex passes
        return 4 * 21 * B3(N) + 4 * 3 * 3 * C3(N)

    def point_stages(self):
        return float(np.prod(self.wl["shape"])) * 4

    def flops_per_step(self):
        return 4 * 21 * fft_flops(self.wl["shape"])

    def kernel_bytes(self, label):
        n = int(np.prod(self.wl["shape"]))
        if label == "les_mlp":
            # 9 gradients in, 6 stresses out: float fields on the FP32 path, double on FP64
            return 15 * (4 if self.wl["precision"] == "fp32" else 8) * n
        return None

    def kernel_flops(self, label):
        if label == "les_mlp":
            return 2 * (10 * 64 + 64 * 64 + 64 * 6) * int(np.prod(self.wl["shape"]))
        return None

    def config(self, ws):
        w = self.wl
        meta = self.cl.meta or {}
        return {"workload": "64^3 LES of 3D incompressible hydro with the learned subgrid closure (MLP "
                            "10-64-64-6, BF16 tensor cores), RK4, dt=%g, nu=%g, 2/3 dealiasing, %s transforms, "
                            "one CUDA graph per step" % (w["dt"], w["nu"], w["precision"]),
                "grid": list(w["shape"]), "integrator": "RK4", "dt": w["dt"], "precision": w["precision"],
                "closure_weights": os.path.basename(self.dd.closure.DEFAULT_WEIGHTS),
                "closure_training": meta.get("data"), "closure_accuracy": meta.get("eval"),
                "parallelism": "replicas x%d" % ws, "l2": "state fits in L2 (launch/latency-bound workload)"}

    def metric(self):
        return "64³ LES + closure steps/s", "steps/s"


RUNNERS = {"hydro3d": Hydro3Runner, "mhd3d": Hydro3Runner, "hydro2d": Hydro2Runner, "ensemble": EnsembleRunner,
           "les": LesRunner}


# ---------------------------------------------------------------- CPU side
def cpu_reference_steps(wl, nsteps, workers, time_budget, seed=0):
    """Wall time of RK steps of the oracle (the reference's CPU algorithm)."""
    import __graft_entry__
    dd = __graft_entry__.load_package()
    from oracle import physics as OP, time_step as OT, representation as OR
    OR.FFT_WORKERS = workers
    kind = wl["kind"]
    if kind == "ensemble":
        return cpu_ensemble_times(wl, dd, OP, OT, OR, nsteps, time_budget)
    shape = wl["shape"]
    if kind == "mhd3d":
        rhs = OP.IncompressibleMHD(shape, OR.FourierRepresentation)
        rhs.parameters.update({"nu": wl["nu"], "eta": wl["nu"]})
        u = dd.init_cond.turbulence_3d(shape, seed=seed, k0=3.0)
        b = dd.init_cond.turbulence_3d(shape, seed=seed + 1000, k0=3.0)
        fields = list(zip([("u", 0), ("u", 1), ("u", 2), ("B", 0), ("B", 1), ("B", 2)], u + b))
        ti_cls = OT.RK4
    elif kind == "hydro3d":
        rhs = OP.IncompressibleHydro(shape, OR.FourierRepresentation)
        rhs.parameters["nu"] = wl["nu"]
        fields = list(zip([("u", 0), ("u", 1), ("u", 2)], dd.init_cond.turbulence_3d(shape, seed=seed)))
        ti_cls = OT.RK4
    elif kind == "les":
        from oracle import closure as OC
        z = np.load(dd.closure.DEFAULT_WEIGHTS)
        norm = z["norm"].copy()
        if "gain" in z.files:
            norm[40:46] *= np.float32(z["gain"])
        band = tuple(float(b) for b in z["band"]) if "band" in z.files else (0.0, 0.0)
        shells = z["shell_w"] if "shell_w" in z.files else None
        rhs = OC.les_physics(shape, z["params"], norm, float(z["delta"]), band=band, shells=shells)
        rhs.parameters["nu"] = wl["nu"]
        fields = list(zip([("u", 0), ("u", 1), ("u", 2)], dd.init_cond.turbulence_3d(shape, seed=seed)))
        ti_cls = OT.RK4
    else:
        rhs = OP.IncompressibleHydro(shape, OR.FourierRepresentation)
        rhs.parameters["nu"] = wl["nu"]
        fields = list(zip([("u", 0), ("u", 1)], dd.init_cond.turbulence_2d(shape, seed=seed)))
        ti_cls = OT.RK2mid
    data = rhs.create_fields(0.)
    for (f, c), a in fields:
        data[f][c]["kspace"] = a
    ti = ti_cls(rhs)
    times = []
    t_start = time.perf_counter()
    for _ in range(nsteps):
        t0 = time.perf_counter()
        ti.do_advance(data, wl["dt"])
        times.append(time.perf_counter() - t0)
        if time.perf_counter() - t_start + times[-1] > time_budget:
            break
    return times


def cpu_ensemble_times(wl, dd, OP, OT, OR, nsteps, budget):
    """One oracle run per size class, a few steps each; the ensemble-step time
    is sum over classes of (runs in class) x (time per run-step)."""
    rng = np.random.Generator(np.random.PCG64(1234))
    sizes = [int(s) for s in rng.choice(wl["sizes"], wl["nrun"])]
    per = {}
    for n in wl["sizes"]:
        rhs = OP.BoussinesqHydro((n, n), OR.FourierRepresentation)
        rhs.parameters.update({"nu": wl["nu"], "kappa": wl["nu"], "boussinesq_direction": "y"})
        d = rhs.create_fields(0.)
        d["T"]["kspace"] = dd.init_cond.band_limited_noise_2d((n, n), seed=n)
        ti = OT.RK2mid(rhs)
        ti.do_advance(d, wl["dt"])
        k = 3 if n < 512 else 2
        t0 = time.perf_counter()
        for _ in range(k):
            ti.do_advance(d, wl["dt"])
        per[n] = (time.perf_counter() - t0) / k
    t_step = sum(per[n] for n in sizes)
    return [t_step] * max(1, nsteps)


def run_reference(args, wl, ws, rank):
    if rank != 0:
        return 0
    cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()
    # every requested warm-up and timed step runs (no time budget): one 256^3
    # FP64 step takes a few seconds on all host cores
    budget = float("inf")
    times = cpu_reference_steps(wl, args.warmup + args.steps, cores, budget)
    timed = times[min(args.warmup, len(times) - 1):] if len(times) > 1 else times
    v = len(timed) / sum(timed)
    if wl["kind"] == "ensemble":
        # independent runs spread over all cores
        v = v * cores
        sample = ("one oracle run per size class timed for 2-3 RK2mid steps on one core, summed over the 512 runs "
                  "and divided over %d cores (independent runs)" % cores)
    else:
        sample = ("%d timed step(s) after %d warm-up step(s) of the %s workload on the host, the reference's "
                  "numpy-FFT algorithm with pocketfft on %d threads" % (len(timed), len(times) - len(timed),
                                                                       args.workload, cores))
    metric, unit = metric_of(wl)
    line = {"impl": "reference", "metric": metric, "value": v, "unit": unit, "n_gpus": ws,
            "steps": len(timed), "warmup": len(times) - len(timed), "ms_per_step": 1e3 / v,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": DATA3 if "3d" in wl["kind"] else "synthetic (seeded)",
            "config": {"workload": args.workload, "description": workload_description(wl)},
            "cpu_baseline": {"value": v, "unit": unit, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def workload_description(wl):
    k = wl["kind"]
    if k in ("hydro3d", "mhd3d"):
        return "%s %dx%dx%d, RK4 (ETD stages), dt=%g, nu=%g%s, 2/3 dealiasing" % (
            "3D incompressible MHD" if k == "mhd3d" else "3D incompressible hydro", *wl["shape"], wl["dt"], wl["nu"],
            ", eta=%g" % wl["nu"] if k == "mhd3d" else "")
    if k == "hydro2d":
        return "2D incompressible hydro %dx%d, RK2mid, dt=%g, nu=%g" % (*wl["shape"], wl["dt"], wl["nu"])
    if k == "ensemble":
        return "%d 2D Boussinesq runs, sizes uniform in %s^2, RK2mid, dt=%g, nu=kappa=%g" % (
            wl["nrun"], list(wl["sizes"]), wl["dt"], wl["nu"])
    return "64^3 LES + learned closure, RK4, dt=%g, nu=%g" % (wl["dt"], wl["nu"])


def metric_of(wl):
    return {"hydro3d": (HEADLINE, "steps/s"), "mhd3d": ("256³ MHD steps/s", "steps/s"),
            "hydro2d": ("128² 2D hydro steps/s", "steps/s"),
            "ensemble": ("512-run 2D Boussinesq ensemble steps/s", "ensemble steps/s"),
            "les": ("64³ LES + closure steps/s", "steps/s")}[wl["kind"]]


# ---------------------------------------------------------------- clocks
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

    def mark(self):
        return len(self.lines)

    def stop(self, since=0):
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
        for line in self.lines[since:]:
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
        return "GPU-" + str(torch.cuda.get_device_properties(dev).uuid)
    except Exception:
        return None


def setup_dist():
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


class Replicas:
    """The host side of an N-rank run: independent replicas (one per GPU),
    joined only by barriers and a max over ranks of the timed durations (no
    collective on the data path).  backend "nccl" on GPUs, "gloo" on CPU."""

    def __init__(self, ws, backend="nccl", device=None):
        self.ws = ws
        self.dist = None
        self.device = device
        if ws > 1:
            import torch.distributed as dist
            if backend == "nccl":
                dist.init_process_group("nccl", device_id=device)
            else:
                dist.init_process_group(backend)
            self.dist = dist

    def barrier(self):
        if self.dist is not None:
            self.dist.barrier()

    def max(self, x):
        """Max of a float over ranks (every rank gets it)."""
        if self.dist is None:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64, device=self.device)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def throughput(self, steps, ms_local):
        """(whole-job steps/s over all replicas, slowest rank's ms)."""
        ms = self.max(ms_local)
        return self.ws * steps / (ms / 1e3), ms

    def close(self):
        if self.dist is not None:
            self.dist.barrier()
            self.dist.destroy_process_group()


# ---------------------------------------------------------------- main
def dns_spectrum_error(dd, torch, stream, prec, ref, seed, wl):
    """The 256^3 DNS with `prec` transforms from the same initial state as the
    FP64 reference trajectory `ref` (dns_reference with full_spectrum): the max
    over its record times of the E(k) error against the FP64 DNS spectrum, over
    the reference's bins centred at k <= kmax/2 and k <= kmax (kmax = 85, the
    256^3 grid's 2/3 cutoff), and its steps/s over the trajectory."""
    M = dd.mods
    dd.config.decfg.set("FFT", "precision", prec)
    try:
        shape = (256,) * 3
        rhs = M.IncompressibleHydro(shape, M.FourierRepresentation)
        rhs.parameters["nu"] = wl["nu"]
        data = rhs.create_fields(0.)
        for i, c in enumerate(dd.init_cond.turbulence_3d(shape, seed=seed)):
            data["u"][i]["kspace"] = c
        ti = M.RK4(rhs)
        kc = ref["kc_dns"]
        e_half, e_full, t_run = [], [], 0.0
        for step in range(0, ref["steps"][-1] + 1):
            if step:
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                ti.do_advance(data, ref["dt"])
                b.record(stream)
                b.synchronize()
                t_run += a.elapsed_time(b) / 1e3
            if step % ref["every"] == 0:
                r = ref["steps"].index(step)
                _, e = dd.diagnostics.power_spectrum(data["u"])
                e_half.append(dd.closure.compare_spectra(kc, ref["E_dns"][r], e, 85 / 2.0))
                e_full.append(dd.closure.compare_spectra(kc, ref["E_dns"][r], e, 85.0))
        return {"ek_err_k_le_kmax_over_2_max_over_time": max(e_half), "ek_err_k_le_kmax_max_over_time": max(e_full),
                "steps_per_s_in_trajectory": ref["steps"][-1] / t_run}
    finally:
        dd.config.decfg.set("FFT", "precision", "fp64")


def les_arm(dd, torch, stream, dns_steps_per_s, ws, rank, horizon, test_seed=7):
    """64^3 LES + learned closure (one CUDA graph per RK4 step): steps/s with
    CUDA events, the ratio to the FP64 256^3 DNS steps/s measured in the same
    run, and, after `horizon` steps from the same filtered state on a test
    seed no closure choice used, the max over time of the E(k) error for
    1 <= k <= kmax/2 against the filtered FP64 DNS and the dissipation error
    (LES resolved + closure drain against the DNS total)."""
    wl = WORKLOADS["les64-closure"]
    r = LesRunner(dd, wl, rank)
    for _ in range(3):
        r.step()
    torch.cuda.synchronize()
    n = 200
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for _ in range(n):
        r.step()
    b.record(stream)
    torch.cuda.synchronize()
    les_sps = n * 1e3 / a.elapsed_time(b)
    del r
    out = {"workload": "les64-closure", "description": workload_description(wl),
           "steps_per_s": ws * les_sps, "timed_steps": n, "les_over_dns": les_sps / dns_steps_per_s,
           "target_speed": ">= 20x the plain-DNS steps/s",
           "target_accuracy": "E(k) within 5% for k <= kmax/2 over 1000 steps"}
    if horizon > 0:
        C = dd.closure
        cl = C.MLPClosure.load(C.DEFAULT_WEIGHTS)
        every = max(1, horizon // 10)
        ref = C.dns_reference(test_seed, nsteps=horizon, every=every, dt=wl["dt"], nu=wl["nu"], full_spectrum=True)
        dd.config.decfg.set("FFT", "precision", "fp64")
        for name, model in (("closure", cl), ("no_model", None)):
            t = C.les_trajectory(model, ref, wl["precision"])
            out[name] = {
                "ek_err_k_le_kmax_over_2_max_over_time": max(t["err_half"]),
                "ek_err_k_le_kmax_over_2_final": t["err_half"][-1],
                "ek_err_unit_shells_k_le_kmax_over_2_max_over_time": max(t["err_half_shells"]),
                "ek_err_k_le_kmax_max_over_time": max(t["err_full"]),
                "dissipation_rel_err_final": t["diss_err"][-1],
                "dissipation_rel_err_max_abs_over_time": max(abs(v) for v in t["diss_err"][1:])}
        # the other two arms at the same horizon: the 256^3 DNS with FP32 and
        # double-float transforms against the FP64 DNS spectrum (their own grid)
        for prec in ("fp32", "df64"):
            out["dns_%s" % prec] = dns_spectrum_error(dd, torch, stream, prec, ref, test_seed, wl)
        out["accuracy_check"] = ("test seed %d, %d steps of dt %g from the filtered FP64 256^3 DNS state, compared "
                                 "every %d steps; kmax = %d; E(k) in the reference's spectrum bins (PowerSpectrum) "
                                 "centred at k <= kmax/2, and in unit shells k = 1..kmax/2; "
                                 "dissipation = LES resolved viscous dissipation minus "
                                 "the closure term's energy input, against the DNS dissipation rate"
                                 % (test_seed, horizon, wl["dt"], every, ref["kmax"]))
    return out


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
    ap.add_argument("--no-les", action="store_true", help="leave out the LES arm of the headline line")
    ap.add_argument("--les-horizon", type=int, default=1000,
                    help="steps of the LES accuracy check against the filtered FP64 DNS (headline line)")
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
    reps = Replicas(ws, "nccl", dev)
    barrier, max_over_ranks = reps.barrier, reps.max

    run = RUNNERS[wl["kind"]](dd, wl, rank)
    stream = torch.cuda.current_stream()
    for _ in range(max(args.warmup, 0)):
        run.step()
    torch.cuda.synchronize()

    sampler = ClockSampler(gpu_uuid(torch, local))
    sampler.start()
    t_wait = time.time()
    while sampler.proc is not None and sampler.mark() == 0 and time.time() - t_wait < 3.0:
        time.sleep(0.02)                  # nvidia-smi's first (pre-region) line
    clock_mark = sampler.mark()
    # per-launch CUDA events inside the timed region only where their host cost
    # is negligible (not for CUDA-graph or launch-bound workloads, whose kernel
    # table comes from a separate eager pass after the timed region)
    events_in_timed = run.launches_per_step is None and not getattr(run, "launch_bound", False)
    dd._lib.timing_enable(events_in_timed)
    dd._lib.timing_reset()
    n0 = dd._lib.launch_count()
    barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        run.step()
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    launches = dd._lib.launch_count() - n0
    if run.launches_per_step is not None:
        launches = run.launches_per_step * args.steps      # graph replays launch the captured kernels
    value, ms = reps.throughput(args.steps, e0.elapsed_time(e1))
    kt = dd._lib.timing_report() if events_in_timed else {}
    dd._lib.timing_enable(False)
    # a timed region shorter than the 200 ms sampling period may hold no
    # sample: keep stepping (untimed) until two samples follow its start
    extra = 0
    t_wait = time.time()
    while sampler.proc is not None and sampler.mark() - clock_mark < 2 and time.time() - t_wait < 5.0:
        run.step()
        torch.cuda.synchronize()
        extra += 1
    clocks = sampler.stop(since=clock_mark)
    if clocks is not None:
        clocks["window"] = ("timed region" if extra == 0 else
                            "timed region + %d untimed steps of the same workload right after it" % extra)
    kernel_timing = "CUDA events per launch inside the timed region"
    if not events_in_timed and hasattr(run, "eager_step"):
        kp = max(3, min(args.steps, 20))
        dd._lib.timing_enable(True)
        run.eager_step()
        torch.cuda.synchronize()
        dd._lib.timing_reset()
        for _ in range(kp):
            run.eager_step()
        torch.cuda.synchronize()
        kt = dd._lib.timing_report()
        kernel_timing = "CUDA events per launch in a separate eager pass of %d steps after the timed region" % kp
    dd._lib.timing_enable(False)
    ms_per_step = ms / args.steps

    peaks = {}
    pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.isfile(pk):
        peaks = json.load(open(pk))
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    bf16_peak = float(peaks.get("bf16_tflops", 1900.0))
    _arith = {}

    def arith_peak(pipe):
        if pipe not in _arith:
            _arith[pipe] = measured_gemm_tflops(torch, torch.float64 if pipe == "fp64" else torch.float32)
        return _arith[pipe]
    kernels, roofline = {}, None
    total_kt = sum(v[1] for v in kt.values()) or 1.0
    for name, (cnt, tot) in sorted(kt.items(), key=lambda kv: -kv[1][1]):
        b = run.kernel_bytes(name)
        kernels[name] = {"launches": cnt, "ms_total": round(tot, 4), "share": round(tot / total_kt, 4),
                         "gbs": (round(b / (tot / cnt / 1e3) / 1e9, 1) if b else None)}
    B = run.bytes_per_step()
    if kt:
        name, (cnt, tot) = max(kt.items(), key=lambda kv: kv[1][1])
        b = run.kernel_bytes(name)
        avg = tot / cnt / 1e3
        ach = b / avg / 1e9 if b else None
        tr = TRAFFIC.get((args.workload, name))
        roofline = {"bound": "hbm", "kernel": name, "achieved": ach, "peak": hbm_peak, "unit": "GB/s",
                    "frac": (ach / hbm_peak) if ach else None, "traffic": tr[0] if tr else None,
                    "traffic_source": tr[1] if tr else None, "peak_source": peak_src,
                    "algorithmic_bytes_per_launch": b, "avg_launch_ms": avg * 1e3, "kernel_timing": kernel_timing}
        fl = getattr(run, "kernel_flops", lambda _n: None)(name)
        pipe = getattr(run, "kernel_flops_pipe", "bf16")
        if fl and pipe == "bf16":
            roofline["tensor"] = {"achieved": fl / avg / 1e12, "peak": bf16_peak, "unit": "TFLOP/s",
                                  "frac": fl / avg / 1e12 / bf16_peak, "algorithmic_flops_per_launch": fl}
        elif fl and pipe in ("fp64", "fp32"):
            P = arith_peak(pipe)
            roofline["compute"] = {"pipe": pipe, "achieved": fl / avg / 1e12, "peak": P, "unit": "TFLOP/s",
                                   "frac": fl / avg / 1e12 / P, "algorithmic_flops_per_launch": fl,
                                   "peak_source": "measured cuBLAS %s 4096^3 in this run" % (
                                       "DGEMM" if pipe == "fp64" else "SGEMM (no TF32)")}
    else:
        ach = B / (ms_per_step / 1e3) / 1e9
        roofline = {"bound": "hbm", "kernel": "whole step (CUDA graph)", "achieved": ach, "peak": hbm_peak,
                    "unit": "GB/s", "frac": ach / hbm_peak, "traffic": None, "peak_source": peak_src,
                    "algorithmic_bytes_per_launch": B, "avg_launch_ms": ms_per_step}
    step_hbm = {"algorithmic_bytes_per_step": B, "t_roofline_ms": B / (hbm_peak * 1e9) * 1e3,
                "hbm_frac": (B / (hbm_peak * 1e9)) / (ms_per_step / 1e3),
                "grid_point_stages_per_s": run.point_stages() * value}
    # combined roofline max(B / BW, F / P) with P the measured cuBLAS GEMM rate
    # of the transform arithmetic (FP64 DGEMM, FP32 SGEMM without TF32)
    if wl["precision"] in ("fp64", "fp32") and hasattr(run, "flops_per_step"):
        F = run.flops_per_step()
        P = arith_peak(wl["precision"])
        t_b, t_f = B / (hbm_peak * 1e9), F / (P * 1e12)
        step_hbm.update({"flops_per_step": F, "arith_peak_tflops": P,
                         "arith_peak_source": "measured cuBLAS %s GEMM 4096^3 in this run" % (
                             "DGEMM" if wl["precision"] == "fp64" else "SGEMM (no TF32)"),
                         "t_flops_ms": t_f * 1e3, "combined_bound": "hbm" if t_b >= t_f else "flops",
                         "combined_frac": max(t_b, t_f) / (ms_per_step / 1e3)})
        if hasattr(run, "transforms_per_rhs"):
            step_hbm["transforms_per_rhs"] = run.transforms_per_rhs()
            nt0 = run.canonical_transforms_per_rhs()
            if run.transforms_per_rhs() != nt0:
                # the same step measured against the curl forms' transform count
                F0, B0 = F * nt0 / run.transforms_per_rhs(), run.canonical_bytes_per_step()
                step_hbm["combined_frac_vs_%d_transform_count" % nt0] = max(
                    B0 / (hbm_peak * 1e9), F0 / (P * 1e12)) / (ms_per_step / 1e3)

    # end to end through the public API: the state in from pinned host memory,
    # one step, the state back out, every step
    e2e = None
    if not args.no_e2e:
        host_in = [torch.as_tensor(h).pin_memory() for h in
                   (run.host if isinstance(run.host[0], torch.Tensor) else [torch.from_numpy(h) for h in run.host])]
        host_out = [torch.empty_like(h).pin_memory() for h in host_in]
        dev_state = run.state()
        ke = max(3, min(args.steps, 10))
        barrier()
        torch.cuda.synchronize()
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        api_step = getattr(run, "api_step", run.step)
        for _ in range(ke):
            for d, h in zip(dev_state, host_in):
                d.copy_(h, non_blocking=True)
            getattr(run, "touch", lambda: None)()     # the state was written behind the API's back
            api_step()
            for d, h in zip(dev_state, host_out):
                h.copy_(d, non_blocking=True)
        f1.record(stream)
        torch.cuda.synchronize()
        me = max_over_ranks(f0.elapsed_time(f1))
        nb = sum(h.numel() * h.element_size() for h in host_in)
        e2e = {"value": ws * ke / (me / 1e3), "unit": run.metric()[1], "h2d_bytes_per_step": nb,
               "d2h_bytes_per_step": nb, "steps": ke,
               "path": "eager public API (ti.advance)" if hasattr(run, "api_step") else "same step as value"}

    # the headline workload with the other transform arithmetics, each with its
    # difference from the FP64 state after the same steps
    variants = None
    if not args.no_variants and args.workload == "hydro3d-256-fp64":
        variants = {}
        kv = max(3, min(args.steps, 10))

        def run_prec(prec):
            w2 = dict(wl, precision=prec)
            r = Hydro3Runner(dd, w2, rank)
            try:
                r.step()
                torch.cuda.synchronize()
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                for _ in range(kv):
                    r.step()
                b.record(stream)
                torch.cuda.synchronize()
                return a.elapsed_time(b) / kv, [x.clone() for x in r.state()]
            finally:
                dd.config.decfg.set("FFT", "precision", wl["precision"])

        ms64, ref = run_prec("fp64")
        den = sum(float(torch.sum(torch.abs(x) ** 2)) for x in ref)
        for prec in ("df64", "fp32"):
            msv, outv = run_prec(prec)
            num = sum(float(torch.sum(torch.abs(x - y) ** 2)) for x, y in zip(outv, ref))
            variants[prec] = {"steps_per_s": ws * 1e3 / msv, "ms_per_step": msv,
                              "rel_l2_vs_fp64_after_%d_steps" % (kv + 1): (num / den) ** 0.5}
        variants["ek_error_at_the_les_horizon"] = "les.dns_fp32 / les.dns_df64"
        variants["fp64_repeat"] = {"steps_per_s": ws * 1e3 / ms64, "ms_per_step": ms64}

    # FP32 transforms against FP64 from the same state: per-field error and
    # total-energy drift (MHD), or the whole-ensemble error (ensemble)
    if not args.no_variants and wl["kind"] in ("mhd3d", "ensemble") and wl["precision"] == "fp32":
        kv = max(3, min(args.steps, 10))
        variants = {"steps_compared": kv}

        def states(prec):
            w2 = dict(wl, precision=prec)
            r = RUNNERS[wl["kind"]](dd, w2, rank)
            series = []
            for _ in range(kv):
                r.step()
                if wl["kind"] == "mhd3d":
                    series.append(dd.diagnostics.ekin(r.data) + dd.diagnostics.emag(r.data))
            torch.cuda.synchronize()
            out = [x.clone() for x in r.state()]
            dd.config.decfg.set("FFT", "precision", wl["precision"])
            return out, series

        s32, e32 = states("fp32")
        s64, e64 = states("fp64")
        if wl["kind"] == "mhd3d":
            names = ["u_x", "u_y", "u_z", "B_x", "B_y", "B_z"]
            variants["per_field_rel_l2_vs_fp64"] = {
                n: float(torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(b))
                for n, a, b in zip(names, s32, s64)}
            variants["total_energy_fp64"] = e64
            variants["total_energy_drift_fp32_vs_fp64"] = [(a - b) / b for a, b in zip(e32, e64)]
        else:
            num = sum(float(torch.sum(torch.abs(a - b) ** 2)) for a, b in zip(s32, s64))
            den = sum(float(torch.sum(torch.abs(b) ** 2)) for b in s64)
            variants["ensemble_rel_l2_vs_fp64"] = (num / den) ** 0.5

    # the third arm of the headline metric: the 64^3 LES with the learned
    # closure, timed in this run against the FP64 DNS value above, and its
    # accuracy against the filtered FP64 DNS on a fixed test seed
    les = None
    if not args.no_les and args.workload == "hydro3d-256-fp64":
        les = les_arm(dd, torch, stream, value / ws, ws, rank, args.les_horizon)

    # the LES against the plain FP64 DNS it stands in for (256^3, same nu, dt)
    versus_dns = None
    if wl["kind"] == "les":
        rd = Hydro3Runner(dd, WORKLOADS["hydro3d-256-fp64"], rank)
        rd.step()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(3):
            rd.step()
        b.record(stream)
        torch.cuda.synchronize()
        dns = 3e3 / a.elapsed_time(b)
        versus_dns = {"dns_256_fp64_steps_per_s": dns, "les_over_dns": (value / ws) / dns,
                      "target": ">= 20x the plain-DNS steps/s"}
        del rd
        dd.config.decfg.set("FFT", "precision", "fp64")

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        times = cpu_reference_steps(wl, 1, 1, 60.0)
        cpu = {"value": 1.0 / times[0], "unit": run.metric()[1], "cores": 1, "kind": "port",
               "sample": ("one step of the %s workload, oracle (the reference's numpy-FFT algorithm + C restatement "
                          "of its Cython stage kernels), single thread" % args.workload) if wl["kind"] != "ensemble"
               else "one oracle run per size class timed for 2-3 steps on one core, summed over the 512 runs"}

    reps.close()
    if rank != 0:
        return 0
    # the workload key is the one the reference arm prints; the runner's
    # prose goes to "description"
    config = run.config(ws)
    config["description"] = config.pop("workload")
    config = dict({"workload": args.workload}, **config)
    metric, unit = run.metric()
    line = {"metric": metric, "value": value, "unit": unit, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None,
            "dtype": {"fp64": "f64", "df64": "df64", "fp32": "f32"}[wl["precision"]] + (
                "+bf16 (closure MLP)" if wl["kind"] == "les" else ""),
            "data": (DATA3 if wl["kind"] in ("hydro3d", "mhd3d", "les") else "synthetic (seeded)") + (
                "; closure trained on filtered snapshots of the FP64 256^3 DNS of the same generator"
                if wl["kind"] == "les" else ""), "config": config,
            "clocks": clocks, "e2e": e2e, "gpu_launches": launches, "roofline": roofline,
            "step_roofline": step_hbm, "kernels": kernels, "variants": variants, "cpu_baseline": cpu}
    if versus_dns is not None:
        line["versus_dns"] = versus_dns
    if les is not None:
        line["les"] = les
    print(json.dumps(line))
    return 0


if __name__ == "__main__":
    sys.exit(main())
