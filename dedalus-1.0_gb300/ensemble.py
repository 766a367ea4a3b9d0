"""Ensembles of independent 2D Boussinesq runs of uneven grid sizes, advanced
together on one GPU.

Each run is the reference's 2D ``BoussinesqHydro`` (physics.py:612-721, gravity
along y) integrated with ``RK2mid`` (time_step.py:275-309).  Runs are grouped
by grid size into size classes; a class keeps its runs in one device slab
``[run][field][kx][ky]`` (fields u_x, u_y, T) and one fused C-ABI call
(``dd_rk2mid_step2d`` with nrun > 1) advances a whole chunk of runs.  Size
classes are issued on their own CUDA streams, and a complete ensemble step
(every class, every chunk) is captured once into a CUDA graph and replayed, so
an ensemble step costs one graph launch on the host.

``autotune`` measures, per size class, the tile schedule of its y passes
(dd_plan_set_schedule: the default tile or two smaller ones with the same
radix sequence, so results are bitwise unchanged for classes of more than
one run), the chunking of its runs
(runs per launch) and the order in which classes are issued, keeps the
fastest schedule and caches it in a JSON file keyed by GPU, size, run count
and precision.  Each size class owns its plan, so a tuned schedule does not
leak into other users of the same grid size.
"""
import ctypes
import json
import os
import time

import numpy as np
import torch

from . import _lib
from .engine import Plan, dptr
from . import init_cond

PHYS_BOUSS = 1
PHYS_BOUSS_DIV = 3            # divergence form, for solenoidal velocities
DIV_TOL2 = 1e-24
# FP32 transforms keep the increments, and so the state's divergence, at FP32
# accuracy (the low-storage step projects in float): a relative divergence up
# to 1e-6, below the FP32 path's own error, still takes the divergence form.
DIV_TOL2_FP32 = 1e-12
_TUNE_ENV = "DD_TUNE_CACHE"


def _default_cache():
    return os.environ.get(_TUNE_ENV, os.path.join(os.path.expanduser("~"), ".cache", "dedalus_gb300", "tune.json"))


class _SizeClass:
    def __init__(self, n, runs, precision, device):
        self.n = n
        self.runs = list(runs)                    # global run indices
        self.nrun = len(self.runs)
        self.shape = (n, n)
        self.plan = Plan(self.shape, (2 * np.pi, 2 * np.pi), '2/3 cython')   # own plan: own tile schedule
        self.ysched = 0
        kx, ky = self.plan.kshape
        self.kshape = (kx, ky)
        self.fsize = kx * ky                      # complex entries per field
        self.slab = torch.zeros((self.nrun, 3, kx, ky), dtype=torch.complex128, device=device)
        self.precision = precision
        self.chunk = self.nrun
        self.ws = None
        self.stream = torch.cuda.Stream(device=device)
        self.phys = PHYS_BOUSS

    def set_ysched(self, v):
        _lib.call("dd_plan_set_schedule", self.plan.handle, 0, int(v))
        self.ysched = int(v)

    def ysched_count(self):
        v, n = ctypes.c_int(), ctypes.c_int()
        _lib.call("dd_plan_get_schedule", self.plan.handle, 0, ctypes.byref(v), ctypes.byref(n))
        return n.value

    def workspace(self, chunk):
        n = ctypes.c_size_t()
        _lib.call("dd_rhs2d_workspace_size", self.plan.handle, chunk, self.precision, ctypes.byref(n))
        if self.ws is None or self.ws.numel() < n.value:
            self.ws = torch.empty(n.value, dtype=torch.uint8, device=self.slab.device)
        return self.ws


class BoussinesqEnsemble2D:
    """Ensemble of 2D Boussinesq runs (u = (u_x, u_y), T) of sizes ``sizes``."""

    def __init__(self, sizes, nu=2e-3, kappa=2e-3, g=1., alpha_t=1., beta=1., precision='fp64',
                 viscosity_order=1, device=None):
        self.sizes = [int(n) for n in sizes]
        self.device = torch.device('cuda', torch.cuda.current_device() if device is None else device)
        self.prec = {'fp64': _lib.DD_FP64, 'fp32': _lib.DD_FP32}[precision]
        self.precision = precision
        self.nu, self.kappa, self.vo = float(nu), float(kappa), int(viscosity_order)
        self.params = (ctypes.c_double * 4)(float(g), float(alpha_t), float(beta), 1.0)   # direction y
        self.classes = []
        for n in sorted(set(self.sizes)):
            runs = [i for i, s in enumerate(self.sizes) if s == n]
            self.classes.append(_SizeClass(n, runs, self.prec, self.device))
        self.order = list(range(len(self.classes)))
        self.time = 0.
        self.iteration = 0
        # per size class: 1 while some run may hold energy outside the kept
        # modes (their decay is then applied every step), 0 once known clean
        self._nonkept = {c.n: ctypes.c_int(1) for c in self.classes}
        self._tables = {}
        self._graph = None
        self._graph_dt = None

    # ---------------------------------------------------------------- state
    def load_initial_conditions(self, seed=0, kmax=8.0, amplitude=1e-3):
        """T: white noise of rms `amplitude` band-limited to |k| <= kmax, u = 0,
        seeded per run (seed + run index)."""
        for c in self.classes:
            host = np.zeros((c.nrun, 3) + c.kshape, dtype=np.complex128)
            for j, r in enumerate(c.runs):
                host[j, 2] = init_cond.band_limited_noise_2d(c.shape, seed=seed + r, kmax=kmax, amplitude=amplitude)
            c.slab.copy_(torch.from_numpy(host))
            self._nonkept[c.n].value = int(self._has_nonkept(c, host))
        self._graph = None

    def run_state(self, r):
        """Host copies (u_x, u_y, T) of run r in the reference k-layout."""
        for c in self.classes:
            if r in c.runs:
                j = c.runs.index(r)
                return [c.slab[j, f].cpu().numpy() for f in range(3)]
        raise IndexError(r)

    def set_run_state(self, r, fields):
        for c in self.classes:
            if r in c.runs:
                j = c.runs.index(r)
                for f in range(3):
                    c.slab[j, f].copy_(torch.as_tensor(np.asarray(fields[f])))
                if self._has_nonkept(c, np.stack([np.asarray(x) for x in fields])[None]):
                    self._nonkept[c.n].value = 1
                self._graph = None
                return
        raise IndexError(r)

    @staticmethod
    def _has_nonkept(c, host):
        """Any non-zero entry outside the kept modes in host [run][field][kx][ky]?"""
        kx, ky = c.kshape
        M = c.plan.mx
        keep = np.zeros((kx, ky), dtype=bool)
        iy = np.arange(ky)
        keep[:M + 1, :] = ((iy <= c.plan.my) | (iy >= ky - c.plan.my))[None, :]
        return bool(np.any(host[..., ~keep] != 0))

    # ---------------------------------------------------------------- tables
    def _phi(self, c, coeff, h):
        key = (c.n, coeff, h)
        t = self._tables.get(key)
        if t is None:
            qmax = 2 * (c.n // 2) ** 2
            t = torch.empty((qmax + 1, 4), dtype=torch.float64, device=self.device)
            _lib.call("dd_phi_table", 2, float(coeff), self.vo, float(h), qmax, dptr(t),
                      ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
            self._tables[key] = t
        return t

    def _inv_k2(self, c):
        key = ('ik2', c.n)
        t = self._tables.get(key)
        if t is None:
            qmax = 2 * (c.n // 2) ** 2
            q = np.arange(qmax + 1, dtype=np.float64)
            q[0] = 1.
            t = torch.from_numpy(1.0 / q).to(self.device)
            self._tables[key] = t
        return t

    # ---------------------------------------------------------------- stepping
    def _issue_class(self, c, dt, stream):
        """Launch one RK2mid step of every run of class c on `stream`."""
        ik2 = self._inv_k2(c)
        coeffs = [self.nu, self.nu, self.kappa]
        th = [self._phi(c, cf, dt / 2.) for cf in coeffs]
        tf = [self._phi(c, cf, dt) for cf in coeffs]
        thp, _a = _lib.ptr_array([t.data_ptr() for t in th])
        tfp, _b = _lib.ptr_array([t.data_ptr() for t in tf])
        nus = (ctypes.c_double * 3)(*coeffs)
        st = ctypes.c_void_p(stream.cuda_stream)
        rs = 3 * c.fsize
        for j0 in range(0, c.nrun, c.chunk):
            nr = min(c.chunk, c.nrun - j0)
            ws = c.workspace(c.chunk)
            base = c.slab[j0]
            fp, _f = _lib.ptr_array([base[f].data_ptr() for f in range(3)])
            _lib.call("dd_rk2mid_step2d", c.plan.handle, c.phys, self.params, nr, fp, rs, dptr(ik2), thp, tfp,
                      nus, self.vo, float(dt), self.prec, ctypes.byref(self._nonkept[c.n]), dptr(ws), ws.numel(),
                      st)

    def _issue_step(self, dt):
        main = torch.cuda.current_stream()
        ev = torch.cuda.Event()
        ev.record(main)
        for ci in self.order:
            c = self.classes[ci]
            c.stream.wait_event(ev)
            with torch.cuda.stream(c.stream):
                self._issue_class(c, dt, c.stream)
        for ci in self.order:
            e = torch.cuda.Event()
            e.record(self.classes[ci].stream)
            main.wait_event(e)

    def _update_forms(self):
        """Per size class: the divergence form of the nonlinear terms when every
        run's velocity is solenoidal (dd_divergence_sums2d), else the curl form.
        The dynamics keep a solenoidal state solenoidal, so the choice holds
        until the state is set again (which drops the captured graph)."""
        buf = torch.empty(2, dtype=torch.float64, device=self.device)
        st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        for c in self.classes:
            base = c.slab[0]
            _lib.call("dd_divergence_sums2d", c.plan.handle, c.nrun, dptr(base[0]), dptr(base[1]), 3 * c.fsize,
                      dptr(buf), st)
            num, den = buf.tolist()
            tol = DIV_TOL2_FP32 if self.prec == _lib.DD_FP32 else DIV_TOL2
            c.phys = PHYS_BOUSS_DIV if self.nonlinear_form == 'auto' and num <= tol * den else PHYS_BOUSS

    nonlinear_form = 'auto'

    def step(self, dt, graph=True):
        """Advance every run by one RK2mid step (one graph replay when graph=True)."""
        if graph:
            if self._graph is None or self._graph_dt != dt:
                self.capture(dt)
            self._graph.replay()
        else:
            self._update_forms()
            self._issue_step(dt)
        self.time += dt
        self.iteration += 1

    def capture(self, dt):
        """Capture one ensemble step into a CUDA graph.  The schedule (chunks,
        order) and every table and workspace are prepared by an eager step on a
        scratch copy first, so nothing allocates or configures inside capture."""
        self._update_forms()
        saved = [c.slab.clone() for c in self.classes]
        self._issue_step(dt)                      # warm-up: tables, workspaces, kernel attributes
        torch.cuda.synchronize()
        for c, s in zip(self.classes, saved):
            c.slab.copy_(s)
        g = torch.cuda.CUDAGraph()
        cap = torch.cuda.Stream(device=self.device)
        cap.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(cap):
            with torch.cuda.graph(g, stream=cap):
                self._issue_step(dt)
        torch.cuda.current_stream().wait_stream(cap)
        torch.cuda.synchronize()
        self._graph, self._graph_dt = g, dt

    # ---------------------------------------------------------------- metrics
    def transforms_per_rhs(self, n):
        """Transforms per RHS of a run of size n: 5 + 3 (curl form) or 3 + 4
        (divergence form)."""
        c = next(c for c in self.classes if c.n == n)
        return 7 if c.phys == PHYS_BOUSS_DIV else 8

    def algorithmic_bytes_per_step(self, canonical=False):
        """Algorithmic bytes of one ensemble step: per run, 2 RHS x 8 (or 7)
        transforms x (one real + one complex 2D field pass) + 2 stages x 3 fields
        x 3 complex passes (B2(N) = 8 N^2 + 16 N (N/2 + 1)); the divergence
        form's stages read one more product field.  canonical: the curl form's
        count."""
        tot = 0
        for n in self.sizes:
            b2 = 8 * n * n + 16 * n * (n // 2 + 1)
            c2 = 16 * n * (n // 2 + 1)
            nt = 8 if canonical else self.transforms_per_rhs(n)
            tot += 2 * nt * b2 + 2 * 3 * 3 * c2 + (2 * c2 if nt == 7 else 0)
        return tot

    def grid_point_stages(self):
        return sum(2 * n * n for n in self.sizes)

    # ---------------------------------------------------------------- tuning
    def _time_schedule(self, dt, reps=3):
        self.capture(dt)
        saved = [c.slab.clone() for c in self.classes]
        self._graph.replay()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(reps):
            self._graph.replay()
        b.record()
        torch.cuda.synchronize()
        for c, s in zip(self.classes, saved):
            c.slab.copy_(s)
        return a.elapsed_time(b) / reps

    def autotune(self, dt, cache=None, chunks=(None, 128, 64, 32, 16), verbose=False):
        """Choose per class the y-pass tile schedule and the run chunking, and
        the class issue order, by timing graph replays; results are cached as
        JSON.  Returns the schedule."""
        cache = cache or _default_cache()
        gpu = torch.cuda.get_device_name(self.device)
        key = "%s|%s|%s|%s" % (gpu, self.precision, ",".join(str(c.n) for c in self.classes),
                               ",".join(str(c.nrun) for c in self.classes))
        db = {}
        if os.path.isfile(cache):
            try:
                db = json.load(open(cache))
            except (OSError, ValueError):
                db = {}
        if key in db:
            sched = db[key]
            for c, ch in zip(self.classes, sched["chunks"]):
                c.chunk = ch
            for c, ys in zip(self.classes, sched.get("ysched", [0] * len(self.classes))):
                c.set_ysched(ys)
            self.order = sched["order"]
            self._graph = None
            return sched
        # largest classes first, then refine each class's tile schedule and chunk in turn
        self.order = sorted(range(len(self.classes)), key=lambda i: -self.classes[i].n ** 2 * self.classes[i].nrun)
        best = self._time_schedule(dt)
        for c in self.classes:
            best_ys = c.ysched
            for ys in range(c.ysched_count()):
                if ys == best_ys:
                    continue
                c.set_ysched(ys)
                t = self._time_schedule(dt)
                if verbose:
                    print("class %d y tiles %d: %.3f ms" % (c.n, ys, t))
                if t < best:
                    best, best_ys = t, ys
            c.set_ysched(best_ys)
            best_ch = c.chunk
            for ch in chunks:
                cand = c.nrun if ch is None else min(ch, c.nrun)
                if cand == best_ch:
                    continue
                c.chunk = cand
                t = self._time_schedule(dt)
                if verbose:
                    print("class %d chunk %d: %.3f ms" % (c.n, cand, t))
                if t < best:
                    best, best_ch = t, cand
            c.chunk = best_ch
        rev = list(reversed(self.order))
        saved_order = self.order
        self.order = rev
        t = self._time_schedule(dt)
        if t >= best:
            self.order = saved_order
        else:
            best = t
        sched = {"chunks": [c.chunk for c in self.classes], "ysched": [c.ysched for c in self.classes],
                 "order": self.order, "ms_per_step": best,
                 "when": time.strftime("%Y-%m-%dT%H:%M:%S")}
        db[key] = sched
        try:
            os.makedirs(os.path.dirname(cache), exist_ok=True)
            with open(cache, "w") as f:
                json.dump(db, f, indent=1)
        except OSError:
            pass
        self._graph = None
        return sched
