"""Learned subgrid closure for a 64^3 LES of 3D incompressible hydro.

The LES right-hand side is the reference's IncompressibleHydro RHS
(dedalus/physics/physics.py:527-599) on the coarse grid plus -P[d_j tau_ij],
where the subgrid stress tau is predicted pointwise by an MLP
(10 -> 64 -> 64 -> 6, tanh) from the resolved velocity-gradient tensor and the
filter width.  The network runs on the tensor cores (BF16 weights and
activations, FP32 accumulation; csrc/mlp.cuh) and is trained on the GPU by the
library's own forward/backward and Adam kernels.

Training data come from the plain FP64 DNS: at a snapshot the DNS velocity is
filtered with a sharp spectral cut at the LES kept set (|k_i| <= 21 for 64^3,
the LES grid's 2/3 cutoff), and
    tau_ij = filt(u_i u_j) - filt(ubar_i ubar_j),   ubar = filt(u)
is sampled at the LES grid points together with the filtered gradients.  With a
sharp filter this tau is exactly the stress the LES misses: the LES computes
filt(ubar_i ubar_j) exactly (2/3 rule) and the filtered DNS evolves with
filt(u_i u_j).  (The pointwise form filt(u_i u_j) - ubar_i ubar_j has the same
kept modes but adds the unresolvable high-pass part of ubar_i ubar_j, which
would dominate the regression target.)

Everything on the data path is a C-ABI call (dd_les_products,
dd_les_truncate3, dd_les_gradients, dd_les_samples, dd_mlp_*); PyTorch holds
the buffers and shuffles the sample order.
"""
import concurrent.futures as cf
import ctypes
import json
import os
import time

import numpy as np
import torch

from . import _lib
from .engine import current_stream, dptr, get_plan

PAIRS = [(0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2)]
COMPONENTS = ["xx", "yy", "zz", "xy", "xz", "yz"]
DATA_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data")
DEFAULT_WEIGHTS = os.path.join(DATA_DIR, "les_closure_256to64.npz")


def _sizes():
    v = [ctypes.c_int() for _ in range(5)]
    _lib.call("dd_mlp_sizes", *[ctypes.byref(x) for x in v])
    return [x.value for x in v]


def _ptrs(ts):
    return _lib.ptr_array([t.data_ptr() for t in ts])


def init_params(seed=0):
    """Glorot-uniform weights on the used inputs (10) and outputs (6), zero
    biases; layout W1[64][16], b1[64], W2[64][64], b2[64], W3[8][64], b3[8]."""
    rng = np.random.Generator(np.random.PCG64(seed))
    W1, W2, W3 = np.zeros((64, 16)), np.zeros((64, 64)), np.zeros((8, 64))

    def glorot(fo, fi):
        a = np.sqrt(6.0 / (fi + fo))
        return rng.uniform(-a, a, size=(fo, fi))

    W1[:, :10] = glorot(64, 10)
    W2[:] = glorot(64, 64)
    W3[:6] = glorot(6, 64)
    return np.concatenate([W1.ravel(), np.zeros(64), W2.ravel(), np.zeros(64), W3.ravel(), np.zeros(8)]).astype(
        np.float32)


class MLPClosure:
    """Network state on the device: FP32 master parameters, their BF16 copy,
    Adam moments and the input/output normalisation."""

    def __init__(self, delta, seed=0, device=None):
        self.nparam, self.nbf16, self.nnorm, self.in_dim, self.out_dim = _sizes()
        self.device = torch.device('cuda', torch.cuda.current_device() if device is None else device)
        self.delta = float(delta)
        self.params = torch.from_numpy(init_params(seed)).to(self.device)
        self.wbf16 = torch.zeros(self.nbf16, dtype=torch.bfloat16, device=self.device)
        norm = np.zeros(self.nnorm, dtype=np.float32)
        norm[16:32] = 1.0
        norm[40:48] = 1.0
        self.norm = torch.from_numpy(norm).to(self.device)
        self.m = torch.zeros_like(self.params)
        self.v = torch.zeros_like(self.params)
        self.grad_buf = torch.zeros_like(self.params)
        self.loss_buf = torch.zeros(1, dtype=torch.float32, device=self.device)
        self.step = 0
        self.meta = {}
        # spectral band of the closure term: weight 0 below band[0], 1 above
        # band[1], linear between; (0, 0) applies it at every mode
        self.band = (0.0, 0.0)
        self.gain = 1.0                 # applied to the stress fluctuation (out_scale)
        # per-shell closure-term weights (entry i at |k| = i, linear between);
        # when set they replace the band
        self.shell_w = None
        self._ws = None
        self.pack()

    # ------------------------------------------------------------ plumbing
    def pack(self):
        _lib.call("dd_mlp_pack", dptr(self.params), dptr(self.wbf16), current_stream())

    def struct(self):
        """dd_closure for the C ABI (keep the returned object alive)."""
        sw = self.shell_w
        return _lib.Closure(self.wbf16.data_ptr(), self.params.data_ptr(), self.norm.data_ptr(), self.delta,
                            float(self.band[0]), float(self.band[1]), None if sw is None else sw.data_ptr(),
                            0 if sw is None else int(sw.numel()))

    def with_band(self, lo, hi, gain=1.0):
        """A view of this network (shared weights) with another closure-term
        band and the predicted stress fluctuation scaled by gain (the
        constant mean stress has no divergence)."""
        c = object.__new__(MLPClosure)
        c.__dict__.update(self.__dict__)
        c.band = (float(lo), float(hi))
        if gain != 1.0:
            c.norm = self.norm.clone()
            c.norm[40:46] *= float(gain)
        c.gain = float(gain) * self.gain
        return c

    def with_shells(self, weights):
        """A view of this network (shared weights) whose closure term is
        weighted per wavenumber shell: w(|k|) = weights linearly interpolated
        at |k| (entry i at |k| = i, the last entry beyond the table)."""
        w = np.asarray(weights, dtype=np.float64).reshape(-1)
        if w.size < 2:
            raise ValueError("the shell table needs at least two entries")
        c = object.__new__(MLPClosure)
        c.__dict__.update(self.__dict__)
        c.shell_w = torch.from_numpy(w.copy()).to(self.device)
        return c

    def set_norm(self, in_mean, in_scale, out_mean, out_scale):
        n = np.zeros(self.nnorm, dtype=np.float32)
        n[0:10], n[16:26] = in_mean[:10], in_scale[:10]
        n[16 + 10:32] = 1.0
        n[32:38], n[40:46] = out_mean[:6], out_scale[:6]
        n[38:40] = 0.0
        n[46:48] = 1.0
        self.norm.copy_(torch.from_numpy(n))

    def workspace(self, n):
        b = ctypes.c_size_t()
        _lib.call("dd_mlp_workspace_size", int(n), ctypes.byref(b))
        if self._ws is None or self._ws.numel() < b.value:
            self._ws = torch.empty(b.value, dtype=torch.uint8, device=self.device)
        return self._ws

    # ------------------------------------------------------------ compute
    def predict(self, X):
        """Y [n][8] FP32 for BF16 inputs X [n][16]."""
        Y = torch.empty((X.shape[0], self.out_dim), dtype=torch.float32, device=self.device)
        _lib.call("dd_mlp_infer", dptr(X), dptr(Y), int(X.shape[0]), dptr(self.wbf16), dptr(self.params),
                  current_stream())
        return Y

    def gradient(self, X, T, idx=None, n=None, n_total=None, idx_offset=0):
        """Loss gradient into self.grad_buf and the squared-error sum into
        self.loss_buf over n samples (rows idx[idx_offset:idx_offset+n])."""
        n = int(X.shape[0] if (n is None and idx is None) else (n if n is not None else idx.numel() - idx_offset))
        n_total = n if n_total is None else int(n_total)
        ws = self.workspace(n)
        ip = None if idx is None else ctypes.c_void_p(idx.data_ptr() + 8 * int(idx_offset))
        _lib.call("dd_mlp_grad", dptr(X), dptr(T), ip, n, n_total, dptr(self.wbf16), dptr(self.params),
                  dptr(self.grad_buf), dptr(self.loss_buf), dptr(ws), ws.numel(), current_stream())
        return self.grad_buf, self.loss_buf

    def adam(self, lr, beta1=0.9, beta2=0.999, eps=1e-8):
        self.step += 1
        _lib.call("dd_mlp_adam", dptr(self.params), dptr(self.grad_buf), dptr(self.m), dptr(self.v), self.step,
                  float(lr), float(beta1), float(beta2), float(eps), dptr(self.wbf16), current_stream())

    def mse(self, X, T, idx=None, chunk=1 << 22):
        """Mean squared (normalised) error over the samples (idx or all)."""
        n = X.shape[0] if idx is None else idx.numel()
        tot = 0.0
        for o in range(0, n, chunk):
            m = min(chunk, n - o)
            if idx is None:
                self.gradient(X[o:o + m], T[o:o + m])
            else:
                self.gradient(X, T, idx=idx, n=m, idx_offset=o)
            tot += float(self.loss_buf.item())
        return tot / (6.0 * n)

    # ------------------------------------------------------------ storage
    def save(self, path, **meta):
        meta = dict(self.meta, **meta)
        norm = self.norm.cpu().numpy().copy()
        norm[40:46] /= np.float32(self.gain)          # stored without the gain
        extra = {} if self.shell_w is None else {"shell_w": self.shell_w.cpu().numpy()}
        np.savez(path, params=self.params.cpu().numpy(), norm=norm, delta=np.float64(self.delta),
                 band=np.array(self.band, dtype=np.float64), gain=np.float64(self.gain),
                 meta=np.array(json.dumps(meta)), **extra)

    @classmethod
    def load(cls, path=DEFAULT_WEIGHTS, device=None):
        z = np.load(path)
        c = cls(float(z["delta"]), device=device)
        c.params.copy_(torch.from_numpy(z["params"].astype(np.float32)))
        c.norm.copy_(torch.from_numpy(z["norm"].astype(np.float32)))
        c.meta = json.loads(str(z["meta"]))
        if "band" in z.files:
            c.band = tuple(float(x) for x in z["band"])
        if "gain" in z.files and float(z["gain"]) != 1.0:
            c.gain = float(z["gain"])
            c.norm[40:46] *= c.gain
        if "shell_w" in z.files:
            c.shell_w = torch.from_numpy(z["shell_w"].astype(np.float64)).to(c.device)
        c.pack()
        return c


# ------------------------------------------------------------- training data
class FilteredSampler:
    """Samples (G, delta, tau) of DNS states filtered to an LES grid."""

    def __init__(self, dns_shape, les_shape, length=(2 * np.pi,) * 3):
        self.dns = get_plan(dns_shape, length)
        self.les = get_plan(les_shape, length)
        self.dns_shape, self.les_shape = tuple(dns_shape), tuple(les_shape)
        # sharp spectral cut at k_c = mx: filter width pi / k_c
        self.delta = float(length[0]) / (2.0 * self.les.mx)
        dev = self.dns.device
        kd, kl = tuple(self.dns.kshape), tuple(self.les.kshape)
        self._ux = [torch.empty(self.dns_shape, dtype=torch.float64, device=dev) for _ in range(3)]
        self._pr = [torch.empty(self.dns_shape, dtype=torch.float64, device=dev) for _ in range(6)]
        self._pk = [torch.empty(kd, dtype=torch.complex128, device=dev) for _ in range(6)]
        self._lk = [torch.empty(kl, dtype=torch.complex128, device=dev) for _ in range(9)]
        self._lx = [torch.empty(self.les_shape, dtype=torch.float64, device=dev) for _ in range(9)]
        self._g = [torch.empty(self.les_shape, dtype=torch.float64, device=dev) for _ in range(9)]
        self._rp = [torch.empty(self.les_shape, dtype=torch.float64, device=dev) for _ in range(6)]
        self._rk = [torch.empty(kl, dtype=torch.complex128, device=dev) for _ in range(6)]
        n = ctypes.c_size_t()
        _lib.call("dd_les_workspace_size", self.les.handle, _lib.DD_FP64, ctypes.byref(n))
        self._ws = torch.empty(n.value, dtype=torch.uint8, device=dev)

    @property
    def npts(self):
        return int(np.prod(self.les_shape))

    def filter_velocity(self, u_k):
        """LES-grid k arrays of the filtered DNS velocity (new tensors)."""
        out = [torch.empty(tuple(self.les.kshape), dtype=torch.complex128, device=self.les.device)
               for _ in range(3)]
        sp, _a = _ptrs(u_k)
        dp, _b = _ptrs(out)
        _lib.call("dd_les_truncate3", self.dns.handle, self.les.handle, 3, sp, dp, current_stream())
        return out

    def samples(self, u_k, raw, raw_band=None, band=None):
        """Fill raw [npts][16] FP32 with the samples of the DNS velocity u_k
        (3 full-layout k arrays on the DNS grid); with raw_band and band =
        (lo, hi), also the samples of the stress restricted to that spectral
        band (weight 0 below lo, 1 above hi, linear between)."""
        st = current_stream()
        self.dns.c2r(list(u_k), self._ux)
        up, _a = _ptrs(self._ux)
        pp, _b = _ptrs(self._pr)
        _lib.call("dd_les_products", int(np.prod(self.dns_shape)), up, pp, st)
        self.dns.r2c(self._pr, self._pk)
        sp, _c = _ptrs(list(u_k) + self._pk)
        dp, _d = _ptrs(self._lk)
        _lib.call("dd_les_truncate3", self.dns.handle, self.les.handle, 9, sp, dp, st)
        self.les.c2r(self._lk[:3], self._lx[:3])
        self.les.c2r(self._lk[3:], self._lx[3:])
        # filt(ubar_a ubar_b): resolved products, cut at the same kept set
        ubp, _h = _ptrs(self._lx[:3])
        rpp, _i = _ptrs(self._rp)
        _lib.call("dd_les_products", self.npts, ubp, rpp, st)
        self.les.r2c(self._rp, self._rk)
        self.les.c2r(self._rk, self._rp)
        kp, _e = _ptrs(self._lk[:3])
        gp, _f = _ptrs(self._g)
        _lib.call("dd_les_gradients", self.les.handle, kp, gp, _lib.DD_FP64, dptr(self._ws), self._ws.numel(), st)
        fp, _g = _ptrs(self._lx[3:])
        _lib.call("dd_les_samples", self.npts, gp, fp, rpp, self.delta, dptr(raw), st)
        if raw_band is not None:
            tau = [a - b for a, b in zip(self._lx[3:], self._rp)]
            self.les.r2c(tau, self._rk)
            kp2, _j = _ptrs(self._rk)
            _lib.call("dd_les_band", self.les.handle, 6, kp2, float(band[0]), float(band[1]), st)
            self.les.c2r(self._rk, tau)
            zero = [torch.zeros_like(tau[0])] * 6
            tp, _k = _ptrs(tau)
            zp, _l = _ptrs(zero)
            _lib.call("dd_les_samples", self.npts, gp, tp, zp, self.delta, dptr(raw_band), st)

    def transfer(self, u_k, closures, nbins):
        """Per-shell subgrid energy transfer (dd_les_transfer) at the filtered
        DNS state u_k: the exact one, from tau = filt(u u) - filt(ub ub), and
        that of the stress each closure predicts from the filtered velocity
        (its band and shell weights are not applied).  Returns (exact [nbins],
        {name: [nbins]}) as host float64 arrays."""
        if getattr(self, '_raw1', None) is None:
            self._raw1 = torch.empty((self.npts, 16), dtype=torch.float32, device=self.les.device)
            self._tau = [torch.empty(self.les_shape, dtype=torch.float64, device=self.les.device) for _ in range(6)]
        st = current_stream()
        self.samples(u_k, self._raw1)
        for c in range(6):
            torch.sub(self._lx[3 + c], self._rp[c], out=self._tau[c])
        up, _a = _ptrs(self._lk[:3])
        tp, _b = _ptrs(self._tau)
        out = torch.empty(nbins, dtype=torch.float64, device=self.les.device)
        _lib.call("dd_les_transfer", self.les.handle, up, tp, int(nbins), dptr(out), dptr(self._ws),
                  self._ws.numel(), st)
        exact = out.cpu().numpy().copy()
        models = {}
        for name, cl in closures.items():
            s = cl.struct()
            _lib.call("dd_les_stress", self.les.handle, up, tp, ctypes.byref(s), _lib.DD_FP64, dptr(self._ws),
                      self._ws.numel(), st)
            _lib.call("dd_les_transfer", self.les.handle, up, tp, int(nbins), dptr(out), dptr(self._ws),
                      self._ws.numel(), st)
            models[name] = out.cpu().numpy().copy()
        return exact, models


def generate_dataset(n_seeds=50, n_snap=20, stride=50, dns_n=256, les_n=64, nu=5e-3, dt=2e-3, seed0=1000,
                     log=None, band=None):
    """Run the FP64 DNS (RK4, nu, dt) from n_seeds random turbulent states
    (turbulence_3d, unit energy) and sample n_snap filtered snapshots per seed,
    one every `stride` steps.  Returns (raw [n][16] FP32 device tensor, seed of
    each snapshot, info); with band = (lo, hi) the info dict also holds
    "raw_band", the samples of the band-restricted stress."""
    from . import mods
    from .init_cond import turbulence_3d
    shape = (dns_n,) * 3
    sampler = FilteredSampler(shape, (les_n,) * 3)
    npts = sampler.npts
    raw = torch.empty((n_seeds * n_snap * npts, 16), dtype=torch.float32, device=sampler.les.device)
    raw_band = torch.empty_like(raw) if band is not None else None
    RHS = mods.IncompressibleHydro(shape, mods.FourierRepresentation)
    RHS.parameters['nu'] = nu
    data = RHS.create_fields(0.)
    ti = mods.RK4(RHS)
    seeds = []
    t0 = time.time()
    steps = 0
    # the next seed's initial state is drawn on a host thread while the DNS runs
    pool = cf.ThreadPoolExecutor(max_workers=1)
    nxt = pool.submit(turbulence_3d, shape, seed=seed0)
    for s in range(n_seeds):
        u0 = nxt.result()
        if s + 1 < n_seeds:
            nxt = pool.submit(turbulence_3d, shape, seed=seed0 + s + 1)
        for i in range(3):
            data['u'][i]['kspace'] = u0[i]
        data.set_time(0.)
        for j in range(n_snap):
            for _ in range(stride):
                ti.do_advance(data, dt)
                steps += 1
            k = (s * n_snap + j) * npts
            sampler.samples([data['u'][i].kdata for i in range(3)], raw[k:k + npts],
                            None if raw_band is None else raw_band[k:k + npts], band)
            seeds.append(seed0 + s)
        if log:
            torch.cuda.synchronize()
            log("seed %d done: %d DNS steps, %.1f s" % (seed0 + s, steps, time.time() - t0))
    pool.shutdown()
    torch.cuda.synchronize()
    info = {"n_seeds": n_seeds, "n_snap": n_snap, "stride": stride, "dns_n": dns_n, "les_n": les_n, "nu": nu,
            "dt": dt, "seed0": seed0, "dns_steps": steps, "seconds": time.time() - t0, "delta": sampler.delta}
    if raw_band is not None:
        info["band"] = list(band)
        info["raw_band"] = raw_band
    return raw, np.array(seeds), info


def shell_count(les_n):
    """Bins of round(|k|) over the kept modes of an les_n^3 grid (2 pi box)."""
    m = int(np.ceil(les_n / 3.0)) - 1
    return int(np.floor(np.sqrt(3.0) * m + 0.5)) + 1


def calibrate_shells(closure, n_seeds=4, n_snap=20, stride=50, dns_n=256, les_n=64, nu=5e-3, dt=2e-3, seed0=1000,
                     wmax=8.0, log=None):
    """Per-shell closure-term weights that make the network's mean subgrid
    energy transfer equal the exact one over filtered DNS snapshots (the FP64
    DNS of generate_dataset, seeds seed0 .. seed0 + n_seeds - 1):
    w(k) = sum T_exact(k) / sum T_model(k) over the snapshots, 0 where the
    model transfers nothing, clipped to [-wmax, wmax]; w(0) = w(1) (the mean
    mode carries no force).  Returns (w, {"exact": sums, "model": sums})."""
    from . import mods
    from .init_cond import turbulence_3d
    shape = (dns_n,) * 3
    sampler = FilteredSampler(shape, (les_n,) * 3)
    nb = shell_count(les_n)
    RHS = mods.IncompressibleHydro(shape, mods.FourierRepresentation)
    RHS.parameters['nu'] = nu
    data = RHS.create_fields(0.)
    ti = mods.RK4(RHS)
    se = np.zeros(nb)
    sm = np.zeros(nb)
    t0 = time.time()
    for s in range(n_seeds):
        u0 = turbulence_3d(shape, seed=seed0 + s)
        for i in range(3):
            data['u'][i]['kspace'] = u0[i]
        data.set_time(0.)
        for j in range(n_snap):
            for _ in range(stride):
                ti.do_advance(data, dt)
            e, m = sampler.transfer([data['u'][i].kdata for i in range(3)], {"m": closure}, nb)
            se += e
            sm += m["m"]
        if log:
            log("calibration seed %d done, %.1f s" % (seed0 + s, time.time() - t0))
    tiny = 1e-6 * np.max(np.abs(sm))
    w = np.where(np.abs(sm) > tiny, se / np.where(np.abs(sm) > tiny, sm, 1.0), 0.0)
    w = np.clip(w, -wmax, wmax)
    w[0] = w[1]
    return w, {"exact": se.tolist(), "model": sm.tolist(), "seconds": time.time() - t0,
               "snapshots": n_seeds * n_snap, "seed0": seed0}


def fit_norm(raw, chunk=1 << 24):
    """Per-column mean and standard deviation (FP64 accumulation)."""
    n = raw.shape[0]
    s = torch.zeros(16, dtype=torch.float64, device=raw.device)
    s2 = torch.zeros(16, dtype=torch.float64, device=raw.device)
    for o in range(0, n, chunk):
        r = raw[o:o + chunk].to(torch.float64)
        s += r.sum(0)
        s2 += (r * r).sum(0)
    mean = (s / n).cpu().numpy()
    var = np.maximum((s2 / n).cpu().numpy() - mean ** 2, 0.0)
    std = np.sqrt(var)
    in_scale = np.where(std[:10] > 0, 1.0 / np.where(std[:10] > 0, std[:10], 1.0), 1.0)
    in_mean = mean[:10].copy()
    if std[9] == 0:            # constant filter width: a unit input
        in_mean[9], in_scale[9] = 0.0, 1.0 / mean[9] if mean[9] else 1.0
    out_scale = np.where(std[10:] > 0, std[10:], 1.0)
    return in_mean, in_scale, mean[10:], out_scale


def normalise(closure, raw):
    """BF16 inputs X [n][16] and FP32 targets T [n][8] of raw samples."""
    n = raw.shape[0]
    X = torch.empty((n, 16), dtype=torch.bfloat16, device=raw.device)
    T = torch.empty((n, 8), dtype=torch.float32, device=raw.device)
    _lib.call("dd_mlp_normalize", dptr(raw), n, dptr(closure.norm), dptr(X), dptr(T), current_stream())
    return X, T


def train(closure, X, T, train_idx, val_idx=None, epochs=4, batch=65536, lr=2e-3, lr_min=2e-5, seed=0, log=None):
    """Adam on minibatches of a fresh random permutation each epoch, cosine
    learning-rate decay; returns the history of (epoch, train mse, val mse)."""
    gen = torch.Generator(device=X.device)
    gen.manual_seed(seed)
    n = train_idx.numel()
    nb = n // batch
    total = epochs * nb
    hist = []
    k = 0
    t0 = time.time()
    for ep in range(epochs):
        perm = train_idx[torch.randperm(n, generator=gen, device=X.device)]
        acc = torch.zeros(1, dtype=torch.float64, device=X.device)
        for b in range(nb):
            f = k / max(total - 1, 1)
            cur = lr_min + 0.5 * (lr - lr_min) * (1.0 + np.cos(np.pi * f))
            closure.gradient(X, T, idx=perm, n=batch, idx_offset=b * batch)
            acc += closure.loss_buf
            closure.adam(cur)
            k += 1
        tr = float(acc.item()) / (6.0 * nb * batch)
        va = closure.mse(X, T, val_idx) if val_idx is not None else float('nan')
        hist.append((ep, tr, va))
        if log:
            log("epoch %d: train mse %.5f  val mse %.5f  (%.1f s)" % (ep, tr, va, time.time() - t0))
    return hist


def correlation(closure, X, T, idx, chunk=1 << 22):
    """Per-component correlation between predicted and true normalised stress."""
    n = idx.numel()
    s = torch.zeros((5, 6), dtype=torch.float64, device=X.device)
    for o in range(0, n, chunk):
        ii = idx[o:o + chunk]
        y = closure.predict(X[ii])[:, :6].to(torch.float64)
        t = T[ii][:, :6].to(torch.float64)
        s += torch.stack([y.sum(0), t.sum(0), (y * y).sum(0), (t * t).sum(0), (y * t).sum(0)])
    s = s.cpu().numpy() / n
    cov = s[4] - s[0] * s[1]
    return cov / np.sqrt((s[2] - s[0] ** 2) * (s[3] - s[1] ** 2))


# ------------------------------------------------------------------ runs
def les_problem(les_n=64, nu=5e-3, closure=None, precision='fp32'):
    """(physics, data, RK4 integrator) for a closed (or unclosed) LES; the LES
    transforms run in FP32 by default (state and stage updates FP64)."""
    from . import mods
    RHS = mods.LESHydro((les_n,) * 3, mods.FourierRepresentation, closure=closure, precision=precision)
    RHS.parameters['nu'] = nu
    data = RHS.create_fields(0.)
    return RHS, data, mods.RK4(RHS)


def compare_spectra(kc, e_ref, e, kcut):
    """max over the spectrum bins centred at 0 < k <= kcut (kc: bin centres)
    of |e - e_ref| / e_ref."""
    kc, e_ref, e = np.asarray(kc), np.asarray(e_ref), np.asarray(e)
    sel = (kc > 0) & (kc <= kcut) & (e_ref > 0)
    return float(np.max(np.abs(e[sel] - e_ref[sel]) / e_ref[sel]))


def sgs_dissipation(closure, data, precision='fp32'):
    """-<tau_ij S_ij>: the mean energy drain of the closure for the LES state
    (S the resolved strain rate), the closure's share of the dissipation."""
    comps = [data['u'][i] for i in range(3)]
    for c in comps:
        c.require_space('kspace')
    plan = comps[0].plan
    prec = _lib.DD_FP32 if precision == 'fp32' else _lib.DD_FP64
    n = ctypes.c_size_t()
    _lib.call("dd_les_workspace_size", plan.handle, prec, ctypes.byref(n))
    ws = plan.workspace(n.value, tag='les_diag')
    shape = tuple(plan.xshape)
    g = [torch.empty(shape, dtype=torch.float64, device=plan.device) for _ in range(9)]
    tau = [torch.empty(shape, dtype=torch.float64, device=plan.device) for _ in range(6)]
    up, _a = _ptrs([c.kdata for c in comps])
    gp, _b = _ptrs(g)
    tp, _c = _ptrs(tau)
    _lib.call("dd_les_gradients", plan.handle, up, gp, prec, dptr(ws), ws.numel(), current_stream())
    cl = closure.struct()
    _lib.call("dd_les_stress", plan.handle, up, tp, ctypes.byref(cl), prec, dptr(ws), ws.numel(), current_stream())
    tot = torch.zeros((), dtype=torch.float64, device=plan.device)
    for c, (a, b) in enumerate(PAIRS):
        s_ab = 0.5 * (g[3 * a + b] + g[3 * b + a])
        tot += (1.0 if a == b else 2.0) * (tau[c] * s_ab).mean()
    return -float(tot.item())


def evaluate(models, seed=7, dns_n=256, les_n=64, nu=5e-3, dt=2e-3, nsteps=1000, every=100, log=None,
             precision='fp32'):
    """Run the FP64 DNS and LES runs from the same filtered initial state for
    nsteps, comparing every `every` steps each LES's spectrum, energy and
    dissipation with those of the DNS.  models: {name: MLPClosure or None}
    (an MLPClosure alone means {"closure": it, "no_model": None}).  E(k)
    errors are max over bins 1 <= k <= kmax/2 ("err_half") and kmax
    ("err_full") of |E_les - E_dns| / E_dns, E_dns the filtered DNS spectrum;
    dissipation: DNS total vs LES resolved + closure (sgs) drain."""
    from . import mods, diagnostics as D
    from .init_cond import turbulence_3d
    if not isinstance(models, dict):
        models = {"closure": models, "no_model": None}
    shape = (dns_n,) * 3
    sampler = FilteredSampler(shape, (les_n,) * 3)
    dns = mods.IncompressibleHydro(shape, mods.FourierRepresentation)
    dns.parameters['nu'] = nu
    dd = dns.create_fields(0.)
    ti = mods.RK4(dns)
    u0 = turbulence_3d(shape, seed=seed)
    for i in range(3):
        dd['u'][i]['kspace'] = u0[i]
    runs = {}
    for name, cl in models.items():
        RHS, data, ti_l = les_problem(les_n, nu, cl, precision)
        ub = sampler.filter_velocity([dd['u'][i].kdata for i in range(3)])
        for i in range(3):
            data['u'][i].kdata.copy_(ub[i])
            data['u'][i].touch()
        runs[name] = (RHS, data, ti_l, cl)
    ref = les_problem(les_n, nu, None)
    kmax = sampler.les.mx
    out = {"steps": [], "dns_diss": [], "dns_diss_filtered": [], "dns_E": [], "dns_ekin_filtered": []}
    for name in runs:
        out[name] = {"diss": [], "diss_sgs": [], "ekin": [], "E": [], "err_half": [], "err_full": []}
    t_dns = t_les = 0.0

    def record(step):
        ub = sampler.filter_velocity([dd['u'][i].kdata for i in range(3)])
        for i in range(3):
            ref[1]['u'][i].kdata.copy_(ub[i])
            ref[1]['u'][i]._curr_space = 'kspace'
            ref[1]['u'][i].data = ref[1]['u'][i].kdata
        kc, e_ref = D.power_spectrum(ref[1]['u'])
        out["steps"].append(step)
        out["dns_E"].append(e_ref.tolist())
        out["dns_diss"].append(D.energy_dissipation(dd, nu))
        out["dns_diss_filtered"].append(D.energy_dissipation(ref[1], nu))
        out["dns_ekin_filtered"].append(D.ekin(ref[1]))
        for name, (RHS, data, _t, cl) in runs.items():
            _, e = D.power_spectrum(data['u'])
            r = out[name]
            r["E"].append(e.tolist())
            r["diss"].append(D.energy_dissipation(data, nu))
            r["diss_sgs"].append(sgs_dissipation(cl, data, precision) if cl is not None else 0.0)
            r["ekin"].append(D.ekin(data))
            r["err_half"].append(compare_spectra(kc, e_ref, e, kmax / 2.0))
            r["err_full"].append(compare_spectra(kc, e_ref, e, kmax))

    record(0)
    for step in range(1, nsteps + 1):
        torch.cuda.synchronize()
        a = time.time()
        ti.do_advance(dd, dt)
        torch.cuda.synchronize()
        b = time.time()
        for name, (RHS, data, ti_l, _c) in runs.items():
            ti_l.do_advance(data, dt)
        torch.cuda.synchronize()
        c = time.time()
        t_dns += b - a
        t_les += (c - b) / len(runs)
        if step % every == 0:
            record(step)
            if log:
                log("step %d: E(k<=kmax/2) err %s" % (step, "  ".join(
                    "%s %.4f" % (n, out[n]["err_half"][-1]) for n in runs)))
    out["dns_steps_per_s"] = nsteps / t_dns
    out["les_steps_per_s_incl_host"] = nsteps / t_les
    out["kmax"] = kmax
    out["models"] = list(runs)
    return out


# ------------------------------------------------- a-posteriori weight fit
def dns_reference(seed, dns_n=256, les_n=64, nu=5e-3, dt=2e-3, nsteps=1000, every=100, sampler=None,
                  full_spectrum=False):
    """One plain FP64 DNS trajectory as the judge of an LES: the filtered
    initial state on the LES grid (device k arrays) and, every `every` steps,
    the filtered-DNS spectrum E(k) and the DNS dissipation rate
    2 nu <|curl u|^2> / 2 (volume_average.py:254-265); with full_spectrum,
    also the DNS's own spectrum on its grid ("E_dns", bin centres "kc_dns")."""
    from . import mods, diagnostics as D
    from .init_cond import turbulence_3d
    shape = (dns_n,) * 3
    sampler = sampler or FilteredSampler(shape, (les_n,) * 3)
    dns = mods.IncompressibleHydro(shape, mods.FourierRepresentation)
    dns.parameters['nu'] = nu
    dd = dns.create_fields(0.)
    u0 = turbulence_3d(shape, seed=seed)
    for i in range(3):
        dd['u'][i]['kspace'] = u0[i]
    ti = mods.RK4(dns)
    _rhs, probe, _t = les_problem(les_n, nu, None)
    ref = {"seed": seed, "nu": nu, "dt": dt, "every": every, "les_n": les_n, "steps": [], "E": [], "Es": [],
           "diss": [],
           "u0": [c.clone() for c in sampler.filter_velocity([dd['u'][i].kdata for i in range(3)])]}
    t0 = time.time()
    for step in range(0, nsteps + 1):
        if step:
            ti.do_advance(dd, dt)
        if step % every == 0:
            ub = sampler.filter_velocity([dd['u'][i].kdata for i in range(3)])
            for i in range(3):
                probe['u'][i].kdata.copy_(ub[i])
                probe['u'][i]._curr_space = 'kspace'
                probe['u'][i].data = probe['u'][i].kdata
            kc, e = D.power_spectrum(probe['u'])
            ks, es = D.power_spectrum(probe['u'], shells=True)
            ref["kc"], ref["ks"] = np.asarray(kc), np.asarray(ks)
            ref["steps"].append(step)
            ref["E"].append(np.asarray(e))
            ref["Es"].append(np.asarray(es))
            ref["diss"].append(D.energy_dissipation(dd, nu))
            if full_spectrum:
                kd, ed = D.power_spectrum(dd['u'])
                ref["kc_dns"] = np.asarray(kd)
                ref.setdefault("E_dns", []).append(np.asarray(ed))
    torch.cuda.synchronize()
    ref["seconds"] = time.time() - t0
    ref["kmax"] = sampler.les.mx
    return ref


def _closure_energy_rate(RHS, data, d_with, d_without):
    """Energy the closure term feeds into the LES state per unit time:
    sum over modes of Re(conj(u) . F), F = RHS with the closure minus RHS
    without it (Hermitian weight 2 for kx > 0), in the normalisation of
    ekin.  Negative for a draining closure."""
    cl = RHS.closure
    RHS.RHS(data, d_with)
    RHS.closure = None
    try:
        RHS.RHS(data, d_without)
    finally:
        RHS.closure = cl
    tot = 0.0
    for i in range(3):
        u = data['u'][i].kdata
        f = d_with['u'][i].kdata - d_without['u'][i].kdata
        p = (u.conj() * f).real
        tot += float(2.0 * p.sum() - p[..., 0].sum())
    return tot


def les_trajectory(closure, ref, precision='fp32'):
    """Run the 64^3 LES (closure or None) from the reference's filtered
    initial state over its steps.  At each of its record steps: the E(k)
    error against the filtered DNS, max over the reference's spectrum bins
    (PowerSpectrum, analysis_set.py:778-815) centred at k <= kmax/2
    ("err_half") and k <= kmax ("err_full"), and over unit shells
    k = 1 .. kmax/2 ("err_half_shells"); and the LES energy-loss rate
    (resolved viscous dissipation minus the closure term's energy input)
    relative to the DNS dissipation rate ("diss_err", (LES - DNS) / DNS)."""
    from . import diagnostics as D
    nu, dt, every = ref["nu"], ref["dt"], ref["every"]
    les_n = ref["les_n"]
    RHS, data, ti = les_problem(les_n, nu, closure, precision)
    for i in range(3):
        data['u'][i].kdata.copy_(ref["u0"][i])
        data['u'][i].touch()
    out = {"steps": [], "err_half": [], "err_full": [], "err_half_shells": [], "diss_err": [], "diss": [],
           "closure_input": []}
    d1 = RHS.create_fields(0.) if closure is not None else None
    d2 = RHS.create_fields(0.) if closure is not None else None
    kmax = ref["kmax"]
    nsteps = ref["steps"][-1]
    for step in range(0, nsteps + 1):
        if step:
            ti.do_advance(data, dt)
        if step % every == 0:
            r = ref["steps"].index(step)
            _, e = D.power_spectrum(data['u'])
            _, es = D.power_spectrum(data['u'], shells=True)
            diss = D.energy_dissipation(data, nu)
            inp = _closure_energy_rate(RHS, data, d1, d2) if closure is not None else 0.0
            out["steps"].append(step)
            out["err_half"].append(compare_spectra(ref["kc"], ref["E"][r], e, kmax / 2.0))
            out["err_full"].append(compare_spectra(ref["kc"], ref["E"][r], e, kmax))
            out["err_half_shells"].append(compare_spectra(ref["ks"], ref["Es"][r], es, kmax / 2.0))
            out["diss"].append(diss)
            out["closure_input"].append(inp)
            out["diss_err"].append((diss - inp - ref["diss"][r]) / ref["diss"][r])
    return out


def shell_table(knots, values, les_n=64):
    """Closure-term weights per integer |k| (the dd_closure shell table):
    piecewise linear through (knots, values), constant beyond either end."""
    kk = np.arange(shell_count(les_n), dtype=np.float64)
    return np.interp(kk, np.asarray(knots, dtype=np.float64), np.asarray(values, dtype=np.float64))


def posteriori_score(trajs):
    """max over runs of the largest of: the max over time of the E(k <= kmax/2)
    error in the reference's bins and in unit shells, and the max over time
    (after the start) of |dissipation error|."""
    s = 0.0
    for t in trajs:
        s = max(s, max(t["err_half"]), max(t["err_half_shells"]), max(abs(x) for x in t["diss_err"][1:]))
    return s


def fit_posteriori(closure, refs, knots, x0, max_evals=300, log=None, precision='fp32'):
    """Fit the closure-term weight table a posteriori: the weights at the
    knots (piecewise linear in |k|) that minimise posteriori_score of the
    LES runs against the DNS references refs (training seeds), by the
    Nelder-Mead simplex (scipy.optimize).  Returns (weights at the knots,
    info)."""
    from scipy.optimize import minimize
    hist = []

    def obj(x):
        cl = closure.with_shells(shell_table(knots, x))
        trajs = [les_trajectory(cl, r, precision) for r in refs]
        sc = posteriori_score(trajs)
        hist.append({"x": [float(v) for v in x], "score": sc,
                     "err_half": [max(t["err_half"]) for t in trajs],
                     "err_half_shells": [max(t["err_half_shells"]) for t in trajs],
                     "diss_err": [max(abs(v) for v in t["diss_err"][1:]) for t in trajs]})
        if log and len(hist) % 10 == 0:
            best = min(hist, key=lambda h: h["score"])
            log("fit eval %d: score %.4f (best %.4f at %s)" % (len(hist), sc, best["score"],
                                                                 np.round(best["x"], 3).tolist()))
        return sc

    x0 = np.asarray(x0, dtype=np.float64)
    simplex = [x0] + [x0 + np.eye(len(x0))[i] * max(0.25, 0.3 * abs(x0[i])) for i in range(len(x0))]
    t0 = time.time()
    res = minimize(obj, x0, method='Nelder-Mead',
                   options={"maxfev": max_evals, "xatol": 1e-3, "fatol": 1e-4, "initial_simplex": np.array(simplex)})
    best = min(hist, key=lambda h: h["score"])
    return np.asarray(best["x"]), {"evals": len(hist), "seconds": time.time() - t0, "best": best,
                                   "start": hist[0], "knots": list(knots), "message": str(res.message)}
