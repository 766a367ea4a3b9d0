"""CPU oracle -- test infrastructure only.

The learned subgrid closure has no counterpart in the reference; this module
restates, in numpy, what the CUDA closure computes, so that the kernels can be
checked on small cases:

* the MLP 10 -> 64 -> 64 -> 6 (tanh) with the kernels' BF16 rounding points
  (inputs, weights, hidden activations and backward signals rounded to BF16,
  everything else FP64 here) and, with ``rounding=False``, the exact FP64
  network whose analytic gradient ``grad`` is pinned by central finite
  differences in the tests;
* the filtered-DNS training samples: products u_i u_j on the DNS grid, the
  sharp spectral truncation to the LES kept modes, and
  tau_ij = filt(u_i u_j) - filt(ubar_i ubar_j), ubar = filt(u), at the LES
  grid points;
* the closure term -P[d_j tau_ij] of the LES right-hand side, with the k-space
  layout of the reference's Fourier representation (3D k arrays
  [ky][kz][kx], dedalus/data_objects/representations.py:86-93, 173-176).

Parameter layout (FP32 vector): W1[64][16], b1[64], W2[64][64], b2[64],
W3[8][64], b3[8].  Normalisation vector: in_mean[16], in_scale[16],
out_mean[8], out_scale[8]; stress component order xx, yy, zz, xy, xz, yz.
"""
import numpy as np

NIN, NH, NOUT, IN_PAD, OUT_PAD = 10, 64, 6, 16, 8
SHAPES = [("W1", (NH, IN_PAD)), ("b1", (NH,)), ("W2", (NH, NH)), ("b2", (NH,)), ("W3", (OUT_PAD, NH)),
          ("b3", (OUT_PAD,))]
NPARAM = sum(int(np.prod(s)) for _, s in SHAPES)
PAIRS = [(0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2)]


def unpack(p):
    out, o = {}, 0
    for name, s in SHAPES:
        n = int(np.prod(s))
        out[name] = np.asarray(p[o:o + n]).reshape(s)
        o += n
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], dtype=np.float64).ravel() for name, _ in SHAPES])


def bf16(x):
    """Round to the nearest BF16 (ties to even) through FP32, as
    __float2bfloat16_rn does on an FP32 value; returns float64."""
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float64).astype(np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32).astype(np.float64)


def _r(x, rounding):
    return bf16(x) if rounding else np.asarray(x, dtype=np.float64)


def forward(p, X, rounding=True):
    """Y [n][8] and the activations (H1, H2) for inputs X [n][16]."""
    w = unpack(np.asarray(p, dtype=np.float64))
    W1, W2, W3 = (_r(w[k], rounding) for k in ("W1", "W2", "W3"))
    X = _r(X, rounding)
    H1 = _r(np.tanh(X @ W1.T + w["b1"]), rounding)
    H2 = _r(np.tanh(H1 @ W2.T + w["b2"]), rounding)
    Y = H2 @ W3.T + w["b3"]
    return Y, (X, H1, H2, W1, W2, W3)


def loss(p, X, T, n_total=None, rounding=True):
    Y, _ = forward(p, X, rounding)
    n_total = len(X) if n_total is None else n_total
    e = Y[:, :NOUT] - np.asarray(T, dtype=np.float64)[:, :NOUT]
    return float(np.sum(e * e)) / (n_total * NOUT), float(np.sum(e * e))


def grad(p, X, T, n_total=None, rounding=True):
    """Gradient of loss() (FP64 parameter vector) and the squared-error sum."""
    Y, (Xr, H1, H2, W1, W2, W3) = forward(p, X, rounding)
    n_total = len(X) if n_total is None else n_total
    e = Y[:, :NOUT] - np.asarray(T, dtype=np.float64)[:, :NOUT]
    if rounding:
        scale = float(np.float32(2.0) / (np.float32(n_total) * np.float32(NOUT)))
    else:
        scale = 2.0 / (n_total * NOUT)
    dYf = np.zeros_like(Y)
    dYf[:, :NOUT] = scale * e
    dY = _r(dYf, rounding)
    dH2 = _r((dY @ W3) * (1.0 - H2 * H2), rounding)
    dH1 = _r((dH2 @ W2) * (1.0 - H1 * H1), rounding)
    g = {"W3": dY.T @ H2, "b3": dYf.sum(0), "W2": dH2.T @ H1, "b2": dH2.sum(0), "W1": dH1.T @ Xr, "b1": dH1.sum(0)}
    return pack(g), float(np.sum(e * e))


def init_params(seed=0):
    """Glorot-uniform weights over the used inputs/outputs, zero biases (the
    same draw as the package's initialiser)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    d = {name: np.zeros(s) for name, s in SHAPES}

    def glorot(fo, fi):
        a = np.sqrt(6.0 / (fi + fo))
        return rng.uniform(-a, a, size=(fo, fi))

    d["W1"][:, :NIN] = glorot(NH, NIN)
    d["W2"][:] = glorot(NH, NH)
    d["W3"][:NOUT] = glorot(NOUT, NH)
    return pack(d).astype(np.float32)


# ------------------------------------------------------------ grids / fields
def _k1(n):
    return np.fft.fftfreq(n, 1.0 / n)


def kvectors(shape):
    """(kx, ky, kz) broadcast over the 3D k layout [ky][kz][kx] of an
    x-space shape (Nz, Ny, Nx) on a 2 pi box."""
    nz, ny, nx = shape
    kx = np.arange(nx // 2 + 1, dtype=np.float64)
    ky, kz = _k1(ny), _k1(nz)
    ky[ny // 2] = -abs(ky[ny // 2])
    kz[nz // 2] = -abs(kz[nz // 2])
    return kx[None, None, :], ky[:, None, None], kz[None, :, None]


def kept_mask(shape):
    """2/3 kept set |m_i| <= ceil(N_i/3) - 1 on the k layout."""
    nz, ny, nx = shape
    mx, my, mz = (int(np.ceil(n / 3.0)) - 1 for n in (nx, ny, nz))
    kx, ky, kz = kvectors(shape)
    return (np.abs(kx) <= mx) & (np.abs(ky) <= my) & (np.abs(kz) <= mz)


def to_x(k, shape):
    """Grid-point values of one k array (kept modes; unnormalised inverse)."""
    return np.fft.irfftn(np.transpose(k, (1, 0, 2)), s=shape, axes=(0, 1, 2)) * np.prod(shape)


def to_k(x):
    """k array (reference layout, /N) of grid-point values, 2/3 dealiased."""
    shape = x.shape
    return np.transpose(np.fft.rfftn(x) / np.prod(shape), (1, 0, 2)) * kept_mask(shape)


def truncate(k, src_shape, dst_shape):
    """Sharp spectral filter: the dst-kept modes of a src k array, in dst layout."""
    kxs, kys, kzs = kvectors(src_shape)
    kxd, kyd, kzd = kvectors(dst_shape)
    out = np.zeros((dst_shape[1], dst_shape[0], dst_shape[2] // 2 + 1), dtype=np.complex128)
    keep = kept_mask(dst_shape)
    iy = np.array([int(v) % src_shape[1] for v in kyd.ravel()])
    iz = np.array([int(v) % src_shape[0] for v in kzd.ravel()])
    sub = k[np.ix_(iy, iz, np.arange(dst_shape[2] // 2 + 1))]
    out[keep] = sub[keep]
    return out


def gradients(u, shape):
    """G[3 a + j] = d_j u_a at the grid points."""
    kx, ky, kz = kvectors(shape)
    kv = (kx, ky, kz)
    return [to_x(1j * kv[j] * u[a], shape) for a in range(3) for j in range(3)]


def band_weight(shape, band):
    """w(|k|) on the k layout: 0 for |k| <= band[0], 1 for |k| >= band[1]."""
    kx, ky, kz = kvectors(shape)
    kk = np.sqrt(kx ** 2 + ky ** 2 + kz ** 2)
    return np.clip((kk - band[0]) / (band[1] - band[0]), 0.0, 1.0)


def samples(u_dns, dns_shape, les_shape, delta, band=None):
    """raw [n][16] FP32 rows (G, delta, tau) of one DNS state u_dns (k arrays);
    with band = (lo, hi) the stress is restricted to that spectral band."""
    ux = [to_x(c, dns_shape) for c in u_dns]
    prods = [to_k(ux[a] * ux[b]) for a, b in PAIRS]
    ub = [truncate(c, dns_shape, les_shape) for c in u_dns]
    fb = [truncate(c, dns_shape, les_shape) for c in prods]
    ubx = [to_x(c, les_shape) for c in ub]
    fbx = [to_x(c, les_shape) for c in fb]
    G = gradients(ub, les_shape)
    n = int(np.prod(les_shape))
    raw = np.zeros((n, 16), dtype=np.float32)
    for a in range(9):
        raw[:, a] = G[a].ravel()
    raw[:, 9] = delta
    for c, (a, b) in enumerate(PAIRS):
        fr = to_x(to_k(ubx[a] * ubx[b]), les_shape)
        tau = fbx[c] - fr
        if band is not None:
            tau = to_x(to_k(tau) * band_weight(les_shape, band), les_shape)
        raw[:, 10 + c] = tau.ravel()
    return raw


def stress(u, shape, p, norm, delta, rounding=True):
    """Grid-point stresses (6 fields) predicted by the network for velocity u."""
    G = gradients(u, shape)
    n = int(np.prod(shape))
    feat = np.zeros((n, IN_PAD), dtype=np.float64)
    for a in range(9):
        feat[:, a] = G[a].ravel()
    feat[:, 9] = delta
    norm = np.asarray(norm, dtype=np.float32)
    f32 = feat.astype(np.float32)
    X = np.zeros_like(f32)
    X[:, :NIN] = (f32[:, :NIN] - norm[:NIN]) * norm[16:16 + NIN]
    Y, _ = forward(p, X, rounding)
    Yf = Y.astype(np.float32)
    tau = Yf[:, :NOUT] * norm[40:46] + norm[32:38]
    return [tau[:, c].astype(np.float64).reshape(shape) for c in range(NOUT)]


def shell_weight(shape, table):
    """w(|k|) on the k layout: table linearly interpolated at |k| (entry i at
    |k| = i), the last entry beyond the table."""
    kx, ky, kz = kvectors(shape)
    kk = np.sqrt(kx ** 2 + ky ** 2 + kz ** 2)
    t = np.asarray(table, dtype=np.float64)
    i = np.floor(kk).astype(np.int64)
    inside = i < t.size - 1
    ic = np.where(inside, i, 0)
    f = kk - i
    return np.where(inside, t[ic] + f * (t[np.minimum(ic + 1, t.size - 1)] - t[ic]), t[-1])


def transfer(u, tau, shape, nbins):
    """Per-shell subgrid energy transfer: sum over the modes with round(|k|) =
    b of Re(conj(u_a) (-i k_j tau_ij)^_a), over the full spectrum (kx > 0
    columns twice); u: 3 k arrays, tau: 6 grid-point fields."""
    th = [to_k(t) for t in tau]
    kx, ky, kz = kvectors(shape)
    kv = (kx, ky, kz)
    rows = [(0, 3, 4), (3, 1, 5), (4, 5, 2)]
    t = sum((np.conj(u[a]) * sum(-1j * kv[j] * th[rows[a][j]] for j in range(3))).real for a in range(3))
    nx = shape[2]
    ix = np.arange(nx // 2 + 1).reshape(1, 1, -1)
    m = np.where((ix > 0) & (2 * ix < nx), 2.0, 1.0)
    t = t * m * kept_mask(shape)
    b = np.floor(np.sqrt(kx ** 2 + ky ** 2 + kz ** 2) + 0.5).astype(np.int64)
    b = np.broadcast_to(b, t.shape)
    out = np.zeros(nbins)
    sel = b < nbins
    np.add.at(out, b[sel], t[sel])
    return out


def closure_term(u, shape, p, norm, delta, rounding=True, band=(0.0, 0.0), shells=None):
    """-w(|k|) P[d_j tau_ij]^ (3 k arrays, kept modes) for velocity u; w ramps
    linearly from 0 at |k| = band[0] to 1 at band[1] (w = 1 if band[1] <= 0),
    or, with a shell table, is shell_weight(shape, shells)."""
    tau = [to_k(t) for t in stress(u, shape, p, norm, delta, rounding)]
    kx, ky, kz = kvectors(shape)
    kv = (kx, ky, kz)
    rows = [(0, 3, 4), (3, 1, 5), (4, 5, 2)]
    s = [sum(1j * kv[j] * tau[rows[a][j]] for j in range(3)) for a in range(3)]
    k2 = kx ** 2 + ky ** 2 + kz ** 2
    k2 = np.where(k2 == 0, 1.0, k2)
    div = sum(kv[a] * s[a] for a in range(3)) / k2
    keep = kept_mask(shape)
    w = 1.0
    if shells is not None:
        w = shell_weight(shape, shells)
    elif band[1] > 0:
        kk = np.sqrt(kx ** 2 + ky ** 2 + kz ** 2)
        w = np.clip((kk - band[0]) / (band[1] - band[0]), 0.0, 1.0)
    return [-(s[a] - kv[a] * div) * keep * w for a in range(3)]


def les_physics(shape, p, norm, delta, band=(0.0, 0.0), shells=None):
    """Oracle RHS object of the closed LES: the oracle IncompressibleHydro RHS
    with its pressure projection, plus closure_term()."""
    from .physics import IncompressibleHydro
    from .representation import FourierRepresentation

    class _LES(IncompressibleHydro):
        def RHS(self, data, deriv):
            IncompressibleHydro.RHS(self, data, deriv)
            self.pressure_projection(data, deriv)     # skipped by the base for subclasses
            u = [data['u'][i]['kspace'] for i in range(3)]
            term = closure_term(u, shape, p, norm, delta, band=band, shells=shells)
            for i in range(3):
                deriv['u'][i]['kspace'] += term[i]

    return _LES(shape, FourierRepresentation)
