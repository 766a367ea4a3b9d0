"""The closure oracle (oracle/closure.py) pinned on the CPU: the analytic MLP
gradient against central finite differences, the BF16 rounding helper against
known values, and the sharp-filter identity of the training stress."""
import numpy as np
import pytest

from oracle import closure as OC


def _problem(n=37, seed=0):
    rng = np.random.Generator(np.random.PCG64(seed))
    p = OC.init_params(seed).astype(np.float64)
    w = OC.unpack(p.copy())
    w["b1"][:] = rng.normal(0, 0.1, 64)
    w["b2"][:] = rng.normal(0, 0.1, 64)
    w["b3"][:6] = rng.normal(0, 0.1, 6)
    p = OC.pack(w)
    X = np.zeros((n, 16))
    X[:, :10] = rng.normal(0, 1, (n, 10))
    T = np.zeros((n, 8))
    T[:, :6] = rng.normal(0, 1, (n, 6))
    return p, X, T


def test_exact_gradient_matches_finite_differences():
    p, X, T = _problem()
    g, _ = OC.grad(p, X, T, rounding=False)
    rng = np.random.Generator(np.random.PCG64(5))
    live = [i for i in range(OC.NPARAM) if g[i] != 0.0]
    pick = rng.choice(live, 60, replace=False)
    h = 1e-6
    for i in pick:
        a, b = p.copy(), p.copy()
        a[i] += h
        b[i] -= h
        fd = (OC.loss(a, X, T, rounding=False)[0] - OC.loss(b, X, T, rounding=False)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-7 * max(1.0, abs(g[i])), (i, fd, g[i])


def test_unused_inputs_and_outputs_get_zero_gradient():
    p, X, T = _problem()
    g = OC.unpack(OC.grad(p, X, T)[0])
    assert np.all(g["W1"][:, 10:] == 0)
    assert np.all(g["W3"][6:] == 0) and np.all(g["b3"][6:] == 0)


def test_bf16_rounding():
    v = np.array([1.0, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -8, -2.5, 3.0e-3, 1.0 + 2.0 ** -7])
    r = OC.bf16(v)
    assert r[0] == 1.0
    assert r[1] == 1.0                       # tie -> even
    assert r[2] == 1.0 + 2.0 ** -6           # tie -> even (upwards)
    assert r[3] == -2.5
    assert abs(r[4] - 3.0e-3) <= 3.0e-3 * 2.0 ** -8
    assert r[5] == 1.0 + 2.0 ** -7


def test_sharp_filter_identity():
    """A DNS field that is band-limited to the LES kept set gives stresses
    whose kept modes vanish: filt(uu) - filt(ubar ubar) = 0."""
    dns, les = (24, 24, 24), (12, 12, 12)
    rng = np.random.Generator(np.random.PCG64(2))
    keep = OC.kept_mask(les)
    u = []
    for _ in range(3):
        x = rng.normal(size=les)
        u.append(OC.to_k(x) * keep)
    # embed on the DNS grid
    u_dns = []
    kxl, kyl, kzl = OC.kvectors(les)
    for c in u:
        big = np.zeros((dns[1], dns[0], dns[2] // 2 + 1), dtype=np.complex128)
        for iy in range(les[1]):
            for iz in range(les[0]):
                big[int(kyl.ravel()[iy]) % dns[1], int(kzl.ravel()[iz]) % dns[0], :les[2] // 2 + 1] = c[iy, iz]
        u_dns.append(big * OC.kept_mask(dns))
    raw = OC.samples(u_dns, dns, les, delta=np.pi / 3)
    assert np.all(raw[:, 9] == np.float32(np.pi / 3))
    scale = max(np.max(np.abs(OC.to_x(c, les))) for c in u) ** 2
    assert np.max(np.abs(raw[:, 10:])) < 1e-12 * scale
    # gradients are those of the filtered field itself
    G = OC.gradients(u, les)
    assert np.allclose(raw[:, 0].reshape(les), G[0], atol=1e-5 * np.max(np.abs(G[0])))


def test_constant_stress_gives_no_closure_term():
    shape = (12, 12, 12)
    rng = np.random.Generator(np.random.PCG64(3))
    u = [OC.to_k(rng.normal(size=shape)) for _ in range(3)]
    p = OC.init_params(1)
    w = OC.unpack(p.astype(np.float64))
    w["W3"][:] = 0.0
    norm = np.zeros(48, dtype=np.float32)
    norm[16:32] = 1.0
    norm[40:48] = 1.0
    norm[32:38] = [0.3, 0.2, 0.1, 0.05, 0.0, -0.1]
    t = OC.closure_term(u, shape, OC.pack(w), norm, 0.1)
    assert max(np.max(np.abs(c)) for c in t) < 1e-14


def _solenoidal(shape, seed):
    """Random kept-mode solenoidal velocity (3 k arrays)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    u = [OC.to_k(rng.normal(size=shape)) for _ in range(3)]
    kx, ky, kz = OC.kvectors(shape)
    k2 = kx ** 2 + ky ** 2 + kz ** 2
    d = (kx * u[0] + ky * u[1] + kz * u[2]) / np.where(k2 == 0, 1.0, k2)
    return [u[0] - kx * d, u[1] - ky * d, u[2] - kz * d]


def test_transfer_sums_to_stress_strain_product():
    """Parseval: the per-shell transfers of a solenoidal velocity add up to
    <tau_ij S_ij> over the grid (all shells kept)."""
    shape = (16, 16, 16)
    u = _solenoidal(shape, 5)
    rng = np.random.Generator(np.random.PCG64(6))
    tau = [OC.to_x(OC.to_k(rng.normal(size=shape)), shape) for _ in range(6)]
    T = OC.transfer(u, tau, shape, 64)
    G = OC.gradients(u, shape)           # G[3 a + j] = d_j u_a
    ts = 0.0
    for c, (a, b) in enumerate(OC.PAIRS):
        s = 0.5 * (G[3 * a + b] + G[3 * b + a])
        ts += (1.0 if a == b else 2.0) * np.mean(tau[c] * s)
    assert abs(T.sum() - ts) <= 1e-12 * max(abs(ts), np.max(np.abs(T)))


def test_shell_table_interpolates_and_reproduces_a_ramp():
    shape = (16, 16, 16)
    lo, hi = 2.0, 6.0
    table = np.clip((np.arange(8.0) - lo) / (hi - lo), 0.0, 1.0)
    w = OC.shell_weight(shape, table)
    kx, ky, kz = OC.kvectors(shape)
    kk = np.sqrt(kx ** 2 + ky ** 2 + kz ** 2)
    ramp = np.clip((kk - lo) / (hi - lo), 0.0, 1.0)
    assert np.allclose(w, ramp, rtol=0, atol=1e-15)
    # beyond the table: its last entry
    w2 = OC.shell_weight(shape, [0.5, 1.5, 2.5])
    assert np.all(w2[kk >= 2.0] == 2.5)
    sel = kk < 2.0
    assert np.allclose(w2[sel], (0.5 + kk)[sel], atol=1e-15)


def test_shell_count_covers_the_kept_modes():
    """closure.shell_count bins round(|k|) over the kept cube |m_i| <= ceil(N/3) - 1."""
    pytest.importorskip("torch")
    import __graft_entry__
    dd = __graft_entry__.load_package()
    for n in (16, 32, 64):
        shape = (n, n, n)
        kx, ky, kz = OC.kvectors(shape)
        kk = np.sqrt(kx ** 2 + ky ** 2 + kz ** 2)
        top = int(np.max(np.floor(kk[np.broadcast_to(OC.kept_mask(shape), kk.shape)] + 0.5)))
        assert dd.closure.shell_count(n) == top + 1
