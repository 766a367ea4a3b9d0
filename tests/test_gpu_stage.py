"""Stage-kernel parity: dd_euler / dd_etd1 / dd_etd2rk1 / dd_etd2rk2 and the
phi table (C ABI) against the oracle's C restatement of the reference's
Cython kernels.  The arithmetic is the same operation by operation; exp/pow
may differ in the last bit, so the tolerance is 1e-14 relative."""
import ctypes

import numpy as np
import pytest

from oracle._cstage import stage2d, stage3d


def _inputs(n, seed):
    rng = np.random.default_rng(seed)
    s = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    d1 = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    d2 = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    # intfactor spanning Z == 0, the Taylor branch |Z| < 0.5 and the exp branch
    intf = -np.abs(rng.standard_normal(n)) * rng.choice([0., 0.1, 1., 30., 1e3], n)
    return s, d1, d2, intf


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


@pytest.mark.gpu
@pytest.mark.parametrize("ndim", [2, 3])
@pytest.mark.parametrize("dt", [1e-3, 0.05, 0.7])
def test_stage_kernels(dd, cuda, ndim, dt):
    import torch
    n = 4099
    s, d1, d2, intf = _inputs(n, ndim * 10 + int(dt * 1000))
    ks = stage2d if ndim == 2 else stage3d
    shp = (n, 1) if ndim == 2 else (n, 1, 1)
    S, D1, D2, IF = (a.reshape(shp).copy() for a in (s, d1, d2, intf))
    T = {k: torch.from_numpy(v.reshape(-1)).to(cuda) for k, v in dict(s=s, d1=d1, d2=d2, f=intf).items()}
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    L = dd._lib

    def check(got, ref):
        assert np.abs(got - ref).max() <= 1e-14 * max(1., np.abs(ref).max())

    o = torch.empty_like(T['s'])
    L.call("dd_euler", _p(T['s']), _p(o), _p(T['d1']), dt, n, st)
    r = np.empty_like(S); ks.euler(S, r, D1, dt)
    check(o.cpu().numpy(), r.reshape(-1))

    L.call("dd_etd1", ndim, _p(T['s']), _p(o), _p(T['d1']), _p(T['f']), dt, n, st)
    r = np.empty_like(S); ks.etd1(S, r, D1, IF, dt)
    check(o.cpu().numpy(), r.reshape(-1))

    L.call("dd_etd2rk1", ndim, _p(T['s']), _p(o), _p(T['d1']), _p(T['d2']), _p(T['f']), dt, n, st)
    r = np.empty_like(S); ks.etd2rk1(S, r, D1, D2, IF, dt)
    check(o.cpu().numpy(), r.reshape(-1))

    L.call("dd_etd2rk2", ndim, _p(T['s']), _p(o), _p(T['d1']), _p(T['d2']), _p(T['f']), dt, n, st)
    r = np.empty_like(S); ks.etd2rk2(S, r, D1, D2, IF, dt)
    check(o.cpu().numpy(), r.reshape(-1))

    # output aliasing start (the reference calls etd2rk2(data, data, ...))
    a = T['s'].clone()
    L.call("dd_etd2rk2", ndim, _p(a), _p(a), _p(T['d1']), _p(T['d2']), _p(T['f']), dt, n, st)
    check(a.cpu().numpy(), r.reshape(-1))


@pytest.mark.gpu
@pytest.mark.parametrize("ndim", [2, 3])
def test_phi_table(dd, cuda, ndim):
    import torch
    nu, h, qmax = 5e-3, 2e-3, 49152
    tab = torch.empty((qmax + 1, 4), dtype=torch.float64, device=cuda)
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    dd._lib.call("dd_phi_table", ndim, nu, 1, h, qmax, _p(tab), st)
    t = tab.cpu().numpy()
    q = np.arange(qmax + 1, dtype=np.float64)
    intf = -(nu * q)
    # etd1 of start=1, deriv=0 gives f0; start=0, deriv=1 gives f1*dt
    ks = stage2d if ndim == 2 else stage3d
    shp = (qmax + 1, 1) if ndim == 2 else (qmax + 1, 1, 1)
    one = np.ones(shp, complex); zero = np.zeros(shp, complex); out = np.empty(shp, complex)
    IF = intf.reshape(shp).copy()
    ks.etd1(one, out, zero, IF, h)
    assert np.abs(t[:, 1] - out.real.reshape(-1)).max() <= 1e-15
    ks.etd1(zero, out, one, IF, h)
    f1 = np.where(t[:, 0] == 0, 1.0, t[:, 2])
    assert np.abs(f1 * h - out.real.reshape(-1)).max() <= 1e-15 * h
    np.testing.assert_array_equal(t[:, 0], intf * h)
