"""Pin the oracle: its C restatement of the stage and dealias kernels
(oracle/stage.c) against the reference's own Cython kernels compiled from the
reference sources into oracle/_ref (oracle/build_ref.py).  Same machine, same
libm, no FMA contraction on either side: results must be bit-identical.
Skipped where oracle/_ref was not built (the GPU host has no Cython)."""
import numpy as np
import pytest

from oracle import build_ref
from oracle._cstage import stage2d, stage3d, dealias_23
from oracle.representation import FourierRepresentation


def _ref(name):
    mod = build_ref.load(name)
    if mod is None:
        pytest.skip("oracle/_ref/%s not built" % name)
    return mod


def _inputs(shape, seed):
    rng = np.random.default_rng(seed)
    c = lambda: rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    intf = -np.abs(rng.standard_normal(shape)) * rng.choice([0., 0.1, 1., 30., 1e3], shape)
    return c(), c(), c(), intf


@pytest.mark.parametrize("ndim", [2, 3])
@pytest.mark.parametrize("dt", [1e-3, 0.3, 2.0])
def test_stage_kernels_bit_exact(ndim, dt):
    ref = _ref("forward_step_cy_%dd" % ndim)
    mine = stage2d if ndim == 2 else stage3d
    shape = (9, 17) if ndim == 2 else (5, 7, 9)
    s, d1, d2, intf = _inputs(shape, ndim)
    for name, args in (("euler", (d1,)), ("etd1", (d1, intf)), ("etd2rk1", (d1, d2, intf)),
                       ("etd2rk2", (d1, d2, intf))):
        a = np.empty_like(s)
        b = np.empty_like(s)
        getattr(ref, name)(s, a, *args, dt)
        getattr(mine, name)(s, b, *args, dt)
        assert np.array_equal(a.view(np.float64), b.view(np.float64)), name


@pytest.mark.parametrize("ndim", [2, 3])
def test_stage_rejects_wrong_dtype(ndim):
    mine = stage2d if ndim == 2 else stage3d
    shape = (4, 4) if ndim == 2 else (2, 2, 2)
    s = np.zeros(shape, np.complex64)
    with pytest.raises(ValueError):
        mine.euler(s, s, s, 0.1)


@pytest.mark.parametrize("shape", [(12, 16), (32, 8), (8, 12, 16), (16, 16, 16)])
def test_dealias_bit_exact(shape):
    ndim = len(shape)
    ref = _ref("dealias_cy_%dd" % ndim)
    rep = FourierRepresentation(None, shape, (2 * np.pi,) * ndim)
    rng = np.random.default_rng(1)
    a = rng.standard_normal(rep.kdata.shape) + 1j * rng.standard_normal(rep.kdata.shape)
    b = a.copy()
    c = a.copy()
    k = [rep.k['x'], rep.k['y']] + ([rep.k['z']] if ndim == 3 else [])
    ref.dealias_23(a, *k, rep.kny)
    dealias_23(b, *k, rep.kny)
    assert np.array_equal(a, b)
    # the numpy '2/3' method of the representation gives the same mask
    rep.kdata[:] = c
    rep.dealias_23()
    assert np.array_equal(rep.kdata, a)
