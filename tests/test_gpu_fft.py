"""Transform parity: dd_fft_r2c / dd_fft_c2r (through the C ABI) against the
oracle's numpy restatement of the reference's forward/backward
(representations.py:327-357: rfftn(x/N) transposed then 2/3 dealias;
dealias then irfftn*N).  FP64 tolerance: 1e-13 relative max error; FP32
compute path: 2e-6."""
import numpy as np
import pytest

from oracle.representation import FourierRepresentation, decfg

SHAPES_3D = [(8, 8, 8), (16, 8, 32), (32, 64, 16), (64, 64, 64), (128, 32, 256), (256, 256, 256)]
SHAPES_2D = [(8, 8), (16, 64), (128, 128), (256, 32), (512, 512)]


def _oracle_rep(shape, dealias='2/3 cython'):
    decfg.set('FFT', 'dealiasing', dealias)
    try:
        return FourierRepresentation(None, shape, (2 * np.pi,) * len(shape))
    finally:
        decfg.set('FFT', 'dealiasing', '2/3 cython')


def _relerr(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.gpu
@pytest.mark.parametrize("shape", SHAPES_3D + SHAPES_2D)
@pytest.mark.parametrize("dealias", ['2/3 cython', 'None'])
def test_r2c_matches_oracle(dd, cuda, shape, dealias):
    import torch
    rng = np.random.default_rng(sum(shape) + len(str(dealias)))
    x = rng.standard_normal(shape)
    rep = _oracle_rep(shape, dealias)
    rep['xspace'] = x
    kref = rep['kspace'].copy()
    plan = dd.engine.Plan(shape, (2 * np.pi,) * len(shape), dealias)
    xd = torch.from_numpy(x).to(cuda)
    kd = torch.full(plan.kshape, complex(7, 7), dtype=torch.complex128, device=cuda)
    plan.r2c([xd], [kd])
    got = kd.cpu().numpy()
    assert _relerr(got, kref) < 1e-13
    # dealiased modes are exactly zero
    assert np.array_equal(got[kref == 0], kref[kref == 0])


@pytest.mark.gpu
@pytest.mark.parametrize("shape", SHAPES_3D + SHAPES_2D)
def test_c2r_matches_oracle(dd, cuda, shape):
    import torch
    rng = np.random.default_rng(sum(shape))
    rep = _oracle_rep(shape)
    # arbitrary (not Hermitian) spectrum: c2r semantics of the kx=0 plane must match numpy
    k = rng.standard_normal(rep.kdata.shape) + 1j * rng.standard_normal(rep.kdata.shape)
    rep['kspace'] = k
    xref = rep['xspace'].copy()   # dealias + irfftn * N
    plan = dd.engine.Plan(shape, (2 * np.pi,) * len(shape))
    kd = torch.from_numpy(k).to(cuda)
    xd = torch.empty(shape, dtype=torch.float64, device=cuda)
    plan.c2r([kd], [xd])
    assert _relerr(xd.cpu().numpy(), xref) < 1e-13
    # the input is read only
    assert np.array_equal(kd.cpu().numpy(), k)


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(32, 64, 16), (64, 64, 64), (128, 128)])
def test_multifield_and_fp32(dd, cuda, shape):
    import torch
    rng = np.random.default_rng(5)
    xs = [rng.standard_normal(shape) for _ in range(3)]
    refs = []
    for x in xs:
        rep = _oracle_rep(shape)
        rep['xspace'] = x
        refs.append(rep['kspace'].copy())
    plan = dd.engine.Plan(shape, (2 * np.pi,) * len(shape))
    xd = [torch.from_numpy(x).to(cuda) for x in xs]
    for prec, tol in ((dd._lib.DD_FP64, 1e-13), (dd._lib.DD_FP32, 2e-6)):
        kd = [torch.zeros(plan.kshape, dtype=torch.complex128, device=cuda) for _ in xs]
        plan.r2c(xd, kd, precision=prec)
        for got, ref in zip(kd, refs):
            assert _relerr(got.cpu().numpy(), ref) < tol
        xb = [torch.empty(shape, dtype=torch.float64, device=cuda) for _ in xs]
        plan.c2r(kd, xb, precision=prec)
        n = np.prod(shape)
        for got, x, ref in zip(xb, xs, refs):
            rep = _oracle_rep(shape)
            rep['kspace'] = ref
            assert _relerr(got.cpu().numpy(), rep['xspace']) < tol


@pytest.mark.gpu
def test_unsupported_shape_raises(dd, cuda):
    with pytest.raises(NotImplementedError):
        dd.engine.Plan((48, 2, 48), (2 * np.pi,) * 3)
