"""The CUDA path against the reference's own execution.

``tests/golden/ref_*.npz`` were computed by the reference's own Python code
(run under Python 3 after mechanical rewrites, with its compiled Cython
kernels and FFT.method = numpy; ``oracle/ref_fixtures.py``).  Here the
library's public classes -- the same physics, representation and
integrators, on the GPU; the shearing box and rotation through the
reference-ordered path -- start from the stored inputs and must reproduce
the stored RHS, every stored RK2mid / RK2trap step and the CFL dt:
relative L2 <= 1e-12 over all fields, dt to 1e-12 relative."""
import glob
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FILES = sorted(glob.glob(os.path.join(GOLDEN, "ref_*.npz")))


def rel_l2(got, ref):
    num = sum(np.sum(np.abs(g - r) ** 2) for g, r in zip(got, ref))
    den = sum(np.sum(np.abs(r) ** 2) for r in ref)
    return float(np.sqrt(num / den))


def load(path):
    z = np.load(path, allow_pickle=False)
    names = [(str(n)[0], int(str(n)[1:])) for n in z["names"]]
    params = dict(eval(str(z["params"])))
    return z, names, params


@pytest.mark.gpu
@pytest.mark.parametrize("path", FILES, ids=[os.path.basename(f)[4:-4] for f in FILES])
def test_cuda_path_matches_reference_execution(dd, cuda, path):
    z, names, params = load(path)
    M = dd.mods
    shape = tuple(int(v) for v in z["shape"])

    # the plain Fourier representation, or the shearing box for the shear_* fixtures
    rep = getattr(M, str(z["rep"])) if "rep" in z.files else M.FourierRepresentation
    length = tuple(float(v) for v in z["length"]) if "length" in z.files else None

    def seeded():
        rhs = getattr(M, str(z["cls"]))(shape, rep, length=length)
        rhs.parameters.update(params)
        data = rhs.create_fields(0.)
        for f, c in names:
            data[f][c]['kspace'] = z["in_%s%d" % (f, c)]
        return rhs, data

    rhs, data = seeded()
    deriv = rhs.create_fields(0.)
    rhs.RHS(data, deriv)
    got = [deriv[f][c].to_numpy('kspace') for f, c in names]
    e = rel_l2(got, [z["rhs_%s%d" % (f, c)] for f, c in names])
    assert e < 1e-12, ("rhs", e)
    rhs, data = seeded()
    ti = getattr(M, str(z["integrator"]))(rhs)
    for s in range(int(z["nsteps"])):
        ti.do_advance(data, float(z["dt"]))
        got = [data[f][c].to_numpy('kspace') for f, c in names]
        e = rel_l2(got, [z["step%d_%s%d" % (s + 1, f, c)] for f, c in names])
        assert e < 1e-12, ("step %d" % (s + 1), e)
    dt = rhs.compute_dt(data)
    assert abs(dt - float(z["compute_dt"])) <= 1e-12 * float(z["compute_dt"])
    np.testing.assert_allclose(rhs.dtlist, z["dtlist"], rtol=1e-12, atol=0)
