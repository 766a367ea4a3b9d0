"""The oracle against the reference's own execution.

``tests/golden/ref_*.npz`` hold what the reference's own Python code (its
representation, fields, physics and RK2mid / RK2trap integrators, run under
Python 3 after mechanical rewrites, with its own compiled Cython kernels and
FFT.method = numpy) computed on seeded inputs; ``oracle/ref_fixtures.py``
made them.  The oracle must reproduce every stored RHS, every step and the
CFL dt from the same inputs to roundoff (relative L2 <= 1e-14 over all
fields; the dt to 1e-15), which pins the restatement's layout, lazy space
switching, operator order, projection and integrators to the reference
itself rather than to a reading of it.  On the machine type and numpy version
that made the fixtures the match is required to be bit-exact (it is: the
oracle performs the reference's numpy operations in the reference's order).
CPU only."""
import glob
import os
import platform

import numpy as np
import pytest

from oracle import physics as OP, time_step as OT
from oracle import representation as OR

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


def physics(z, params):
    # the plain Fourier representation, or the shearing box
    # (representations.py:558-740) for the shear_* fixtures
    rep = getattr(OR, str(z["rep"])) if "rep" in z.files else OR.FourierRepresentation
    length = tuple(float(v) for v in z["length"]) if "length" in z.files else None
    rhs = getattr(OP, str(z["cls"]))(tuple(int(v) for v in z["shape"]), rep, length=length)
    rhs.parameters.update(params)
    return rhs


def seeded(rhs, z, names):
    data = rhs.create_fields(0.)
    for f, c in names:
        data[f][c]['kspace'] = z["in_%s%d" % (f, c)].copy()
    return data


def test_fixtures_present():
    assert len(FILES) == 19, FILES
    assert sum(os.path.basename(f).startswith("ref_shear_") for f in FILES) == 6


@pytest.mark.parametrize("path", FILES, ids=[os.path.basename(f)[4:-4] for f in FILES])
def test_oracle_matches_reference_execution(path):
    z, names, params = load(path)
    exact = str(z["numpy_version"]) == np.__version__ and str(z["machine"]) == platform.machine()

    def check(got, ref, what):
        e = rel_l2(got, ref)
        assert e <= 1e-14, (what, e)
        if exact:
            for g, r in zip(got, ref):
                np.testing.assert_array_equal(g, r, err_msg=what)
    # one RHS call
    rhs = physics(z, params)
    data = seeded(rhs, z, names)
    deriv = rhs.create_fields(0.)
    rhs.RHS(data, deriv)
    got = [deriv[f][c]['kspace'] for f, c in names]
    ref = [z["rhs_%s%d" % (f, c)] for f, c in names]
    check(got, ref, "rhs")
    # the integrator's steps
    rhs = physics(z, params)
    data = seeded(rhs, z, names)
    ti = getattr(OT, str(z["integrator"]))(rhs)
    for s in range(int(z["nsteps"])):
        ti.do_advance(data, float(z["dt"]))
        got = [data[f][c]['kspace'] for f, c in names]
        ref = [z["step%d_%s%d" % (s + 1, f, c)] for f, c in names]
        check(got, ref, "step %d" % (s + 1))
    # CFL dt of the final state
    dt = rhs.compute_dt(data)
    assert abs(dt - float(z["compute_dt"])) <= 1e-15 * float(z["compute_dt"])
    if exact:
        assert dt == float(z["compute_dt"])
    np.testing.assert_allclose(rhs.dtlist, z["dtlist"], rtol=1e-15, atol=0)
