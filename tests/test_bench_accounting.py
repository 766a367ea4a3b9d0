"""The algorithmic byte and flop counts that bench.py's roofline fractions
divide by, checked on the CPU against the per-step figures the measurement
plan fixes for each configuration (rotational / curl forms), and the
divergence forms' counts that the measured lines report beside them."""
import importlib.util
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(HERE, "..", "bench.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


class _Rhs:
    def __init__(self, phys):
        self.last_phys3d = phys


def _hydro3(b, kind, phys, shape=(256, 256, 256)):
    r = object.__new__(b.Hydro3Runner)
    r.wl = dict(kind=kind, shape=shape, precision="fp64")
    r.mhd = kind == "mhd3d"
    r.rhs = _Rhs(phys)
    return r


def test_3d_step_bytes_and_flops():
    b = _bench()
    h = _hydro3(b, "hydro3d", 0)
    assert h.bytes_per_step() == 14_571_012_096 == h.canonical_bytes_per_step()
    assert h.transforms_per_rhs() == 9
    assert abs(h.flops_per_step() - 3.62e10) < 0.005e10
    hd = _hydro3(b, "hydro3d", 2)
    assert hd.transforms_per_rhs() == 8 and hd.divergence_form()
    assert hd.bytes_per_step() == 14_575_206_400
    assert abs(hd.flops_per_step() / h.flops_per_step() - 8 / 9) < 1e-12
    m = _hydro3(b, "mhd3d", 1)
    assert m.bytes_per_step() == 29_142_024_192 == m.canonical_bytes_per_step()
    md = _hydro3(b, "mhd3d", 3)
    assert md.transforms_per_rhs() == 14
    # non-cubic grids use the same formula per axis
    assert b.B3s((256, 256, 256)) == b.B3(256) and b.C3s((256, 256, 256)) == b.C3(256)


def test_2d_step_bytes():
    b = _bench()
    r = object.__new__(b.Hydro2Runner)
    r.wl = dict(shape=(128, 128), precision="fp64")
    assert r.bytes_per_step() == 4_239_360
    # one run of the ensemble, curl form: 2 RHS x 8 transforms + 2 stages x 3 fields x 3 passes
    per = {n: 2 * 8 * b.B2(n) + 2 * 3 * 3 * b.C2(n) for n in (64, 128, 256, 512)}
    assert per == {64: 1_673_216, 128: 6_623_232, 256: 26_353_664, 512: 105_136_128}


def test_kernel_bytes_of_the_divergence_form():
    b = _bench()
    hd = _hydro3(b, "hydro3d", 2)
    N, M = 256, 85
    kc = (2 * M + 1) ** 2 * (M + 1) * 16
    w1, w2 = (2 * M + 1) * N * (M + 1) * 16, N * N * (M + 1) * 16
    assert hd.kernel_bytes("x_div_256_f64") == 8 * w2
    assert hd.kernel_bytes("y_inv_256_f64") == 3 * (w1 + w2)
    assert hd.kernel_bytes("y_fwd_256_f64") == 5 * (w2 + w1)
    assert hd.kernel_bytes("z_fwd_compact_256_f64") == 5 * (w1 + kc)
    assert hd.kernel_bytes("rk4_stage3") == 15 * kc + 2 * kc
    assert np.isclose(hd.kernel_flops("x_div_256_f64"), N * N * (8 * 0.5 * 5 * N * np.log2(N) + 7 * N))
