"""Device diagnostics with the reference's definitions: the k-space volume
averages of dedalus/analysis/volume_average.py (ekin, emag, energy
dissipation, enstrophy, divergence, per-component squares) and the binned
power spectrum of PowerSpectrum._compute_spectrum
(dedalus/analysis/analysis_set.py:778-815).  Sums are compensated FP64
reductions on the GPU; each function returns a Python float (or arrays for the
spectrum) and synchronises with the device.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from .engine import current_stream, dptr

ENERGY, DISSIPATION, ENSTROPHY2D, HELICITY, DIV_L2, DIV_ABS_SUM, SQUARE = range(7)


def _reduce(field_comps, kind):
    plan = field_comps[0].plan
    for c in field_comps:
        c.require_space('kspace')
    n = ctypes.c_size_t()
    _lib.call("dd_diag_workspace_size", plan.handle, 0, ctypes.byref(n))
    ws = plan.workspace(n.value, tag='diag')
    out = torch.empty(1, dtype=torch.float64, device=plan.device)
    ptrs, _keep = _lib.ptr_array([c.kdata.data_ptr() for c in field_comps])
    _lib.call("dd_volume_average", plan.handle, kind, len(field_comps), ptrs, dptr(out), dptr(ws), ws.numel(),
              current_stream())
    return float(out.item())


def _comps(field):
    return [c for i, c in field]


def ekin(data):
    """1/2 <|u|^2> (volume_average.py:109-118)."""
    return _reduce(_comps(data['u']), ENERGY)


def emag(data):
    """1/2 <|B|^2> (volume_average.py:180-188)."""
    return _reduce(_comps(data['B']), ENERGY)


def energy_dissipation(data, nu=None):
    """2 nu 1/2 <|curl u|^2> (volume_average.py:254-265), 3D."""
    nu = data.parameters['nu'] if nu is None else nu
    return 2 * nu * _reduce(_comps(data['u']), DISSIPATION)


def enstrophy(data):
    """1/2 <w_z^2> in 2D (volume_average.py:191-200)."""
    return _reduce(_comps(data['u']), ENSTROPHY2D)


def helicity(data):
    """<u . curl u>, 3D."""
    return _reduce(_comps(data['u']), HELICITY)


def divergence_l2(data, name='u'):
    """<(div u)^2>: the mean square divergence."""
    return _reduce(_comps(data[name]), DIV_L2)


def divergence_sum(data, name='u'):
    """sum |div u| over the stored k entries (volume_average.py:288-295)."""
    return _reduce(_comps(data[name]), DIV_ABS_SUM)


def square(comp):
    """< |c|^2 > of one component (ux2, uy2, temp2 ...)."""
    return _reduce([comp], SQUARE)


def spectrum_bins(field):
    """The reference's bin edges for a field (analysis_set.py:791-795)."""
    c0 = field[0]
    kmax = np.sqrt(np.sum(c0.kny ** 2))
    n = np.min(c0.global_shape['xspace']) / 2.
    n = int(np.min([n, 100]))
    kbottom = np.linspace(0, kmax, n, endpoint=False)
    ktop = kbottom + kbottom[1]
    return kbottom, ktop


def shell_bins(field):
    """Unit-width shells centred on the integers: [k - 1/2, k + 1/2) for
    k = 0 .. the largest |k| of the grid (the first shell starts at 0)."""
    c0 = field[0]
    kmax = np.sqrt(np.sum(c0.kny ** 2))
    k = np.arange(int(np.ceil(kmax)) + 2, dtype=np.float64)
    return np.maximum(k - 0.5, 0.0), k + 0.5


def power_spectrum(field, norm=1., shells=False):
    """(bin centres, mean power1d per bin) as PowerSpectrum._compute_spectrum;
    with shells=True the same estimator over unit shells centred on the
    integers (shell_bins) instead of the reference's bins."""
    comps = _comps(field)
    plan = comps[0].plan
    for c in comps:
        c.require_space('kspace')
    kbottom, ktop = shell_bins(field) if shells else spectrum_bins(field)
    nb = kbottom.size
    n = ctypes.c_size_t()
    _lib.call("dd_diag_workspace_size", plan.handle, nb, ctypes.byref(n))
    ws = plan.workspace(n.value, tag='diag_spec')
    kb = torch.from_numpy(kbottom).to(plan.device)
    kt = torch.from_numpy(ktop).to(plan.device)
    s = torch.empty(nb, dtype=torch.float64, device=plan.device)
    cnt = torch.empty(nb, dtype=torch.float64, device=plan.device)
    ptrs, _keep = _lib.ptr_array([c.kdata.data_ptr() for c in comps])
    dk = float(ktop[0] - kbottom[0]) if not shells else 1.0
    _lib.call("dd_spectrum", plan.handle, len(comps), ptrs, float(norm), nb, dptr(kb), dptr(kt), dk,
              dptr(s), dptr(cnt), dptr(ws), ws.numel(), current_stream())
    spec = s.cpu().numpy()
    counts = cnt.cpu().numpy()
    counts[counts == 0] = 1.
    if shells:
        return np.arange(nb, dtype=np.float64), spec / counts
    return kbottom + kbottom[1] / 2., spec / counts
