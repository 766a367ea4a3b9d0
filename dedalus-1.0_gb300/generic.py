"""Reference-ordered right-hand sides on the GPU, for the physics branches the
fused kernels do not cover: the shearing box (``FourierShearRepresentation``
with ``shear_rate`` != 0), rotation (``Omega``), 3D Boussinesq and 2D MHD.

The operator helpers are the reference's (dedalus/physics/physics.py:
``divX`` 180-195, ``XgradY`` 197-228, ``XconstcrossY`` 266-307,
``XcrossY`` 309-354, ``curlX`` 374-405, ``laplace_solve`` 407-416,
``pressure_projection`` 588-599) with the same lazy x/k-space transforms,
operand order and one rounding per numpy operation; every arithmetic step is
a CUDA kernel (``dd_scale_add``, ``dd_kspace_real``, ``dd_xspace_fma``,
``dd_deriv`` / ``dd_shear_deriv_y``) and every transform the representation's
(``dd_fft_*`` or ``dd_shear_*``).  The right-hand sides keep the advective
form u.grad(u) of the reference: with the shear the pressure solve divides by
a k^2 that is not the current one (below), so the gradient that separates the
advective from the rotational form would not cancel.

``laplace_solve`` caches k^2 (no zero) at its first call, as the reference
does (physics.py:412-413): in a shearing box the pressure solve then keeps
dividing by the k^2 of the first RHS time.  ``laplace_k2 = 'current'`` on the
physics object divides by the current k^2 instead.
"""
import numpy as np
import torch

from . import _lib
from .engine import current_stream, dptr


# ----------------------------------------------------------- elementwise ops
def _kset(comp):
    comp.data = comp.kdata
    comp._curr_space = 'kspace'


def _xset(comp):
    comp.data = comp.xdata
    comp._curr_space = 'xspace'


def kaxpy(out, x, w, accumulate):
    """out = x * w, or out + x * w (complex k arrays, real w)."""
    _lib.call("dd_scale_add", dptr(x), dptr(out), float(w), 1 if accumulate else 0, x.numel(), current_stream())


def kreal(out, x, r, w, mode, accumulate=False):
    _lib.call("dd_kspace_real", x.numel(), dptr(x), dptr(r), float(w), int(mode), 1 if accumulate else 0,
              dptr(out), current_stream())


def xfma(out, a, b, w, accumulate):
    _lib.call("dd_xspace_fma", a.numel(), dptr(a), None if b is None else dptr(b), float(w),
              1 if accumulate else 0, dptr(out), current_stream())


def kval(comp):
    """comp['kspace'] as a device tensor (transforming if needed)."""
    comp.require_space('kspace')
    return comp.kdata


def xval(comp):
    comp.require_space('xspace')
    return comp.xdata


class ReferenceOrderRHS:
    """Mixin of the physics classes: the reference's operator sequence."""

    laplace_k2 = 'cached'

    # ---------------------------------------------------------- helpers
    def _aux(self):
        aux = getattr(self, 'aux_fields', None)
        if aux is None:
            # physics.py:108-113, 118-119
            aux = self.aux_fields = self.create_fields(0., self._aux_field_list)
        return aux

    def _base_rhs(self, data, deriv):
        # physics.py:134-149
        for fname, field in deriv:
            field.zero_all()
        for fname, field in self._aux():
            field.zero_all(space='kspace')
        deriv.set_time(data.time)
        self.aux_fields.set_time(data.time)

    def divX(self, X, output):
        # physics.py:180-195
        output.zero()
        out = output.components[0]
        for i in range(X.ncomp):
            d = X[i].deriv(self._trans[i])
            kaxpy(kval(out), d, 1.0, True)
        _kset(out)

    def XgradY(self, X, Y, stmp, vtmp, output):
        # physics.py:197-228: output_c = sum_i (d_i Y_c) X_i at the grid points
        output.zero_all('xspace')
        for cindex, comp in X:
            vtmp[cindex]['kspace'] = kval(comp)
        s = stmp.components[0]
        for cindex, comp in Y:
            out = output[cindex] if Y.ncomp > 1 else output.components[0]
            for i in self.dims:
                s['kspace'] = comp.deriv(self._trans[i])
                xfma(xval(out), xval(s), xval(vtmp[i]), 1.0, True)
                _xset(out)

    def XconstcrossY(self, X, Y, output):
        # physics.py:266-307 (k-space, X constant)
        Yx, Yy = kval(Y['x']), kval(Y['y'])
        if self.ndim == 2:
            if np.isscalar(X):
                Xz = float(X)
                ox, oy = output['x'], output['y']
                kaxpy(ox.kdata, Yy, -Xz, False)
                kaxpy(oy.kdata, Yx, Xz, False)
                _kset(ox)
                _kset(oy)
            else:
                Xy, Xx = (float(v) for v in X)
                o = output.components[0]
                kaxpy(o.kdata, Yy, Xx, False)
                kaxpy(o.kdata, Yx, -Xy, True)
                _kset(o)
            return
        Xz, Xy, Xx = (float(v) for v in X)
        Yz = kval(Y['z'])
        ox, oy, oz = output['x'], output['y'], output['z']
        kaxpy(ox.kdata, Yz, Xy, False)
        kaxpy(ox.kdata, Yy, -Xz, True)
        kaxpy(oy.kdata, Yx, Xz, False)
        kaxpy(oy.kdata, Yz, -Xx, True)
        kaxpy(oz.kdata, Yy, Xx, False)
        kaxpy(oz.kdata, Yx, -Xy, True)
        for o in (ox, oy, oz):
            _kset(o)

    def XcrossY(self, X, Y, output):
        # physics.py:309-354 (grid points)
        if self.ndim == 2:
            Yx, Yy = xval(Y['x']), xval(Y['y'])
            if X.ncomp == 1:
                Xz = xval(X.components[0])
                ox, oy = output['x'], output['y']
                xfma(ox.xdata, Xz, Yy, -1.0, False)
                xfma(oy.xdata, Xz, Yx, 1.0, False)
                _xset(ox)
                _xset(oy)
            else:
                Xx, Xy = xval(X['x']), xval(X['y'])
                o = output.components[0]
                xfma(o.xdata, Xx, Yy, 1.0, False)
                xfma(o.xdata, Xy, Yx, -1.0, True)
                _xset(o)
            return
        Xx, Xy, Xz = xval(X['x']), xval(X['y']), xval(X['z'])
        Yx, Yy, Yz = xval(Y['x']), xval(Y['y']), xval(Y['z'])
        ox, oy, oz = output['x'], output['y'], output['z']
        xfma(ox.xdata, Xy, Yz, 1.0, False)
        xfma(ox.xdata, Xz, Yy, -1.0, True)
        xfma(oy.xdata, Xz, Yx, 1.0, False)
        xfma(oy.xdata, Xx, Yz, -1.0, True)
        xfma(oz.xdata, Xx, Yy, 1.0, False)
        xfma(oz.xdata, Xy, Yx, -1.0, True)
        for o in (ox, oy, oz):
            _xset(o)

    def curlX(self, X, output):
        # physics.py:374-405
        N = X.ncomp
        t = self._trans
        if N == 3:
            pairs = [(2, 1, 1, 2), (0, 2, 2, 0), (1, 0, 0, 1)]
            for o, (a, da, b, db) in enumerate(pairs):
                out = output[o]
                kaxpy(out.kdata, X[a].deriv(t[da]), 1.0, False)
                kaxpy(out.kdata, X[b].deriv(t[db]), -1.0, True)
                _kset(out)
        elif N == 2:
            out = output.components[0]
            kaxpy(out.kdata, X[1].deriv(t[0]), 1.0, False)
            kaxpy(out.kdata, X[0].deriv(t[1]), -1.0, True)
            _kset(out)
        elif N == 1:
            c = X.components[0]
            kaxpy(output[0].kdata, c.deriv(t[1]), 1.0, False)
            _kset(output[0])
            kaxpy(output[1].kdata, c.deriv(t[0]), -1.0, False)
            _kset(output[1])

    def laplace_solve(self, X, output):
        # physics.py:407-416 (k^2 cached at the first call unless laplace_k2 = 'current')
        out = output.components[0]
        if self.laplace_k2 == 'current':
            k2 = out.k2(no_zero=True)
        else:
            if self.k2 is None:
                self.k2 = out.k2(no_zero=True)
            k2 = self.k2
        kreal(out.kdata, kval(X.components[0]), k2, -1.0, 0, False)
        _kset(out)

    def pressure_projection(self, data, deriv):
        # physics.py:588-599
        mathscalar = self.aux_fields['mathscalar']
        S = self.parameters['shear_rate']
        self.divX(deriv['u'], mathscalar)
        if self._shear:
            ms = mathscalar.components[0]
            kaxpy(kval(ms), data['u']['y'].deriv('x'), -S, True)
        self.laplace_solve(mathscalar, mathscalar)
        ms = mathscalar.components[0]
        for i in self.dims:
            d = ms.deriv(self._trans[i])
            kaxpy(kval(deriv['u'][i]), d, -1.0, True)
            _kset(deriv['u'][i])

    # ------------------------------------------------- right-hand sides
    def _generic_if(self, deriv):
        if self._first_rhs or not hasattr(next(iter(deriv.fields.values()))[0], 'integrating_factor'):
            self._setup_integrating_factors(deriv)
            self._first_rhs = False

    def _generic_hydro(self, data, deriv, project):
        """IncompressibleHydro.RHS (physics.py:527-586); tracer and forcing are
        refused by _finalize."""
        self._generic_if(deriv)
        self._base_rhs(data, deriv)
        mathscalar = self.aux_fields['mathscalar']
        mathvector = self.aux_fields['mathvector']
        S = self.parameters['shear_rate']
        Omega = self.parameters['Omega']
        self.XgradY(data['u'], data['u'], mathscalar, mathvector, deriv['u'])
        for i in self.dims:
            c = deriv['u'][i]
            kaxpy(kval(c), c.kdata, -1.0, False)
            _kset(c)
        if self._shear:
            kaxpy(kval(deriv['u']['x']), kval(data['u']['y']), -S, True)
        if self._rotation:
            self.XconstcrossY(Omega, data['u'], mathvector)
            for i in self.dims:
                kaxpy(kval(deriv['u'][i]), kval(mathvector[i]), -2.0, True)
        if project:
            self.pressure_projection(data, deriv)
        if self._shear:
            self._setup_integrating_factors(deriv)

    def _generic_boussinesq(self, data, deriv):
        """BoussinesqHydro.RHS (physics.py:664-712)."""
        self._generic_hydro(data, deriv, project=False)
        mathscalar = self.aux_fields['mathscalar']
        mathvector = self.aux_fields['mathvector']
        g = self.parameters['g']
        alpha_t = self.parameters['alpha_t']
        beta = self.parameters['beta']
        direction = self.parameters['boussinesq_direction']
        ms = mathscalar.components[0]
        ms['kspace'] = kval(data['T'].components[0])
        kaxpy(ms.kdata, ms.kdata, g, False)
        kaxpy(ms.kdata, ms.kdata, alpha_t, False)
        kaxpy(kval(deriv['u'][direction]), ms.kdata, 1.0, True)
        self.pressure_projection(data, deriv)
        self.XgradY(data['u'], data['T'], mathscalar, mathvector, deriv['T'])
        dT = deriv['T'].components[0]
        kaxpy(kval(dT), dT.kdata, -1.0, False)
        _kset(dT)
        ms['kspace'] = kval(data['u'][direction])
        kaxpy(ms.kdata, ms.kdata, beta, False)
        kaxpy(dT.kdata, ms.kdata, -1.0, True)

    def _generic_mhd(self, data, deriv):
        """IncompressibleMHD.RHS (physics.py:770-819)."""
        self._generic_hydro(data, deriv, project=False)
        mathscalar = self.aux_fields['mathscalar']
        mathvector = self.aux_fields['mathvector']
        mathvector2 = self.aux_fields['mathvector2']
        S = self.parameters['shear_rate']
        fpr = 4 * np.pi * self.parameters['rho0']
        if self.ndim == 2:
            self.curlX(data['B'], mathscalar)
            self.XcrossY(mathscalar, data['B'], mathvector2)
        else:
            self.curlX(data['B'], mathvector)
            self.XcrossY(mathvector, data['B'], mathvector2)
        for i in self.dims:
            # numpy's complex / real scalar multiplies by the rounded 1 / fpr
            kaxpy(kval(deriv['u'][i]), kval(mathvector2[i]), 1.0 / fpr, True)
        self.pressure_projection(data, deriv)
        if self.ndim == 2:
            self.XcrossY(data['u'], data['B'], mathscalar)
            self.curlX(mathscalar, deriv['B'])
        else:
            self.XcrossY(data['u'], data['B'], mathvector)
            self.curlX(mathvector, deriv['B'])
        if self._shear:
            kaxpy(kval(deriv['B']['x']), kval(data['B']['y']), S, True)
