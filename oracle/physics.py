"""CPU oracle -- test infrastructure only.

Restatement of the reference's physics classes
(``dedalus/physics/physics.py``): the ``Physics`` base (RHS zeroing, operator
helpers ``divX`` 180, ``XgradY`` 197, ``XcrossY`` 309, ``curlX`` 374,
``laplace_solve`` 407), ``IncompressibleHydro`` 419-610,
``BoussinesqHydro`` 612-721 and ``IncompressibleMHD`` 724-836.  The operator
algebra, its order and its lazy x/k-space transforms are kept exactly,
including the MHD state round trip through x-space.  Fixed: ``== None`` on
arrays (physics.py:412, 497) is written ``is None``.  Shear, rotation,
tracer and forcing branches are kept as written.
"""
import numpy as np

from .fields import create_field_classes, StateData
from .representation import decfg


class Physics:
    """physics.py:42-416."""

    def __init__(self, shape, representation, length=None):
        self.shape = shape
        self._representation = representation
        if length:
            self.length = length
        else:
            self.length = (2 * np.pi,) * len(self.shape)
        self.ndim = len(self.shape)
        self.dims = range(self.ndim)
        self._field_list = []
        self._aux_field_list = []
        self.parameters = {}
        self.aux_eqns = {}
        self.forcing_functions = {}
        self._forcing_function_names = {}
        self._field_classes = create_field_classes(self._representation, self.shape, self.length)
        self._is_finalized = False
        self._tracer = decfg.getboolean('physics', 'use_tracer')
        self.k2 = None

    def __getitem__(self, item):
        value = self.parameters.get(item, None)
        if value is None:
            raise KeyError
        return value

    def _finalize(self):
        self._setup_aux_fields(0., self._aux_field_list)
        self._is_finalized = True

    def create_fields(self, time, field_list=None):
        if field_list is None:
            field_list = self._field_list
        return StateData(time, self.shape, self.length, self._field_classes,
                         field_list=field_list, params=self.parameters)

    def _setup_aux_fields(self, t, aux_field_list=None):
        self.aux_fields = self.create_fields(t, aux_field_list)

    def RHS(self, data, deriv):
        # physics.py:134-149
        if not self._is_finalized:
            self._finalize()
        for fname, field in deriv:
            field.zero_all()
        for fname, field in self.aux_fields:
            field.zero_all(space='kspace')
        deriv.set_time(data.time)
        self.aux_fields.set_time(data.time)

    def compute_dt(self, data):
        self.dtlist = []
        self.set_dtlist(data)
        return min(self.dtlist)

    def divX(self, X, output):
        # physics.py:180-195
        output.zero()
        for i in range(X.ncomp):
            output['kspace'] += X[i].deriv(self._trans[i])

    def XgradY(self, X, Y, stmp, vtmp, output):
        # physics.py:197-228
        output.zero_all('xspace')
        for cindex, comp in X:
            vtmp[cindex]['kspace'] = comp['kspace']
        for cindex, comp in Y:
            for i in self.dims:
                stmp['kspace'] = comp.deriv(self._trans[i])
                stmp['xspace'] *= vtmp[i]['xspace']
                output[cindex]['xspace'] += stmp['xspace']

    def XconstcrossY(self, X, Y, output):
        # physics.py:266-307
        if self.ndim == 2:
            if np.isscalar(X):
                Xz = X
            else:
                Xy, Xx = X
        else:
            Xz, Xy, Xx = X
        Yx = Y['x']['kspace']
        Yy = Y['y']['kspace']
        if self.ndim == 3:
            Yz = Y['z']['kspace']
        if self.ndim == 2:
            if np.isscalar(X):
                output['x']['kspace'] = - Xz * Yy
                output['y']['kspace'] = Xz * Yx
            else:
                output['kspace'] = Xx * Yy - Xy * Yx
        else:
            output['x']['kspace'] = Xy * Yz - Xz * Yy
            output['y']['kspace'] = Xz * Yx - Xx * Yz
            output['z']['kspace'] = Xx * Yy - Xy * Yx

    def XcrossY(self, X, Y, output):
        # physics.py:309-354
        if self.ndim == 2:
            if X.ncomp == 1:
                Xz = X['xspace']
            else:
                Xx = X['x']['xspace']
                Xy = X['y']['xspace']
        else:
            Xx = X['x']['xspace']
            Xy = X['y']['xspace']
            Xz = X['z']['xspace']
        Yx = Y['x']['xspace']
        Yy = Y['y']['xspace']
        if self.ndim == 3:
            Yz = Y['z']['xspace']
        if self.ndim == 2:
            if X.ncomp == 1:
                output['x']['xspace'] = - Xz * Yy
                output['y']['xspace'] = Xz * Yx
            else:
                output['xspace'] = Xx * Yy - Xy * Yx
        else:
            output['x']['xspace'] = Xy * Yz - Xz * Yy
            output['y']['xspace'] = Xz * Yx - Xx * Yz
            output['z']['xspace'] = Xx * Yy - Xy * Yx

    def curlX(self, X, output):
        # physics.py:374-405
        N = X.ncomp
        if N == 3:
            output[0]['kspace'] = X[2].deriv(self._trans[1]) - X[1].deriv(self._trans[2])
            output[1]['kspace'] = X[0].deriv(self._trans[2]) - X[2].deriv(self._trans[0])
            output[2]['kspace'] = X[1].deriv(self._trans[0]) - X[0].deriv(self._trans[1])
        elif N == 2:
            output['kspace'] = X[1].deriv(self._trans[0]) - X[0].deriv(self._trans[1])
        elif N == 1:
            output[0]['kspace'] = X[0].deriv(self._trans[1])
            output[1]['kspace'] = -X[0].deriv(self._trans[0])

    # physics.py:412-413 caches k^2 at the first call, which a shearing box
    # then keeps using; 'current' (test use only) divides by the k^2 of the
    # call's time instead.
    laplace_k2 = 'cached'

    def laplace_solve(self, X, output):
        # physics.py:407-416
        if self.laplace_k2 == 'current':
            k2 = output.k2(no_zero=True)
        else:
            if self.k2 is None:
                self.k2 = output.k2(no_zero=True)
            k2 = self.k2
        output['kspace'] = X['kspace']
        output['kspace'] /= k2
        output['kspace'] *= -1.


class IncompressibleHydro(Physics):
    """physics.py:419-610."""

    def __init__(self, *args, **kwargs):
        Physics.__init__(self, *args, **kwargs)
        self._field_list.append(('u', 'VectorField'))
        self._aux_field_list.append(('mathscalar', 'ScalarField'))
        self._aux_field_list.append(('mathvector', 'VectorField'))
        self.parameters['viscosity_order'] = 1
        self.parameters['nu'] = 0.
        self.parameters['shear_rate'] = 0.
        self.parameters['Omega'] = None
        if self._tracer:
            self._field_list.append(('c', 'ScalarField'))
            self.parameters['c_diff'] = 0.
        self._trans = {0: 'x', 1: 'y', 2: 'z'}
        self._first_rhs = True

    def _finalize(self):
        Physics._finalize(self)
        if self.parameters['shear_rate'] == 0.:
            self._shear = False
        else:
            self._shear = True
            if self._representation._static_k:
                raise ValueError("A shearing representation must be used if shear_rate is nonzero.")
        self._rotation = self.parameters['Omega'] is not None

    def _setup_integrating_factors(self, deriv):
        # physics.py:504-522
        for cindex, comp in deriv['u']:
            nu = self.parameters['nu']
            vo = self.parameters['viscosity_order']
            if nu == 0.:
                comp.integrating_factor = None
            else:
                comp.integrating_factor = nu * comp.k2() ** vo
        if self._tracer:
            comp = deriv['c'][0]
            diff = self.parameters['c_diff']
            vo = self.parameters['viscosity_order']
            if diff == 0.:
                comp.integrating_factor = None
            else:
                comp.integrating_factor = diff * comp.k2() ** vo

    def set_velocity_forcing(self, func):
        self.forcing_functions['VelocityForcing'] = func

    def RHS(self, data, deriv):
        # physics.py:527-586
        if self._first_rhs:
            self._setup_integrating_factors(deriv)
            self._first_rhs = False
        Physics.RHS(self, data, deriv)
        mathscalar = self.aux_fields['mathscalar']
        mathvector = self.aux_fields['mathvector']
        S = self.parameters['shear_rate']
        Omega = self.parameters['Omega']
        self.XgradY(data['u'], data['u'], mathscalar, mathvector, deriv['u'])
        for i in self.dims:
            deriv['u'][i]['kspace'] *= -1.
        if self._shear:
            deriv['u']['x']['kspace'] -= S * data['u']['y']['kspace']
        if self._rotation:
            self.XconstcrossY(Omega, data['u'], mathvector)
            for i in self.dims:
                deriv['u'][i]['kspace'] -= 2 * mathvector[i]['kspace']
        if 'VelocityForcing' in self.forcing_functions:
            for i in self.dims:
                deriv['u'][i]['kspace'] += self.forcing_functions['VelocityForcing'](data, i)
        if self.__class__ == IncompressibleHydro:
            self.pressure_projection(data, deriv)
        if self._tracer:
            self.XgradY(data['u'], data['c'], mathscalar, mathvector, deriv['c'])
            deriv['c']['kspace'] *= -1
        if self._shear:
            self._setup_integrating_factors(deriv)

    def pressure_projection(self, data, deriv):
        # physics.py:588-599
        mathscalar = self.aux_fields['mathscalar']
        S = self.parameters['shear_rate']
        self.divX(deriv['u'], mathscalar)
        if self._shear:
            mathscalar['kspace'] -= S * data['u']['y'].deriv('x')
        self.laplace_solve(mathscalar, mathscalar)
        for i in self.dims:
            deriv['u'][i]['kspace'] -= mathscalar.deriv(self._trans[i])

    def max_abs_vel(self, data):
        return np.sqrt(data['u'].max_square())

    def set_dtlist(self, data):
        dx = data['u']['x'].dx().min()
        self.dtlist.append(dx / self.max_abs_vel(data))


class BoussinesqHydro(IncompressibleHydro):
    """physics.py:612-721."""

    def __init__(self, *args, **kwargs):
        IncompressibleHydro.__init__(self, *args, **kwargs)
        self._field_list.append(('T', 'ScalarField'))
        self.parameters['kappa'] = 0.
        self.parameters['g'] = 1.
        self.parameters['alpha_t'] = 1.
        self.parameters['beta'] = 1.
        self.parameters['boussinesq_direction'] = decfg.get('physics', 'boussinesq_direction')

    def _setup_integrating_factors(self, deriv):
        IncompressibleHydro._setup_integrating_factors(self, deriv)
        kappa = self.parameters['kappa']
        vo = self.parameters['viscosity_order']
        if kappa == 0.:
            deriv['T'][0].integrating_factor = None
        else:
            deriv['T'][0].integrating_factor = kappa * deriv['T'][0].k2() ** vo

    def set_thermal_forcing(self, func):
        self.forcing_functions['ThermalForcing'] = func

    def RHS(self, data, deriv):
        # physics.py:664-712
        IncompressibleHydro.RHS(self, data, deriv)
        mathscalar = self.aux_fields['mathscalar']
        mathvector = self.aux_fields['mathvector']
        g = self.parameters['g']
        alpha_t = self.parameters['alpha_t']
        beta = self.parameters['beta']
        direction = self.parameters['boussinesq_direction']
        mathscalar['kspace'] = data['T']['kspace']
        mathscalar['kspace'] *= g
        mathscalar['kspace'] *= alpha_t
        deriv['u'][direction]['kspace'] += mathscalar['kspace']
        if self.__class__ == BoussinesqHydro:
            self.pressure_projection(data, deriv)
        self.XgradY(data['u'], data['T'], mathscalar, mathvector, deriv['T'])
        deriv['T']['kspace'] *= -1.
        mathscalar['kspace'] = data['u'][direction]['kspace']
        mathscalar['kspace'] *= beta
        deriv['T']['kspace'] -= mathscalar['kspace']
        if 'ThermalForcing' in self.forcing_functions:
            deriv['T']['kspace'] += self.forcing_functions['ThermalForcing'](data)

    def set_dtlist(self, data):
        IncompressibleHydro.set_dtlist(self, data)
        dx = data['u']['x'].dx().min()
        N = np.sqrt(np.abs(self.parameters['alpha_t'] * self.parameters['g'] *
                           self.parameters['beta']))
        self.dtlist.append(dx / N)


class IncompressibleMHD(IncompressibleHydro):
    """physics.py:724-836."""

    def __init__(self, *args, **kwargs):
        IncompressibleHydro.__init__(self, *args, **kwargs)
        self._field_list.append(('B', 'VectorField'))
        self._aux_field_list.append(('mathvector2', 'VectorField'))
        self.parameters['rho0'] = 1.
        self.parameters['eta'] = 0.

    def _setup_integrating_factors(self, deriv):
        IncompressibleHydro._setup_integrating_factors(self, deriv)
        eta = self.parameters['eta']
        vo = self.parameters['viscosity_order']
        for cindex, comp in deriv['B']:
            if eta == 0.:
                comp.integrating_factor = None
            else:
                comp.integrating_factor = eta * comp.k2() ** vo

    def RHS(self, data, deriv):
        # physics.py:770-819
        IncompressibleHydro.RHS(self, data, deriv)
        mathscalar = self.aux_fields['mathscalar']
        mathvector = self.aux_fields['mathvector']
        mathvector2 = self.aux_fields['mathvector2']
        S = self.parameters['shear_rate']
        rho0 = self.parameters['rho0']
        fpr = 4 * np.pi * rho0
        if self.ndim == 2:
            self.curlX(data['B'], mathscalar)
            self.XcrossY(mathscalar, data['B'], mathvector2)
        else:
            self.curlX(data['B'], mathvector)
            self.XcrossY(mathvector, data['B'], mathvector2)
        for i in self.dims:
            deriv['u'][i]['kspace'] += mathvector2[i]['kspace'] / fpr
        if self.__class__ == IncompressibleMHD:
            self.pressure_projection(data, deriv)
        if self.ndim == 2:
            self.XcrossY(data['u'], data['B'], mathscalar)
            self.curlX(mathscalar, deriv['B'])
        else:
            self.XcrossY(data['u'], data['B'], mathvector)
            self.curlX(mathvector, deriv['B'])
        if self._shear:
            deriv['B']['x']['kspace'] += S * data['B']['y']['kspace']

    def max_alfven_speed(self, data):
        fpr = 4 * np.pi * self.parameters['rho0']
        return np.sqrt(data['B'].max_square() / fpr)

    def set_dtlist(self, data):
        IncompressibleHydro.set_dtlist(self, data)
        dx = data['u']['x'].dx().min()
        self.dtlist.append(dx / self.max_alfven_speed(data))
