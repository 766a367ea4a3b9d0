"""Golden fixtures from the reference's own Python code, executed here.

Test infrastructure only (nothing in the product imports this file).  The
oracle restates the reference's Python layer -- representation, fields,
physics, time integrators -- by reading it; this script pins that reading by
running the reference itself on small cases and storing what it computes.

How the reference is made to run under Python 3 (it is Python 2 code):

1. The hot-path modules and the small modules they import are copied from the
   read-only reference checkout into a temporary package tree (never into
   this repository): ``dedalus/config.py``, ``dedalus/utils/{parallelism,
   logger,timer,function_count}.py``, ``dedalus/data_objects/{fields,
   representations,state_data,aux_equation,api}.py``,
   ``dedalus/physics/{physics,api}.py``, ``dedalus/time_stepping/
   {time_step,api}.py``.
2. Only mechanical Python 2 -> 3 rewrites are applied (``GENERIC`` and
   ``SPECIFIC`` below): print statements, ``xrange``, ``iteritems``,
   ``has_key``, ``except X, e``, ``func_name``, ``cPickle`` / ``ConfigParser`` module names,
   ``== None`` / ``!= None`` (numpy arrays no longer compare to None as one
   bool), implicit relative imports, ``keys()[0]`` / ``zip(...)`` indexing,
   the integer divisions that Python 2 performed on integer shapes, indexing
   with a list of slices, and numpy 2's removal of ``asfarray`` (each
   specific one listed with the reference line it touches).
3. One correction of the reference's own code (``CORRECTIONS`` below): its
   numpy backend of the shearing box scales the wrong array after the inverse
   transform (representations.py:740), so that backend is brought to what the
   FFTW backend computes.
4. Modules that are absent here or unrelated to the arithmetic are stubbed:
   the FFTW wrapper (``dedalus/utils/fftw``; FFT.method = numpy is selected,
   the reference's own alternative backend, ``representations.py:327-333``),
   ``h5py`` (snapshots only), ``dedalus/funcs.py`` (IPython / Mercurial
   helpers) and ``dedalus/utils/api.py`` (re-exports only the timer and the
   parallel helpers).  mpi4py is absent, so the reference runs serially, as
   its ``CommunicationSystem`` allows (``utils/parallelism.py:28-50``).
5. The Cython stage and dealias kernels are the reference's own, compiled
   from their ``.pyx`` sources by ``oracle/build_ref.py`` into ``oracle/_ref``
   (the reference imports them by bare module name).

Cases (inputs seeded with numpy PCG64; all fields are real by construction:
drawn in grid space and transformed with the reference's own forward
transform): one ``RHS`` call and two or three ``RK2mid`` steps each of 2D
hydro 32^2, 3D hydro 16^3, 2D Boussinesq 32^2 (direction y), 3D Boussinesq
16^3 (direction z), 3D MHD 16^3 and 2D MHD 32^2, two ``RK2trap`` steps of 3D
hydro 16x8x32 and of 2D Boussinesq 32^2, in the shearing box
(``FourierShearRepresentation``) one RHS call and two steps each of 2D and 3D
hydro, 2D Boussinesq and 2D MHD (RK2trap), with rotation 2D and 3D hydro and,
in the shearing box, 3D hydro and 3D Boussinesq, in boxes whose sides are not
2 pi 3D hydro (anisotropic, hyperviscous), 3D MHD and 2D Boussinesq, and
``compute_dt`` for each.
Outputs go to ``tests/golden/ref_<case>.npz``.  The reference's RK4 cannot
run (``RKBase.forward_step`` calls methods defined nowhere,
``time_step.py:209-218``), so no fixture exists for it.

Run (in the development container, where the reference checkout, Cython and
``oracle/_ref`` exist): ``python oracle/ref_fixtures.py [reference_root]``.
"""
import os
import re
import shutil
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
GOLDEN = os.path.join(ROOT, "tests", "golden")

COPY = [
    "dedalus/config.py",
    "dedalus/utils/parallelism.py",
    "dedalus/utils/logger.py",
    "dedalus/utils/timer.py",
    "dedalus/utils/function_count.py",
    "dedalus/data_objects/api.py",
    "dedalus/data_objects/aux_equation.py",
    "dedalus/data_objects/fields.py",
    "dedalus/data_objects/representations.py",
    "dedalus/data_objects/state_data.py",
    "dedalus/physics/api.py",
    "dedalus/physics/physics.py",
    "dedalus/time_stepping/api.py",
    "dedalus/time_stepping/time_step.py",
]

# (pattern, replacement) applied to every copied file, in order.
GENERIC = [
    (r"^(\s*)print\s*$", r"\1print()"),
    (r"^(\s*)print\s+(?![(=])(.+)$", r"\1print(\2)"),
    (r"\bxrange\(", "range("),
    (r"\.iteritems\(\)", ".items()"),
    (r"([\w\.\[\]'\"]+)\.has_key\(([^()]*)\)", r"(\2 in \1)"),
    (r"except\s+(\w+)\s*,\s*(\w+)\s*:", r"except \1 as \2:"),
    (r"^import cPickle$", "import pickle as cPickle"),
    (r"^import ConfigParser$", "import configparser as ConfigParser"),
    (r"\s==\s*None\b", " is None"),
    (r"\s!=\s*None\b", " is not None"),
    (r"^from (fields|state_data|representations|aux_equation|time_step|physics) import",
     r"from .\1 import"),
    (r"([\w\.]+)\.keys\(\)\[0\]", r"list(\1.keys())[0]"),
    (r"\.func_name\b", ".__name__"),
    # numpy 2 removed asfarray
    (r"np\.asfarray\(([^()]*)\)", r"np.asarray(\1, dtype=np.float64)"),
]

# (file, exact old text, new text, reference line): integer arithmetic that
# Python 2 did with "/" on integers, zip results that are indexed, and
# indexing with a list of slices (a tuple is required since numpy 1.23).
SPECIFIC = [
    ("dedalus/data_objects/representations.py", "sli = [slice(i) for i in self.data.shape]",
     "sli = tuple(slice(i) for i in self.data.shape)", 163),
    ("dedalus/data_objects/representations.py",
     "self.global_shape['kspace'][-1]  = self.global_shape['kspace'][-1] / 2 + 1",
     "self.global_shape['kspace'][-1]  = self.global_shape['kspace'][-1] // 2 + 1", 175),
    ("dedalus/data_objects/representations.py", "ki[ksize / 2] *= -1.", "ki[ksize // 2] *= -1.", 226),
    ("dedalus/data_objects/representations.py", "index = zip(*test.nonzero())",
     "index = list(zip(*test.nonzero()))", 281),
    ("dedalus/data_objects/representations.py", "nyindex = self.local_shape['kspace'][1] / 2",
     "nyindex = self.local_shape['kspace'][1] // 2", 474),
    ("dedalus/data_objects/representations.py", "nyy, nyz = np.array(plane_data.shape) / 2",
     "nyy, nyz = np.array(plane_data.shape) // 2", 484),
    ("dedalus/data_objects/representations.py", "mshape[-1] = mshape[-1] / 2 + 1",
     "mshape[-1] = mshape[-1] // 2 + 1", 624),
    ("dedalus/data_objects/representations.py", "gmshape[-1] = gmshape[-1] / 2 + 1",
     "gmshape[-1] = gmshape[-1] // 2 + 1", 646),
    # np.ogrid now returns a tuple (a list in the numpy of the reference's time),
    # which the next line assigns into; and the slices must be a tuple
    ("dedalus/data_objects/representations.py",
     "grid = refgrid[[slice(i) for i in np.asarray(self.local_shape['xspace'], dtype=np.float64)]]",
     "grid = refgrid[tuple(slice(i) for i in np.asarray(self.local_shape['xspace'], dtype=np.float64))]\n"
     "        if open:\n            grid = list(grid)", 539),
]

# (file, exact old text, new text, reference line): corrections of the
# reference's own code, not Python 2 -> 3 rewrites.  Each makes the numpy
# backend (the only one that runs here) do what the reference's FFTW backend,
# the one its runs use, does.
#  * FourierShearRepresentation.rev_np scales kdata by N after the inverse
#    transforms where the x-space result needs it (the plain representation's
#    rev_np scales its x-space result, representations.py:333; the FFTW
#    backend's rev_fftw is unnormalised and needs no scale): as written the
#    shearing box's x-space values come out N times too small.
CORRECTIONS = [
    ("dedalus/data_objects/representations.py", "        self.kdata *= self.global_shape['xspace'].prod()",
     "        self.xdata *= self.global_shape['xspace'].prod()", 740),
]

STUBS = {
    "dedalus/__init__.py": "",
    "dedalus/utils/__init__.py": "",
    "dedalus/data_objects/__init__.py": "",
    "dedalus/physics/__init__.py": "",
    "dedalus/time_stepping/__init__.py": "",
    "dedalus/utils/fftw/__init__.py": "fftw = None  # FFTW is absent; FFT.method = numpy is used\n",
    "dedalus/utils/api.py": ("from .timer import Timer, timer\n"
                             "from .parallelism import com_sys, load_all, swap_indices\n"),
    "dedalus/funcs.py": ("def insert_ipython(num_up=1):\n    raise NotImplementedError\n\n\n"
                         "def get_mercurial_changeset_id():\n    return 'unknown'\n"),
    "h5py.py": "# snapshots are not exercised\n",
}


def convert(text, rel):
    lines = text.split("\n")
    out = []
    for ln in lines:
        for pat, rep in GENERIC:
            ln = re.sub(pat, rep, ln)
        out.append(ln)
    text = "\n".join(out)
    for f, old, new, line in SPECIFIC + CORRECTIONS:
        if f == rel:
            if text.count(old) != 1:
                raise RuntimeError("%s:%d: expected text found %d times: %r" % (rel, line, text.count(old), old))
            text = text.replace(old, new)
    return text


def make_tree(ref_root, dst):
    for rel, body in STUBS.items():
        p = os.path.join(dst, rel)
        os.makedirs(os.path.dirname(p), exist_ok=True)
        with open(p, "w") as f:
            f.write(body)
    for rel in COPY:
        with open(os.path.join(ref_root, rel)) as f:
            text = f.read()
        p = os.path.join(dst, rel)
        os.makedirs(os.path.dirname(p), exist_ok=True)
        with open(p, "w") as f:
            f.write(convert(text, rel))


def import_reference(ref_root):
    """Build the converted tree in a temporary directory and import it.
    Returns (tmpdir, module dict)."""
    ref_dir = os.path.join(HERE, "_ref")
    if not os.path.isdir(ref_dir):
        raise RuntimeError("oracle/_ref is missing: run oracle/build_ref.py first")
    tmp = tempfile.mkdtemp(prefix="dd_ref_py3_")
    make_tree(ref_root, tmp)
    sys.path.insert(0, tmp)
    sys.path.insert(0, ref_dir)          # the reference's compiled Cython kernels, by bare name
    import importlib
    cfg = importlib.import_module("dedalus.config")
    cfg.decfg.set('FFT', 'method', 'numpy')
    cfg.decfg.set('utils', 'loglevel', 'warning')
    mods = {
        "config": cfg,
        "representations": importlib.import_module("dedalus.data_objects.representations"),
        "physics": importlib.import_module("dedalus.physics.physics"),
        "time_step": importlib.import_module("dedalus.time_stepping.time_step"),
    }
    return tmp, mods


def seed_state(rng, RHS, data, names, amp=1.0):
    """Fill data[f][c] with smooth real random fields through the reference's
    own x -> k path (``__setitem__('xspace')`` then ``['kspace']``)."""
    for f, c in names:
        comp = data[f][c]
        x = rng.standard_normal(tuple(comp.global_shape['xspace']))
        comp['xspace'] = x
        k = comp['kspace']
        kk = sum(comp.k[d] ** 2 for d in comp.k if isinstance(d, str))
        k *= np.exp(-0.35 * kk)
        k *= amp / max(np.sqrt(np.sum(np.abs(k) ** 2)), 1e-300)
        comp['kspace'] = k.copy()


def _state(data, names):
    return {"%s%d" % (f, c): data[f][c]['kspace'].copy() for f, c in names}


def run_case(mods, name, cls, shape, params, names, integrator, nsteps, dt, seed,
             rep_name="FourierRepresentation", length=None):
    P, T = mods["physics"], mods["time_step"]
    rep = getattr(mods["representations"], rep_name)
    rng = np.random.Generator(np.random.PCG64(seed))
    RHS = getattr(P, cls)(shape, rep, length=length)
    RHS.parameters.update(params)
    data = RHS.create_fields(0.)
    seed_state(rng, RHS, data, names)
    import platform
    out = {"numpy_version": np.__version__, "machine": platform.machine(),
           "shape": np.array(shape), "dt": dt, "nsteps": nsteps, "cls": cls, "integrator": integrator,
           "params": repr(sorted(params.items())), "names": np.array(["%s%d" % n for n in names]),
           "rep": rep_name, "length": np.array(length if length is not None else [2 * np.pi] * len(shape))}
    for key, v in _state(data, names).items():
        out["in_" + key] = v
    # one RHS call on the input state
    deriv = RHS.create_fields(0.)
    RHS.RHS(data, deriv)
    for key, v in _state(deriv, names).items():
        out["rhs_" + key] = v
    # a fresh physics object and state for the integrator: the integrating
    # factors are attached to the derivative fields of the first RHS call
    # (physics.py:573-574), which must be the integrator's own
    RHS = getattr(P, cls)(shape, rep, length=length)
    RHS.parameters.update(params)
    data = RHS.create_fields(0.)
    for (f, c) in names:
        data[f][c]['kspace'] = out["in_%s%d" % (f, c)].copy()
    ti = getattr(T, integrator)(RHS)
    for s in range(nsteps):
        ti.do_advance(data, dt)
        for key, v in _state(data, names).items():
            out["step%d_%s" % (s + 1, key)] = v
    # CFL dt of the final state (leaves the velocity in x space: last)
    out["compute_dt"] = float(RHS.compute_dt(data))
    out["dtlist"] = np.array(RHS.dtlist, dtype=np.float64)
    return out


CASES = [
    # name, physics class, shape, parameters, state fields, integrator, steps, dt, seed
    ("hydro2d_32", "IncompressibleHydro", (32, 32), {'nu': 1e-3}, [('u', 0), ('u', 1)], "RK2mid", 3, 1e-2, 1),
    ("hydro3d_16", "IncompressibleHydro", (16, 16, 16), {'nu': 5e-3}, [('u', 0), ('u', 1), ('u', 2)],
     "RK2mid", 3, 1e-2, 2),
    ("hydro3d_16x8x32_trap", "IncompressibleHydro", (16, 8, 32), {'nu': 2e-2}, [('u', 0), ('u', 1), ('u', 2)],
     "RK2trap", 2, 1e-2, 3),
    ("bouss2d_32", "BoussinesqHydro", (32, 32),
     {'nu': 2e-3, 'kappa': 3e-3, 'g': 1., 'alpha_t': 1., 'beta': 1., 'boussinesq_direction': 'y'},
     [('u', 0), ('u', 1), ('T', 0)], "RK2mid", 3, 1e-2, 4),
    ("mhd3d_16", "IncompressibleMHD", (16, 16, 16), {'nu': 5e-3, 'eta': 8e-3, 'rho0': 1.5},
     [('u', 0), ('u', 1), ('u', 2), ('B', 0), ('B', 1), ('B', 2)], "RK2mid", 2, 1e-2, 5),
    ("bouss3d_16", "BoussinesqHydro", (16, 16, 16),
     {'nu': 4e-3, 'kappa': 6e-3, 'g': 1.5, 'alpha_t': 0.8, 'beta': 1.2},
     [('u', 0), ('u', 1), ('u', 2), ('T', 0)], "RK2mid", 2, 1e-2, 6),
    ("mhd2d_32", "IncompressibleMHD", (32, 32), {'nu': 3e-3, 'eta': 5e-3},
     [('u', 0), ('u', 1), ('B', 0), ('B', 1)], "RK2mid", 2, 1e-2, 7),
    ("bouss2d_32_trap", "BoussinesqHydro", (32, 32),
     {'nu': 2e-3, 'kappa': 2e-3, 'g': 1., 'alpha_t': 1., 'beta': 1., 'boussinesq_direction': 'y'},
     [('u', 0), ('u', 1), ('T', 0)], "RK2trap", 2, 1e-2, 8),
    # the shearing box (representations.py:558-740, physics.py shear branches)
    ("shear_hydro2d_32", "IncompressibleHydro", (32, 32), {'nu': 1e-2, 'shear_rate': 1.0},
     [('u', 0), ('u', 1)], "RK2mid", 2, 1e-2, 11, "FourierShearRepresentation"),
    ("shear_hydro3d_16", "IncompressibleHydro", (16, 16, 16), {'nu': 1e-2, 'shear_rate': 1.5},
     [('u', 0), ('u', 1), ('u', 2)], "RK2mid", 2, 1e-2, 12, "FourierShearRepresentation"),
    ("shear_bouss2d_32", "BoussinesqHydro", (32, 32),
     {'nu': 2e-3, 'kappa': 2e-3, 'g': 1., 'alpha_t': 1., 'beta': 1., 'boussinesq_direction': 'y',
      'shear_rate': 1.0},
     [('u', 0), ('u', 1), ('T', 0)], "RK2mid", 2, 1e-2, 13, "FourierShearRepresentation"),
    ("shear_mhd2d_32", "IncompressibleMHD", (32, 32), {'nu': 5e-3, 'eta': 5e-3, 'shear_rate': 0.8},
     [('u', 0), ('u', 1), ('B', 0), ('B', 1)], "RK2trap", 2, 1e-2, 14, "FourierShearRepresentation"),
    # rotation (Omega = (Omega_z, Omega_y, Omega_x) in 3D, a scalar in 2D; physics.py:551-565)
    ("rot_hydro3d_16", "IncompressibleHydro", (16, 16, 16), {'nu': 1e-2, 'Omega': [0.7, -0.2, 0.3]},
     [('u', 0), ('u', 1), ('u', 2)], "RK2mid", 2, 1e-2, 15),
    ("rot_hydro2d_32", "IncompressibleHydro", (32, 32), {'nu': 1e-2, 'Omega': 0.8},
     [('u', 0), ('u', 1)], "RK2mid", 2, 1e-2, 16),
    ("shear_rot_hydro3d_16", "IncompressibleHydro", (16, 16, 16),
     {'nu': 1e-2, 'shear_rate': 1.5, 'Omega': [1.0, 0.0, 0.0]},
     [('u', 0), ('u', 1), ('u', 2)], "RK2mid", 2, 1e-2, 17, "FourierShearRepresentation"),
    ("shear_rot_bouss3d_16", "BoussinesqHydro", (16, 16, 16),
     {'nu': 2e-3, 'kappa': 2e-3, 'g': 1., 'alpha_t': 1., 'beta': 1., 'shear_rate': 1.2,
      'Omega': [1.0, 0.0, 0.0]},
     [('u', 0), ('u', 1), ('u', 2), ('T', 0)], "RK2mid", 2, 1e-2, 18, "FourierShearRepresentation"),
    # boxes whose sides are not 2 pi (non-integer wavenumbers) and hyperviscosity
    ("box_hydro3d_16x16x32_vo2", "IncompressibleHydro", (16, 16, 32), {'nu': 2e-4, 'viscosity_order': 2},
     [('u', 0), ('u', 1), ('u', 2)], "RK2mid", 2, 1e-2, 19, "FourierRepresentation", (3.0, 5.0, 7.0)),
    ("box_mhd3d_16", "IncompressibleMHD", (16, 16, 16), {'nu': 5e-3, 'eta': 7e-3},
     [('u', 0), ('u', 1), ('u', 2), ('B', 0), ('B', 1), ('B', 2)], "RK2mid", 2, 1e-2, 20,
     "FourierRepresentation", (4.0, 4.0, 4.0)),
    ("box_bouss2d_32", "BoussinesqHydro", (32, 32),
     {'nu': 2e-3, 'kappa': 2e-3, 'g': 1., 'alpha_t': 1., 'beta': 1., 'boussinesq_direction': 'y'},
     [('u', 0), ('u', 1), ('T', 0)], "RK2mid", 2, 1e-2, 21, "FourierRepresentation", (2 * np.pi, 4.0)),
]


def main(ref_root="/root/reference"):
    from oracle import build_ref
    build_ref.build(ref_root)
    tmp, mods = import_reference(ref_root)
    try:
        os.makedirs(GOLDEN, exist_ok=True)
        for case in CASES:
            name = case[0]
            out = run_case(mods, *case)
            path = os.path.join(GOLDEN, "ref_%s.npz" % name)
            np.savez_compressed(path, **out)
            print("wrote %s (compute_dt %.6e)" % (os.path.relpath(path, ROOT), out["compute_dt"]))
    finally:
        shutil.rmtree(tmp, ignore_errors=True)


if __name__ == "__main__":
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
