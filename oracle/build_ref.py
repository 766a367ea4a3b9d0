"""Build recipe for ``oracle/_ref``: the reference's own Cython kernels, compiled
from their sources where they lie in the read-only reference checkout.

Test infrastructure only.  The four modules built here are the reference's
native hot-path kernels:

* ``dedalus/time_stepping/forward_step_cy_2d.pyx`` / ``forward_step_cy_3d.pyx``
  (``euler``, ``etd1``, ``etd2rk1``, ``etd2rk2``; reference ``setup.py:127-128``)
* ``dedalus/data_objects/dealias_cy_2d.pyx`` / ``dealias_cy_3d.pyx``
  (``dealias_23``; reference ``setup.py:125-126``)

They are compiled with Cython (``language_level=2``, as the reference's
Python 2 build did) and gcc.  Generated C and the shared objects go only to
``oracle/_ref/`` (git-ignored).  Nothing is copied into the repository.  The
recipe needs Cython, which exists in the development container but not on
the GPU host, so on the GPU host ``oracle/_ref`` is simply absent and the tests
that compare against it are skipped there.

Run: ``python oracle/build_ref.py [reference_root]``.
"""
import os
import subprocess
import sys
import sysconfig

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
MODULES = {
    "forward_step_cy_2d": "dedalus/time_stepping/forward_step_cy_2d.pyx",
    "forward_step_cy_3d": "dedalus/time_stepping/forward_step_cy_3d.pyx",
    "dealias_cy_2d": "dedalus/data_objects/dealias_cy_2d.pyx",
    "dealias_cy_3d": "dedalus/data_objects/dealias_cy_3d.pyx",
}


def build(ref_root="/root/reference", quiet=True):
    """Compile the reference Cython kernels into ``oracle/_ref``.

    Returns the list of built module names; returns an empty list when the
    reference checkout or Cython is unavailable (this is not an error: the
    C restatement in ``oracle/stage.c`` is the oracle; these modules only pin
    it).
    """
    if not os.path.isdir(ref_root):
        return []
    try:
        import Cython  # noqa: F401
        import numpy as np
    except ImportError:
        return []
    os.makedirs(OUT, exist_ok=True)
    ext = sysconfig.get_config_var("EXT_SUFFIX")
    py_inc = sysconfig.get_paths()["include"]
    built = []
    for name, rel in MODULES.items():
        src = os.path.join(ref_root, rel)
        if not os.path.isfile(src):
            continue
        c_out = os.path.join(OUT, name + ".c")
        so_out = os.path.join(OUT, name + ext)
        if os.path.isfile(so_out) and os.path.getmtime(so_out) >= os.path.getmtime(src):
            built.append(name)
            continue
        subprocess.check_call(
            [sys.executable, "-m", "cython", "-2", "-o", c_out, src],
            stdout=subprocess.DEVNULL if quiet else None)
        # Same floating-point contract as the reference build: no FMA
        # contraction, so results are bit-comparable with oracle/stage.c.
        subprocess.check_call(
            ["gcc", "-shared", "-fPIC", "-O2", "-ffp-contract=off",
             "-fno-strict-aliasing", "-w",
             "-I", py_inc, "-I", np.get_include(),
             "-DNPY_NO_DEPRECATED_API=NPY_1_7_API_VERSION",
             c_out, "-o", so_out, "-lm"])
        built.append(name)
    return built


def load(name):
    """Import one built reference module from ``oracle/_ref`` (or None)."""
    import importlib.util
    ext = sysconfig.get_config_var("EXT_SUFFIX")
    path = os.path.join(OUT, name + ext)
    if not os.path.isfile(path):
        return None
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    print(build(root, quiet=False))
