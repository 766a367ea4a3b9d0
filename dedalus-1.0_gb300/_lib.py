"""ctypes binding to libdd_gb300.so (the C ABI declared in include/dd_gb300.h).

Status codes are mapped to the exception classes the reference raises for the
same conditions (ValueError for bad arguments, NotImplementedError for
unsupported shapes/options, RuntimeError for CUDA failures).  There is no CPU
fallback: if the library is missing, every entry point raises.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libdd_gb300.so")

DD_OK, DD_ERR_INVALID, DD_ERR_UNSUPPORTED, DD_ERR_CUDA, DD_ERR_TIMEOUT, DD_ERR_WORKSPACE = range(6)
DD_FP64, DD_FP32, DD_DF64 = 0, 1, 2

_EXC = {
    DD_ERR_INVALID: ValueError,
    DD_ERR_UNSUPPORTED: NotImplementedError,
    DD_ERR_CUDA: RuntimeError,
    DD_ERR_TIMEOUT: TimeoutError,
    DD_ERR_WORKSPACE: ValueError,
}

P = ctypes.c_void_p
PP = ctypes.POINTER(ctypes.c_void_p)
I = ctypes.c_int
I64 = ctypes.c_int64
D = ctypes.c_double
SZ = ctypes.c_size_t

# name -> argtypes; every function returns int status unless listed in _RESTYPE
SIGNATURES = {
    "dd_version": [],
    "dd_last_error": [],
    "dd_launch_count": [],
    "dd_timing_enable": [I],
    "dd_timing_reset": [],
    "dd_timing_report": [ctypes.c_char_p, SZ],
    "dd_plan_create": [I, ctypes.POINTER(I64), P, P, P, I, I, I, ctypes.POINTER(P)],
    "dd_plan_destroy": [P],
    "dd_plan_workspace_size": [P, I, I, ctypes.POINTER(SZ)],
    "dd_fft_r2c": [P, I, PP, PP, I, P, SZ, P],
    "dd_fft_c2r": [P, I, PP, PP, I, P, SZ, P],
    "dd_fft_c2r_noalloc": [P, P, P, P],
    "dd_dealias": [P, P, P],
    "dd_deriv": [P, I, P, P, P],
    "dd_scale_add": [P, P, D, I, I64, P],
    "dd_max_square": [I, PP, I64, P, P],
    "dd_plan_set_schedule": [P, I, I],
    "dd_plan_get_schedule": [P, I, ctypes.POINTER(I), ctypes.POINTER(I)],
    "dd_euler": [P, P, P, D, I64, P],
    "dd_etd1": [I, P, P, P, P, D, I64, P],
    "dd_etd2rk1": [I, P, P, P, P, P, D, I64, P],
    "dd_etd2rk2": [I, P, P, P, P, P, D, I64, P],
    "dd_phi_table": [I, D, I, D, I, P, P],
    "dd_hydro3d_workspace_size": [P, I, ctypes.POINTER(SZ)],
    "dd_hydro3d_rhs": [P, PP, PP, P, I, I, P, SZ, P],
    "dd_hydro3d_rk4_step": [P, PP, P, P, P, D, I, D, I, ctypes.POINTER(I), P, SZ, P],
    "dd_any_nonkept": [P, I, PP, P, P],
    "dd_diag_workspace_size": [P, I, ctypes.POINTER(SZ)],
    "dd_volume_average": [P, I, I, PP, P, P, SZ, P],
    "dd_spectrum": [P, I, PP, D, I, P, P, D, P, P, P, SZ, P],
    "dd_rhs3d_workspace_size": [P, I, I, ctypes.POINTER(SZ)],
    "dd_rhs3d": [P, I, P, PP, PP, P, I, I, P, SZ, P],
    "dd_rk4_step3d": [P, I, P, PP, P, PP, PP, P, I, D, I, ctypes.POINTER(I), P, SZ, P],
    "dd_rhs2d_workspace_size": [P, I, I, ctypes.POINTER(SZ)],
    "dd_rhs2d": [P, I, P, I, PP, I64, PP, I64, P, I, I, P, SZ, P],
    "dd_rk2mid_step2d": [P, I, P, I, PP, I64, P, PP, PP, P, I, D, I, ctypes.POINTER(I), P, SZ, P],
    "dd_mlp_sizes": [ctypes.POINTER(I)] * 5,
    "dd_mlp_workspace_size": [I64, ctypes.POINTER(SZ)],
    "dd_mlp_pack": [P, P, P],
    "dd_mlp_infer": [P, P, I64, P, P, P],
    "dd_mlp_grad": [P, P, P, I64, I64, P, P, P, P, P, SZ, P],
    "dd_mlp_adam": [P, P, P, P, I, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float, P, P],
    "dd_mlp_normalize": [P, I64, P, P, P, P],
    "dd_les_products": [I64, PP, PP, P],
    "dd_les_truncate3": [P, P, I, PP, PP, P],
    "dd_les_gradients": [P, PP, PP, I, P, SZ, P],
    "dd_les_samples": [I64, PP, PP, PP, D, P, P],
    "dd_les_stress": [P, PP, PP, P, I, P, SZ, P],
    "dd_les_band": [P, I, PP, D, D, P],
    "dd_les_transfer": [P, PP, PP, I, P, P, SZ, P],
    "dd_divergence_sums": [P, PP, P, P],
    "dd_divergence_sums2d": [P, I, P, P, I64, P, P],
    "dd_shear_workspace_size": [P, I, ctypes.POINTER(SZ)],
    "dd_shear_r2c": [P, I, PP, PP, P, D, P, D, P, SZ, P],
    "dd_shear_c2r": [P, I, PP, PP, P, D, P, D, P, SZ, P],
    "dd_shear_dealias": [P, I, PP, P, D, P],
    "dd_shear_deriv_y": [P, P, P, P, P],
    "dd_kspace_real": [I64, P, P, D, I, I, P, P],
    "dd_xspace_fma": [I64, P, P, D, I, P, P],
    "dd_les_workspace_size": [P, I, ctypes.POINTER(SZ)],
    "dd_les_rhs3d": [P, PP, PP, P, I, I, P, P, SZ, P],
    "dd_les_rk4_step3d": [P, PP, P, PP, PP, P, I, D, I, ctypes.POINTER(I), P, P, SZ, P],
}


class Closure(ctypes.Structure):
    """dd_closure: device pointers of the BF16 weights, FP32 parameters and
    normalisation vector, the filter width, the closure-term band and the
    optional per-shell weight table (device pointer and length)."""
    _fields_ = [("wbf16", ctypes.c_void_p), ("params", ctypes.c_void_p), ("norm", ctypes.c_void_p),
                ("delta", ctypes.c_double), ("band_lo", ctypes.c_double), ("band_hi", ctypes.c_double),
                ("shell_w", ctypes.c_void_p), ("n_shell", ctypes.c_int)]

_RESTYPE = {"dd_last_error": ctypes.c_char_p, "dd_launch_count": ctypes.c_longlong}


def launch_count():
    return int(lib().dd_launch_count())


def timing_enable(on=True):
    check(lib().dd_timing_enable(1 if on else 0))


def timing_reset():
    check(lib().dd_timing_reset())


def timing_report():
    """{label: (launches, total device ms)} since the last reset."""
    buf = ctypes.create_string_buffer(1 << 20)
    check(lib().dd_timing_report(buf, len(buf)))
    out = {}
    for line in buf.value.decode().splitlines():
        name, n, ms = line.split()
        out[name] = (int(n), float(ms))
    return out

_lib = None


class LibraryMissing(ImportError):
    pass


def lib():
    """Load the CUDA library (raises LibraryMissing if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.isfile(LIB_PATH):
            raise LibraryMissing("%s is not built; run __graft_entry__.build() (nvcc) first" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        for name, args in SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = _RESTYPE.get(name, ctypes.c_int)
        _lib = L
    return _lib


def check(rc, what=""):
    if rc != DD_OK:
        msg = lib().dd_last_error().decode(errors="replace")
        raise _EXC.get(rc, RuntimeError)("%s%s" % (what + ": " if what else "", msg))


def call(name, *args):
    check(getattr(lib(), name)(*args), name)


def ptr_array(ptrs):
    arr = (ctypes.c_void_p * len(ptrs))(*[ctypes.c_void_p(int(p)) for p in ptrs])
    return ctypes.cast(arr, PP), arr
