"""ctypes binding of libmwfgpu.so (include/mwf_gpu.h).

The library is the product: there is no CPU fallback.  Loading fails loudly if the
shared object is missing; build it with ``python -m mwf_gb300.build`` (nvcc, sm_103a).
"""
import ctypes
import os

from .build import LIB

MWF_FP64 = 0
MWF_FP32 = 1

ERRORS = {
    -1: "MWF_ERR_ARG",
    -2: "MWF_ERR_SIZE",
    -3: "MWF_ERR_CUDA",
    -4: "MWF_ERR_NOMEM",
    -5: "MWF_ERR_DEVICE",
    -6: "MWF_ERR_NONFINITE",
}


class MwfError(RuntimeError):
    """A C-ABI call returned a negative status."""

    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class RunDescC(ctypes.Structure):
    """mirror of struct mwf_run_desc"""
    _fields_ = [
        ("K0", ctypes.c_int),
        ("MM", ctypes.c_int),
        ("NN", ctypes.c_int),
        ("precision", ctypes.c_int),
        ("alpha", ctypes.c_double),
        ("gamma", ctypes.c_double),
        ("Re", ctypes.c_double),
        ("dt", ctypes.c_double),
        ("drag", ctypes.c_double),
        ("vdrag", ctypes.c_double),
        ("hypo", ctypes.c_double),
        ("dragall", ctypes.c_int),
        ("reflect", ctypes.c_int),
        ("uvreflect", ctypes.c_int),
        ("wreflect", ctypes.c_int),
        ("theta", ctypes.c_double),
        ("xf_cols", ctypes.c_int),
        ("xi_cols", ctypes.c_int),
        ("z_lines", ctypes.c_int),
        ("x_radix", ctypes.c_int),
        ("z_radix", ctypes.c_int),
    ]


class RunPlanC(ctypes.Structure):
    """mirror of struct mwf_run_plan"""
    _fields_ = [
        ("batched_x", ctypes.c_int),
        ("batched_z", ctypes.c_int),
        ("xf_cols", ctypes.c_int),
        ("xi_cols", ctypes.c_int),
        ("z_lines", ctypes.c_int),
        ("xf_ctas_per_sm", ctypes.c_int),
        ("z_ctas_per_sm", ctypes.c_int),
        ("xi_ctas_per_sm", ctypes.c_int),
        ("xf_smem", ctypes.c_longlong),
        ("z_smem", ctypes.c_longlong),
        ("xi_smem", ctypes.c_longlong),
        ("xf_items", ctypes.c_int),
        ("z_items", ctypes.c_int),
        ("xi_items", ctypes.c_int),
    ]


# symbol -> (restype, argtypes); every entry point declared in include/mwf_gpu.h
SIGNATURES = {
    "mwf_create": (ctypes.c_int, [ctypes.POINTER(RunDescC), ctypes.c_int, ctypes.c_int,
                                  ctypes.POINTER(ctypes.c_void_p)]),
    "mwf_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "mwf_set_state": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]),
    "mwf_get_state": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]),
    "mwf_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "mwf_step_async": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "mwf_synchronize": (ctypes.c_int, [ctypes.c_void_p]),
    "mwf_get_history": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.POINTER(ctypes.c_int)]),
    "mwf_set_history": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]),
    "mwf_query": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]),
    "mwf_reset_history": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "mwf_set_active": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]),
    "mwf_phys_diagnostics": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_double,
                                            ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
    "mwf_test_copy_timeout": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_uint, ctypes.c_double]),
    "mwf_energy": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]),
    "mwf_get_phys": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]),
    "mwf_spectrum_maxima": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]),
    "mwf_history": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                   ctypes.c_void_p]),
    "mwf_remap_x": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]),
    "mwf_blend_state": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_double]),
    "mwf_add_noise": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_ulonglong]),
    "mwf_step_timed": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]),
    "mwf_profile_passes": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]),
    "mwf_set_persistent": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "mwf_kernels_per_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]),
    "mwf_measure_fma_peak": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]),
    "mwf_step_noalloc": (ctypes.c_int, [ctypes.POINTER(RunDescC), ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int]),
    "mwf_spec2phys": (ctypes.c_int, [ctypes.POINTER(RunDescC), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "mwf_phys2spec": (ctypes.c_int, [ctypes.POINTER(RunDescC), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "mwf_run_dof": (ctypes.c_longlong, [ctypes.POINTER(RunDescC)]),
    "mwf_footprint_bytes": (ctypes.c_longlong, [ctypes.POINTER(RunDescC), ctypes.c_int]),
    "mwf_describe_run": (ctypes.c_int, [ctypes.POINTER(RunDescC), ctypes.POINTER(RunPlanC)]),
    "mwf_host_alloc": (ctypes.c_int, [ctypes.c_size_t, ctypes.POINTER(ctypes.c_void_p)]),
    "mwf_host_free": (ctypes.c_int, [ctypes.c_void_p]),
    "mwf_last_error": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_size_t]),
}

_lib = None


def load(path=None):
    """Load libmwfgpu.so (once) and declare its signatures."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    path = path or LIB
    if not os.path.exists(path):
        raise ImportError(f"{path} not found: build the CUDA library first "
                          "(python -m mwf_gb300.build); there is no CPU fallback")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def last_error():
    lib = load()
    buf = ctypes.create_string_buffer(1024)
    lib.mwf_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(rc):
    if rc != 0:
        raise MwfError(rc, last_error())
    return rc
