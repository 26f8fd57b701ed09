"""ctypes binding of libdmrg_gb300.so (C ABI declared in include/dmrg_gb300.h).

The library is built in-tree (``dmrgpy_gb300/build.py``).  Loading fails
loudly when the library is missing or no CUDA device is present: the sweep
has no CPU fallback.
"""
import ctypes
import os
import threading

from . import build as _build

DMRG_OK = 0
DMRG_ERR_ARG = 1
DMRG_ERR_WORKSPACE = 2
DMRG_ERR_CUDA = 3
DMRG_ERR_NAN = 4
DMRG_ERR_NOCONV = 5
DMRG_ERR_TIMEOUT = 6
DMRG_ERR_UNSUPPORTED = 7
DMRG_ERR_PRECISION = 8

# size of the fixed device array behind dmrg_heff_apply_noalloc
# (DMRG_NOALLOC_SCRATCH_BYTES in include/dmrg_gb300.h)
NOALLOC_SCRATCH_BYTES = 64 << 20

REAL64 = 0
COMPLEX128 = 1
PREC_FP64 = 0
PREC_TF32X3 = 1
GRAM_FP64 = 0
GRAM_DIGITS = 1

c_size_t = ctypes.c_size_t
c_int = ctypes.c_int
c_double = ctypes.c_double
c_void_p = ctypes.c_void_p
P_int = ctypes.POINTER(ctypes.c_int)
P_double = ctypes.POINTER(ctypes.c_double)
P_void = ctypes.POINTER(ctypes.c_void_p)


class HeffDesc(ctypes.Structure):
    """Mirror of ``dmrg_heff_t``."""
    _fields_ = [("kind", c_int), ("dtype", c_int), ("precision", c_int),
                ("chil", c_int), ("d1", c_int), ("d2", c_int), ("chir", c_int),
                ("wl", c_int), ("wm", c_int), ("wr", c_int),
                ("L", c_void_p), ("W1", c_void_p), ("W2", c_void_p), ("R", c_void_p)]


# (name, restype, argtypes) for every exported symbol of include/dmrg_gb300.h
SIGNATURES = [
    ("dmrg_version", c_int, []),
    ("dmrg_status_string", ctypes.c_char_p, [c_int]),
    ("dmrg_kernel_launches", ctypes.c_ulonglong, []),
    ("dmrg_heff_workspace_bytes", c_size_t, [ctypes.POINTER(HeffDesc)]),
    ("dmrg_heff_apply", c_int, [ctypes.POINTER(HeffDesc), c_void_p, c_void_p, c_void_p, c_size_t, c_void_p]),
    ("dmrg_heff_prepare", c_int, [ctypes.POINTER(HeffDesc), c_void_p, c_size_t, c_void_p]),
    ("dmrg_heff_apply_prepared", c_int, [ctypes.POINTER(HeffDesc), c_void_p, c_void_p, c_void_p, c_size_t,
                                         c_void_p]),
    ("dmrg_heff_status", c_int, [ctypes.POINTER(HeffDesc), c_void_p, c_size_t, c_void_p]),
    ("dmrg_heff_apply_noalloc", c_int, [ctypes.POINTER(HeffDesc), c_void_p, c_void_p, c_void_p]),
    ("dmrg_env_workspace_bytes", c_size_t, [c_int, c_int, c_int, c_int, c_int, c_int, c_int]),
    ("dmrg_env_extend_left", c_int, [c_int, c_int, c_int, c_int, c_int, c_int, c_int,
                                     c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_size_t, c_void_p]),
    ("dmrg_env_extend_right", c_int, [c_int, c_int, c_int, c_int, c_int, c_int, c_int,
                                      c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_size_t, c_void_p]),
    ("dmrg_env_gradient_workspace_bytes", c_size_t, [c_int, c_int, c_int, c_int, c_int, c_int]),
    ("dmrg_env_gradient", c_int, [c_int, c_int, c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p,
                                  c_void_p, c_size_t, c_void_p]),
    ("dmrg_env_mixed_workspace_bytes", c_size_t, [c_int] * 9),
    ("dmrg_env_extend_mixed", c_int, [c_int] * 9 + [c_void_p] * 6 + [c_size_t, c_void_p]),
    ("dmrg_env_gradient_mixed_workspace_bytes", c_size_t, [c_int] * 8),
    ("dmrg_env_gradient_mixed", c_int, [c_int] * 8 + [c_void_p] * 6 + [c_size_t, c_void_p]),
    ("dmrg_lanczos_workspace_bytes", c_size_t, [ctypes.POINTER(HeffDesc), c_int]),
    ("dmrg_lanczos_ground", c_int, [ctypes.POINTER(HeffDesc), c_void_p, c_int, c_double, P_double, P_int,
                                    c_void_p, c_size_t, c_void_p]),
    ("dmrg_expm_workspace_bytes", c_size_t, [ctypes.POINTER(HeffDesc), c_int]),
    ("dmrg_krylov_expm", c_int, [ctypes.POINTER(HeffDesc), c_void_p, c_double, c_double, c_int, c_double,
                                 c_double, P_int, c_void_p, c_size_t, c_void_p]),
    ("dmrg_svd_workspace_bytes", c_size_t, [c_int, c_int, c_int]),
    ("dmrg_svd_truncate", c_int, [c_int, c_int, c_int, c_void_p, c_double, c_int, c_int, c_int,
                                  c_void_p, c_void_p, P_double, P_int, P_double, c_void_p, c_size_t, c_void_p]),
    ("dmrg_subspace_workspace_bytes", c_size_t, [c_int, c_int, c_int]),
    ("dmrg_subspace_truncate", c_int, [c_int, c_int, c_int, c_void_p, c_void_p, c_int, c_int, c_int, c_void_p,
                                       c_void_p, P_double, c_void_p, c_size_t, c_void_p]),
    ("dmrg_subspace_truncate_ex_workspace_bytes", c_size_t, [c_int, c_int, c_int, c_int]),
    ("dmrg_subspace_truncate_ex", c_int, [c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_int, c_int, c_int,
                                          c_double, c_int, c_void_p, c_void_p, P_double, P_int, P_double, c_void_p,
                                          c_size_t, c_void_p]),
    ("dmrg_syev_workspace_bytes", c_size_t, [c_int]),
    ("dmrg_syev", c_int, [c_int, c_void_p, ctypes.c_longlong, P_double, c_void_p, ctypes.c_longlong, P_int,
                          c_void_p, c_size_t, c_void_p]),
    ("dmrg_gram_workspace_bytes", c_size_t, [c_int, c_int, c_int]),
    ("dmrg_gram", c_int, [c_int, c_int, c_int, c_void_p, ctypes.c_longlong, c_void_p, c_void_p, c_size_t, c_void_p]),
    ("dmrg_wait_timeout_probe", c_int, [c_void_p, c_size_t, c_void_p]),
    ("dmrg_gemm", c_int, [c_int, c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_size_t,
                          c_void_p]),
    ("dmrg_gemm_workspace_bytes", c_size_t, [c_int, c_int, c_int, c_int, c_int]),
    ("dmrg_autotune_enable", c_int, [c_int]),
    ("dmrg_autotune_entries", c_int, [P_int, c_int]),
    ("dmrg_batch_gemm_workspace_bytes", c_size_t, [c_int]),
    ("dmrg_batch_gemm", c_int, [c_int, c_int, P_int, P_int, P_int, P_void, P_void, P_void, c_void_p, c_size_t,
                                c_void_p]),
    ("dmrg_batch_env_workspace_bytes", c_size_t, [c_int, c_int, c_int, P_int, P_int, P_int, P_int, P_int]),
    ("dmrg_batch_env_extend", c_int, [c_int, c_int, c_int, P_int, P_int, P_int, P_int, P_int, P_void, P_void,
                                      P_void, P_void, c_void_p, c_size_t, c_void_p]),
    ("dmrg_batch_lanczos_workspace_bytes", c_size_t, [c_int, ctypes.POINTER(HeffDesc), c_int]),
    ("dmrg_batch_lanczos_ground", c_int, [c_int, ctypes.POINTER(HeffDesc), P_void, c_int, c_double, c_int, P_double,
                                          P_int, c_void_p, c_size_t, c_void_p]),
    ("dmrg_batch_svd_workspace_bytes", c_size_t, [c_int, c_int, P_int, P_int]),
    ("dmrg_batch_svd_factor", c_int, [c_int, c_int, P_int, P_int, P_void, c_double, P_int, c_int, c_int, P_int,
                                      P_double, P_double, c_int, c_void_p, c_size_t, c_void_p]),
    ("dmrg_batch_svd_output", c_int, [c_int, c_int, P_int, P_int, P_int, c_int, P_void, P_void, c_void_p, c_size_t,
                                      c_void_p]),
]


class DmrgError(RuntimeError):
    """A non-zero status from the C ABI."""

    def __init__(self, fn, status, msg):
        super().__init__("{} failed with status {} ({})".format(fn, status, msg))
        self.status = status
        self.fn = fn


_lock = threading.Lock()
_lib = None


def library_path():
    return _build.LIB


def load(build_if_missing=True):
    """Load (building first if needed) the CUDA library."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB
        if build_if_missing:
            path = _build.build()
        if not os.path.exists(path):
            raise OSError("libdmrg_gb300.so not found at {} (run dmrgpy_gb300/build.py)".format(path))
        lib = ctypes.CDLL(path)
        for name, res, args in SIGNATURES:
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def check(fn, status):
    if status != DMRG_OK:
        lib = load(build_if_missing=False)
        raise DmrgError(fn, status, lib.dmrg_status_string(status).decode())
    return status
