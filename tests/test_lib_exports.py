"""The C-ABI library builds for sm_103a, loads, and exports every function
declared in include/dmrg_gb300.h (no compute call: no GPU needed)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_functions():
    src = open(os.path.join(ROOT, "include", "dmrg_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_ \*]*?\b(dmrg_[a-z0-9_]+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_header_declares_the_hot_path_entry_points():
    names = _declared_functions()
    for required in ("dmrg_heff_apply", "dmrg_env_extend_left", "dmrg_env_extend_right",
                     "dmrg_lanczos_ground", "dmrg_krylov_expm", "dmrg_svd_truncate", "dmrg_gemm"):
        assert required in names


def test_library_builds_loads_and_exports_every_declared_symbol():
    from dmrgpy_gb300 import _lib
    lib = _lib.load(build_if_missing=True)
    for name in _declared_functions():
        assert hasattr(lib, name), name
    assert lib.dmrg_version() >= 100
    assert lib.dmrg_status_string(_lib.DMRG_ERR_WORKSPACE) == b"workspace too small"
    # every declared symbol has a ctypes signature in the binding
    bound = {n for n, _, _ in _lib.SIGNATURES}
    assert set(_declared_functions()) <= bound


def test_workspace_queries_are_host_only():
    from dmrgpy_gb300 import _lib
    lib = _lib.load()
    h = _lib.HeffDesc(kind=2, dtype=_lib.REAL64, precision=_lib.PREC_FP64, chil=8, d1=2, d2=2, chir=8,
                      wl=5, wm=5, wr=5, L=1, W1=1, W2=1, R=1)
    assert lib.dmrg_heff_workspace_bytes(ctypes.byref(h)) > 0
    assert lib.dmrg_lanczos_workspace_bytes(ctypes.byref(h), 200) > lib.dmrg_heff_workspace_bytes(ctypes.byref(h))
    assert lib.dmrg_svd_workspace_bytes(_lib.REAL64, 16, 32) > 0
    bad = _lib.HeffDesc(kind=7)
    assert lib.dmrg_heff_workspace_bytes(ctypes.byref(bad)) == 0
    # argument errors are reported as status codes, never as a crash
    assert lib.dmrg_heff_apply(ctypes.byref(bad), None, None, None, 0, None) == _lib.DMRG_ERR_ARG
    assert lib.dmrg_svd_truncate(0, 0, 4, None, 0.0, 0, 1, 0, None, None, None, None, None, None, 0,
                                 None) == _lib.DMRG_ERR_ARG
