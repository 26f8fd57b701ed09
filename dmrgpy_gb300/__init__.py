"""GB300-native backend for dmrgpy's finite-chain two-site DMRG/TDVP sweep.

The sweep (H_eff matvec, Lanczos and Krylov-exponential loops, truncated
SVD, environment updates) runs as hand-written sm_103a CUDA kernels of
``libdmrg_gb300.so`` behind a C ABI (``include/dmrg_gb300.h``), driven from
Python through ctypes.  :class:`Chain` mirrors the session object of dmrgpy's
python backend; :func:`register` plugs it into dmrgpy's backend registry.
"""
from .chain import Chain, Operator  # noqa: F401
from .engine import Engine  # noqa: F401
from .mps import MPS  # noqa: F401
from .backend import BACKEND_TAG, register  # noqa: F401

__version__ = "0.1.0"
