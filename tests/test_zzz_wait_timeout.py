"""Failure detection without a GPU fault: a kernel's bounded mbarrier wait
(the one every tcgen05 pipeline uses) runs out on a barrier that nothing
completes, records DMRG_ERR_TIMEOUT, and returns; the host reads the status
after ~2 s and the device keeps working (a GEMM right after it is exact).
The file name sorts last, so the other GPU tests run first."""
import ctypes
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_bounded_wait_times_out_and_device_stays_usable():
    import torch
    from dmrgpy_gb300 import _lib
    lib = _lib.load()
    work = torch.zeros(256, dtype=torch.uint8, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    t0 = time.perf_counter()
    st = lib.dmrg_wait_timeout_probe(work.data_ptr(), 256, stream)
    dt = time.perf_counter() - t0
    assert st == _lib.DMRG_ERR_TIMEOUT, st
    assert 0.2 < dt < 60.0, dt
    assert lib.dmrg_wait_timeout_probe(None, 0, stream) == _lib.DMRG_ERR_WORKSPACE
    # the context is intact: an FP64 GEMM through the library right after
    rng = np.random.default_rng(1)
    A = torch.from_numpy(rng.standard_normal((64, 48))).cuda()
    B = torch.from_numpy(rng.standard_normal((48, 32))).cuda()
    C = torch.empty((64, 32), dtype=torch.float64, device="cuda")
    assert lib.dmrg_gemm(_lib.REAL64, _lib.PREC_FP64, 64, 48, 32, A.data_ptr(), B.data_ptr(), C.data_ptr(),
                         None, 0, stream) == _lib.DMRG_OK
    torch.cuda.synchronize()
    assert torch.allclose(C, A @ B, rtol=1e-12, atol=1e-12)
