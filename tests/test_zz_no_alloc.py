"""dmrg_heff_apply_noalloc (scratch in a fixed device array inside the
library) against dmrg_heff_apply (caller workspace) on the same operator:
calls in a row must all reproduce the workspace result, and after the
first one they must leave the device's free memory and torch's allocation
unchanged.  The file name
sorts last so the test also runs after every other GPU test, and it needs
nothing from them when run alone."""
import ctypes

import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-13  # same kernels and summation order; only the scratch location differs


def _operands(kind, dtype, chil, d, chir, w, seed):
    import torch
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)

    def rnd(*shape):
        x = torch.randn(*shape, dtype=torch.float64, device="cuda", generator=g)
        if dtype == torch.complex128:
            x = torch.complex(x, torch.randn(*shape, dtype=torch.float64, device="cuda", generator=g))
        return x.contiguous()

    L = rnd(chil, w, chil)
    R = rnd(chir, w, chir)
    W1 = rnd(w, d, d, w)
    W2 = rnd(w, d, d, w)
    x = rnd(chil, d, d, chir) if kind == 2 else rnd(chil, d, chir)
    return L, W1, W2, R, x


def _desc(lib_mod, kind, cdtype, chil, d, chir, w, L, W1, W2, R):
    h = lib_mod.HeffDesc()
    h.kind, h.dtype, h.precision = kind, cdtype, lib_mod.PREC_FP64
    h.chil, h.d1, h.d2, h.chir = chil, d, (d if kind == 2 else 1), chir
    h.wl, h.wm, h.wr = w, w, w
    h.L, h.R = L.data_ptr(), R.data_ptr()
    h.W1 = W1.data_ptr()
    h.W2 = W2.data_ptr() if kind == 2 else None
    return h


@pytest.mark.parametrize("kind,complex_", [(2, False), (2, True), (1, False), (1, True)])
def test_noalloc_matches_workspace_matvec_twice(kind, complex_):
    import torch
    from dmrgpy_gb300 import _lib
    lib = _lib.load()
    dtype = torch.complex128 if complex_ else torch.float64
    cdtype = _lib.COMPLEX128 if complex_ else _lib.REAL64
    chil, d, chir, w = 40, 3, 56, 5
    L, W1, W2, R, x = _operands(kind, dtype, chil, d, chir, w, 17 + kind)
    h = _desc(_lib, kind, cdtype, chil, d, chir, w, L, W1, W2, R)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    need = lib.dmrg_heff_workspace_bytes(ctypes.byref(h))
    assert 0 < need <= _lib.NOALLOC_SCRATCH_BYTES
    work = torch.empty(need, dtype=torch.uint8, device="cuda")
    y_ref = torch.empty_like(x)
    _lib.check("dmrg_heff_apply", lib.dmrg_heff_apply(ctypes.byref(h), x.data_ptr(), y_ref.data_ptr(),
                                                      work.data_ptr(), need, stream))
    outs = [torch.full_like(x, float("nan")) for _ in range(4)]
    _lib.check("dmrg_heff_apply_noalloc", lib.dmrg_heff_apply_noalloc(ctypes.byref(h), x.data_ptr(),
                                                                      outs[0].data_ptr(), stream))
    torch.cuda.synchronize()
    # after the first call (which looks up the array's address) the calls
    # allocate nothing: neither torch's allocator nor the device's free
    # memory moves
    free0, allocated0 = torch.cuda.mem_get_info()[0], torch.cuda.memory_allocated()
    for y in outs[1:]:
        _lib.check("dmrg_heff_apply_noalloc", lib.dmrg_heff_apply_noalloc(ctypes.byref(h), x.data_ptr(),
                                                                          y.data_ptr(), stream))
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    assert torch.cuda.memory_allocated() == allocated0
    scale = float(y_ref.abs().max())
    for y in outs:
        assert torch.isfinite(y).all()
        assert float((y - y_ref).abs().max()) <= TOL * scale


def test_noalloc_rejects_oversize_and_tf32_without_launching():
    import torch
    from dmrgpy_gb300 import _lib
    lib = _lib.load()
    L, W1, W2, R, x = _operands(2, torch.float64, 8, 3, 8, 5, 3)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    # an operator whose scratch would exceed the fixed array (pointers are
    # never dereferenced: the size check comes first)
    big = _desc(_lib, 2, _lib.REAL64, 2048, 3, 2048, 5, L, W1, W2, R)
    assert lib.dmrg_heff_workspace_bytes(ctypes.byref(big)) > _lib.NOALLOC_SCRATCH_BYTES
    y = torch.empty_like(x)
    before = lib.dmrg_kernel_launches()
    assert lib.dmrg_heff_apply_noalloc(ctypes.byref(big), x.data_ptr(), y.data_ptr(), stream) == \
        _lib.DMRG_ERR_WORKSPACE
    tf = _desc(_lib, 2, _lib.REAL64, 8, 3, 8, 5, L, W1, W2, R)
    tf.precision = _lib.PREC_TF32X3
    assert lib.dmrg_heff_apply_noalloc(ctypes.byref(tf), x.data_ptr(), y.data_ptr(), stream) == \
        _lib.DMRG_ERR_UNSUPPORTED
    assert lib.dmrg_kernel_launches() == before
