"""Gram matrix X^T X by exact digit products on the tensor cores
(dmrg_gram, DMRG_GRAM_DIGITS) against the FP64 CUDA-core Gram and an FP64
cuBLAS product: error bound 1e-12 relative to |x_a| |x_b| (the method's
error is ~1e-13; an FP64 product's ~1e-15; a split-TF32 Gram's ~1e-7), an
exactly symmetric result, ragged and tiny shapes, the size limit and a
non-finite input."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _gram(method, X, expect=0):
    import torch
    from dmrgpy_gb300 import _lib
    lib = _lib.load()
    m, k = X.shape
    G = torch.full((k, k), float("nan"), dtype=torch.float64, device=X.device)
    need = lib.dmrg_gram_workspace_bytes(method, m, k)
    work = torch.empty(max(need, 1), dtype=torch.uint8, device=X.device)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    st = lib.dmrg_gram(method, m, k, X.data_ptr(), X.stride(0), G.data_ptr(), work.data_ptr(), need, stream)
    assert st == expect, st
    return G


def _scaled_err(G, ref):
    d = np.sqrt(np.abs(np.diag(ref)))
    den = np.outer(d, d)
    den[den == 0] = 1.0
    return float(np.max(np.abs(G - ref) / den))


def _to_dev(X):
    import torch
    return torch.from_numpy(np.ascontiguousarray(X)).to("cuda")


@pytest.mark.parametrize("m,k", [(3072, 1024), (1000, 77), (33, 129), (5, 3), (1, 1)])
def test_gram_digits_orthonormal_and_general(m, k):
    from dmrgpy_gb300 import _lib
    rng = np.random.default_rng(m * 31 + k)
    if m >= k:
        X = np.linalg.qr(rng.standard_normal((m, k)))[0]
    else:
        X = rng.standard_normal((m, k))
    Xd = _to_dev(X)
    Gd = _gram(_lib.GRAM_DIGITS, Xd).cpu().numpy()
    Gf = _gram(_lib.GRAM_FP64, Xd).cpu().numpy()
    Gt = (Xd.T @ Xd).cpu().numpy()
    assert np.array_equal(Gd, Gd.T)
    assert _scaled_err(Gd, Gt) < TOL
    assert _scaled_err(Gd, Gf) < TOL
    if m >= k:
        assert np.max(np.abs(Gd - np.eye(k))) < 1e-12


def test_gram_digits_columns_of_wildly_different_scale():
    """Per-column power-of-two scaling: columns from 1e-8 to 1e8 (and an
    all-zero column) keep their own relative accuracy."""
    from dmrgpy_gb300 import _lib
    rng = np.random.default_rng(5)
    m, k = 2000, 150
    X = rng.standard_normal((m, k)) * np.exp(rng.uniform(-18.0, 18.0, k))
    X[:, 7] = 0.0
    X[:, 11] = 2.0 ** -3    # a constant column whose maximum is a power of two
    Xd = _to_dev(X)
    Gd = _gram(_lib.GRAM_DIGITS, Xd).cpu().numpy()
    Gt = (Xd.T @ Xd).cpu().numpy()
    assert np.all(Gd[7] == 0.0) and np.all(Gd[:, 7] == 0.0)
    assert _scaled_err(Gd, Gt) < TOL


def test_gram_digits_strided_input_and_largest_m():
    """A leading dimension larger than k (a column block of a wider array),
    and the largest supported m (32768 rows: 1024 K-slices)."""
    import torch
    from dmrgpy_gb300 import _lib
    rng = np.random.default_rng(9)
    W = _to_dev(rng.standard_normal((32768, 96)))
    X = W[:, 10:74]
    assert X.stride(0) == 96
    Gd = _gram(_lib.GRAM_DIGITS, X).cpu().numpy()
    Gt = (X.T @ X).cpu().numpy()
    assert _scaled_err(Gd, Gt) < TOL
    big = torch.zeros((32769, 4), dtype=torch.float64, device="cuda")
    _gram(_lib.GRAM_DIGITS, big, expect=_lib.DMRG_ERR_ARG)


def test_gram_digits_reports_non_finite_input():
    from dmrgpy_gb300 import _lib
    X = np.ones((64, 8))
    X[17, 3] = np.nan
    _gram(_lib.GRAM_DIGITS, _to_dev(X), expect=_lib.DMRG_ERR_NAN)
