"""Split-TF32 (3 products, FP32 accumulation) tcgen05 path against the FP64
oracle.  Tolerance: max|y - y_ref| <= 2e-6 * max|y_ref| -- FP32-level, the
accuracy class of 3xTF32 with FP32 accumulation over K <= ~10^4 terms."""
import numpy as np
import pytest

import oracle as O
from golden_data import meta, terms_heisenberg

pytestmark = pytest.mark.gpu

TOL = 2e-6


def _engine(W, precision):
    from dmrgpy_gb300.engine import Engine
    return Engine(W, real=True, precision=precision)


def _mpo_pair(code):
    from dmrgpy_gb300 import mpo as M
    if code == "hubbard":
        # spinful fermions, d = 4: the two-site MPO step is 96 wide
        md = meta()
        W, real = M.build_mpo(md["types"]["hubbard4"], md["terms"]["hubbard4"])
        assert real
        return W[1], W[2]
    W, real = M.build_mpo([code] * 6, terms_heisenberg(6))
    assert real
    return W[2], W[3]


@pytest.mark.parametrize("chil,chir,code", [(96, 96, 2), (64, 160, 3), (256, 256, 3), (37, 45, 2),
                                            (64, 72, "hubbard")])
def test_tf32x3_two_site_matvec(chil, chir, code):
    rng = np.random.default_rng(chil * 7 + chir)
    Wi, Wj = _mpo_pair(code)
    d = Wi.shape[1]
    L = rng.standard_normal((chil, Wi.shape[0], chil))
    R = rng.standard_normal((chir, Wj.shape[3], chir))
    th = rng.standard_normal((chil, d, d, chir))
    ref = O.heff2_matvec(L, Wi, Wj, R, th).real
    eng = _engine([Wi, Wj], "tf32x3")
    Ld, Rd, thd = eng.to_device([L, R, th])
    h = eng.heff2(Ld, eng.W[0], eng.W[1], Rd, th.shape)
    y = eng.apply(h, thd).cpu().numpy()
    err = np.max(np.abs(y - ref)) / np.max(np.abs(ref))
    assert err < TOL, err
    # two applications in a row give identical results (no stale state)
    y2 = eng.apply(h, thd).cpu().numpy()
    assert np.array_equal(y, y2)


def test_tf32x3_two_site_matvec_at_the_headline_bond():
    """The split-TF32 matvec at the headline bond (chi = 1024, d = 3, w = 5:
    theta is 1024 x 3 x 3 x 1024) against the oracle's FP64 contraction on
    the host, with the environments of a real state's scale replaced by
    seeded Gaussian ones.  Bars: max|y - y_ref| <= 2e-6 max|y_ref| and
    |y - y_ref| <= 1e-6 |y_ref|."""
    rng = np.random.default_rng(1024)
    Wi, Wj = _mpo_pair(3)
    chi = 1024
    L = rng.standard_normal((chi, Wi.shape[0], chi))
    R = rng.standard_normal((chi, Wj.shape[3], chi))
    th = rng.standard_normal((chi, 3, 3, chi))
    ref = O.heff2_matvec(L, Wi, Wj, R, th).real
    eng = _engine([Wi, Wj], "tf32x3")
    Ld, Rd, thd = eng.to_device([L, R, th])
    h = eng.heff2(Ld, eng.W[0], eng.W[1], Rd, th.shape)
    y = eng.apply(h, thd).cpu().numpy()
    assert np.max(np.abs(y - ref)) / np.max(np.abs(ref)) < TOL
    assert np.linalg.norm(y - ref) / np.linalg.norm(ref) < 1e-6


@pytest.mark.parametrize("m,k,n", [(300, 64, 200), (3 * 128, 256, 3 * 128), (5, 7, 9)])
def test_tf32x3_gemm(m, k, n):
    rng = np.random.default_rng(m + k + n)
    A = rng.standard_normal((m, k))
    B = rng.standard_normal((k, n))
    eng = _engine([np.zeros((1, 2, 2, 1))], "tf32x3")
    Ad, Bd = eng.to_device([A, B])
    C = eng.gemm(Ad, Bd).cpu().numpy()
    ref = A @ B
    assert np.max(np.abs(C - ref)) / np.max(np.abs(ref)) < TOL


def test_tf32x3_lanczos_energy_close_to_fp64():
    rng = np.random.default_rng(5)
    Wi, Wj = _mpo_pair(3)
    d, w = Wi.shape[1], Wi.shape[3]
    chi = 128
    # Hermitian environments: symmetrise random blocks per MPO index
    L = rng.standard_normal((chi, w, chi))
    L = 0.5 * (L + L.transpose(2, 1, 0))
    R = rng.standard_normal((chi, w, chi))
    R = 0.5 * (R + R.transpose(2, 1, 0))
    th = rng.standard_normal((chi, d, d, chi))
    out = {}
    for prec in ("fp64", "tf32x3"):
        eng = _engine([Wi, Wj], prec)
        Ld, Rd, thd = eng.to_device([L, R, th])
        h = eng.heff2(Ld, eng.W[0], eng.W[1], Rd, th.shape)
        e, k = eng.ground(h, thd, 200)
        out[prec] = e
    assert abs(out["tf32x3"] - out["fp64"]) <= 1e-5 * abs(out["fp64"])


def test_gemm_tile_order_tuner_changes_nothing_but_speed():
    """The tuner picks a tile width and order per GEMM shape.  Every output
    element sums the same K slices in the same order under every choice, so
    tuned and untuned runs agree to FP32 rounding (bit-identical in practice;
    the bound allows for the tensor core's internal order)."""
    import ctypes
    from dmrgpy_gb300 import _lib
    lib = _lib.load()
    rng = np.random.default_rng(11)
    m, k, n = 2560, 512, 2560          # 400 output tiles: large enough to be tuned
    A = rng.standard_normal((m, k))
    B = rng.standard_normal((k, n))
    eng = _engine([np.zeros((1, 2, 2, 1))], "tf32x3")
    Ad, Bd = eng.to_device([A, B])
    prev = lib.dmrg_autotune_enable(0)
    try:
        C0 = eng.gemm(Ad, Bd).cpu().numpy()
        lib.dmrg_autotune_enable(1)
        C1 = eng.gemm(Ad, Bd).cpu().numpy()      # first call of the shape: tuned
        C2 = eng.gemm(Ad, Bd).cpu().numpy()      # uses the decision
    finally:
        lib.dmrg_autotune_enable(prev)
    scale = np.max(np.abs(C0))
    assert np.max(np.abs(C0 - C1)) <= 1e-6 * scale and np.array_equal(C1, C2)
    count = lib.dmrg_autotune_entries(None, 0)
    buf = (ctypes.c_int * (7 * max(count, 1)))()
    lib.dmrg_autotune_entries(buf, count)
    shapes = [tuple(buf[7 * i:7 * i + 6]) for i in range(count)]
    assert all(s[3] in (64, 128) and s[4] in (0, 1) for s in shapes), shapes
    assert any(s[0] == m and s[1] == n for s in shapes), shapes
    assert np.max(np.abs(C1 - A @ B)) / np.max(np.abs(A @ B)) < TOL


@pytest.mark.parametrize("absorb", [0, 1])
def test_subspace_truncation_is_orthonormal_and_near_optimal(absorb):
    """Fixed-rank truncation by subspace iteration from a warm start (the
    orthonormal tensor across the bond, here the exact singular vectors
    perturbed by 1e-3): the kept basis is orthonormal to FP64 level (FP64-Gram
    correction) and the discarded weight is within 10% of the SVD optimum."""
    rng = np.random.default_rng(21 + absorb)
    m = n = 576
    k = 256
    U, _ = np.linalg.qr(rng.standard_normal((m, m)))
    V, _ = np.linalg.qr(rng.standard_normal((n, n)))
    s = np.exp(-12.0 * np.arange(m) / m)
    th = (U * s) @ V.T
    opt = np.sqrt(np.sum(s[k:] ** 2) / np.sum(s ** 2))
    if absorb == 0:
        start, _ = np.linalg.qr(V[:, :k] + 1e-3 * rng.standard_normal((n, k)))
        start = np.ascontiguousarray(start.T)          # k x n, orthonormal rows
    else:
        start, _ = np.linalg.qr(U[:, :k] + 1e-3 * rng.standard_normal((m, k)))
        start = np.ascontiguousarray(start)            # m x k, orthonormal columns
    eng = _engine([np.zeros((1, 2, 2, 1))], "tf32x3")
    thd, std = eng.to_device([th, start])
    lo, ro, _, kk, disc = eng.subspace_split(thd, k, std, k, absorb)
    lo, ro = lo.cpu().numpy(), ro.cpu().numpy()
    Q = lo if absorb == 0 else ro.T
    assert np.max(np.abs(Q.T @ Q - np.eye(k))) < 1e-10
    rec = np.linalg.norm(lo @ ro - th) / np.linalg.norm(th)
    assert rec < 1.1 * opt, (rec, opt)
    # the discarded weight is 1 - |Q^T theta|^2/|theta|^2 with Q^T theta from
    # the split-TF32 GEMM (~1e-6 relative in |.|^2)
    assert abs(disc - rec ** 2) < 0.1 * rec ** 2 + 2e-6
