"""GPU tests of the Gram-matrix truncation: the blocked-Jacobi eigensolver
(dmrg_syev) against numpy, the Gram route of dmrg_svd_truncate against the
reference's own truncations of real matrices (tests/golden/
reference_truncation.npz, made by make_golden_truncation.py), and the
subspace + Rayleigh-Ritz route (dmrg_subspace_truncate_ex) in FP64 and
split-TF32 against the oracle's truncation rule on exact spectra and on the
two-site tensors of real sweeps.

Tolerances: eigenvalues 1e-12 of the norm, eigenvectors orthonormal to
1e-13; singular values from a Gram matrix are accurate to ~eps*s0^2/s
(pyitensor/svd.py:108-151 documents the same bound), so they are compared
within 1e-13*s0 + 1e-15*s0^2/s; kept counts exactly; discarded weights to
1e-13 absolute.  The split-TF32 route's Ritz values come from FP32-accurate
products: 2e-5 relative."""
import ctypes
import os

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

GOLD = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_truncation.npz"))


def _eng(precision="fp64"):
    from dmrgpy_gb300.engine import Engine
    return Engine([np.zeros((1, 2, 2, 1))], real=True, precision=precision)


def _syev(eng, A):
    from dmrgpy_gb300 import _lib
    torch = __import__("torch")
    n = A.shape[0]
    Ad = torch.as_tensor(np.ascontiguousarray(A), device=eng.device)
    V = torch.empty((n, n), dtype=torch.float64, device=eng.device)
    w = np.zeros(n)
    sw = ctypes.c_int(0)
    ptr, size = eng.ws.get(eng.lib.dmrg_syev_workspace_bytes(n))
    _lib.check("dmrg_syev", eng.lib.dmrg_syev(n, Ad.data_ptr(), n, w.ctypes.data_as(_lib.P_double), V.data_ptr(), n,
                                              ctypes.byref(sw), ptr, size, eng.stream))
    return w, V.cpu().numpy(), sw.value


@pytest.mark.parametrize("n", [1, 5, 31, 32, 33, 100, 257, 640])
def test_syev_matches_numpy(n):
    rng = np.random.default_rng(n)
    X = rng.standard_normal((n, n))
    A = X + X.T
    eng = _eng()
    w, V, sweeps = _syev(eng, A)
    ref = np.linalg.eigvalsh(A)[::-1]
    nrm = np.max(np.abs(ref))
    assert np.max(np.abs(w - ref)) < 1e-12 * nrm
    assert np.max(np.abs(V.T @ V - np.eye(n))) < 1e-13 * max(1.0, np.sqrt(n))
    assert np.max(np.abs((V * w) @ V.T - A)) < 1e-12 * nrm
    assert sweeps <= 15


def test_syev_degenerate_and_graded_spectra():
    rng = np.random.default_rng(5)
    n = 96
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    eng = _eng()
    # multiplets: each value repeated 3 times
    lam = np.repeat(np.linspace(1.0, 2.0, n // 3), 3)
    A = (Q * lam) @ Q.T
    w, V, _ = _syev(eng, A)
    assert np.max(np.abs(w - np.sort(lam)[::-1])) < 1e-13 * 2
    assert np.max(np.abs(V.T @ V - np.eye(n))) < 1e-13 * 10
    assert np.max(np.abs((V * w) @ V.T - A)) < 1e-13 * 10
    # a PSD Gram matrix spanning 14 decades with a null space (rank 60)
    s = np.exp(-np.linspace(0, 16, 60))
    B = rng.standard_normal((n, 60)) @ np.diag(s)
    G = B @ B.T
    w, V, _ = _syev(eng, G)
    ref = np.linalg.eigvalsh(G)[::-1]
    assert np.max(np.abs(w - ref)) < 1e-14 * ref[0]
    assert np.max(np.abs(V.T @ V - np.eye(n))) < 1e-12
    # the zero matrix
    w, V, sweeps = _syev(eng, np.zeros((40, 40)))
    assert np.all(w == 0.0) and np.allclose(V.T @ V, np.eye(40)) and sweeps == 1


TAGS = [str(t) for t in GOLD["tags"]]


@pytest.mark.parametrize("tag", TAGS)
@pytest.mark.parametrize("absorb", [0, 1, 2])
def test_gram_route_matches_reference_truncation(tag, absorb):
    """dmrg_svd_truncate on a real matrix takes the Gram route (the kept
    side's FP64 Gram matrix, dmrg_syev, the reference's keep rule) and
    reproduces the reference's kept count, singular values and truncation
    error (pyitensor/svd.py:32-68, 108-151)."""
    M = GOLD[tag + "_M"]
    cut, md = GOLD[tag + "_cut"]
    Sref = GOLD[tag + "_S"]
    eng = _eng()
    Md = eng.to_device([M])[0]
    lo, ro, s, keep, disc = eng.svd(Md, float(cut), int(md), 1, absorb)
    assert keep == len(Sref)
    s0 = Sref[0]
    assert np.all(np.abs(s[:keep] - Sref) < 1e-13 * s0 + 1e-15 * s0 ** 2 / Sref)
    assert abs(disc - GOLD[tag + "_trunc"][0]) < 1e-13
    L, R = lo.cpu().numpy(), ro.cpu().numpy()
    tail = float(np.sum(s[keep:] ** 2))
    # the singular values below ~1e-8 s0 (and the vectors beside them) carry
    # the Gram route's eps s0^2/s error: an eigensolver whose residual is
    # ~n eps |G| (LAPACK's eigh as much as this Jacobi) mixes a kept vector
    # with a neighbour across a small gap, which costs ~1e-14 s0^2/s_keep of
    # reconstruction
    slack = 1e-10 * s0 + 1e-14 * s0 ** 2 / s[keep - 1]
    if absorb == 0:
        assert np.linalg.norm(L @ R - M) <= np.sqrt(tail) + slack
        assert np.max(np.abs(L.T @ L - np.eye(keep))) < 1e-13
    elif absorb == 1:
        assert np.linalg.norm(L @ R - M) <= np.sqrt(tail) + slack
        assert np.max(np.abs(R @ R.T - np.eye(keep))) < 1e-13
    else:
        S = s[:keep]
        assert np.linalg.norm((L * S) @ R - M) <= np.sqrt(tail) + slack
        bound = 1e-13 * max(1.0, (s0 / S[-1]) ** 2)
        side = L.T @ L if M.shape[0] <= M.shape[1] else R @ R.T
        assert np.max(np.abs(side - np.eye(keep))) < 1e-13
        other = R @ R.T if M.shape[0] <= M.shape[1] else L.T @ L
        assert np.max(np.abs(other - np.eye(keep))) < bound


def _theta(m, n, sv, seed):
    rng = np.random.default_rng(seed)
    r = len(sv)
    U, _ = np.linalg.qr(rng.standard_normal((m, r)))
    V, _ = np.linalg.qr(rng.standard_normal((n, r)))
    return (U * sv) @ V.T, U, V


def _subspace(eng, theta, k, start, kx, absorb, cutoff, prec):
    from dmrgpy_gb300 import _lib
    torch = __import__("torch")
    m, n = theta.shape
    th = eng.to_device([theta])[0]
    st = eng.to_device([start])[0] if start is not None else None
    lo = torch.empty(m * k, dtype=torch.float64, device=eng.device)
    ro = torch.empty(k * n, dtype=torch.float64, device=eng.device)
    s = np.zeros(k)
    keep = ctypes.c_int(0)
    disc = ctypes.c_double(0.0)
    ptr, size = eng.ws.get(eng.lib.dmrg_subspace_truncate_ex_workspace_bytes(prec, m, n, k))
    _lib.check("dmrg_subspace_truncate_ex", eng.lib.dmrg_subspace_truncate_ex(
        prec, m, n, k, th.data_ptr(), st.data_ptr() if st is not None else None, kx, absorb, 1, cutoff, 1,
        lo.data_ptr(), ro.data_ptr(), s.ctypes.data_as(_lib.P_double), ctypes.byref(keep), ctypes.byref(disc),
        ptr, size, eng.stream))
    kp = keep.value
    return lo[:m * kp].view(m, kp).cpu().numpy(), ro[:kp * n].view(kp, n).cpu().numpy(), s, kp, disc.value


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("absorb", [0, 1])
@pytest.mark.parametrize("cutoff", [0.0, 1e-9, 1e-6])
def test_subspace_route_exact_start(prec, absorb, cutoff):
    """With the exact singular vectors across the bond as the start (a
    converged sweep's warm start), the kept count, discarded weight and
    factors follow the reference's rule on the exact spectrum (oracle
    truncate).  The FP64 route decides every case; split-TF32 decides where
    the weight beyond the kept space clears the cutoff (cutoff 0 and 1e-9:
    keep = maxdim) and hands a binding cutoff (1e-6: the rule keeps 227 of
    256) to the FP64 route with DMRG_ERR_PRECISION."""
    from dmrgpy_gb300 import _lib
    m, n, k = 512, 640, 256
    sv = 0.97 ** np.arange(480)
    theta, U, V = _theta(m, n, sv, 1 + absorb)
    start = V[:, :k].T.copy() if absorb == 0 else U[:, :k].copy()
    eng = _eng("fp64" if prec == 0 else "tf32x3")
    kref, dref = O.truncate(sv, cutoff, k, 1)
    if prec == 1 and kref < k:
        with pytest.raises(_lib.DmrgError) as ex:
            _subspace(eng, theta, k, start, k, absorb, cutoff, prec)
        assert ex.value.status == _lib.DMRG_ERR_PRECISION
        return
    lo, ro, s, keep, disc = _subspace(eng, theta, k, start, k, absorb, cutoff, prec)
    assert keep == kref
    tol = 1e-11 if prec == 0 else 2e-5
    assert np.max(np.abs(s[:keep] - sv[:keep]) / sv[:keep]) < tol
    # split-TF32: with a cutoff the weight outside the kept space comes from
    # the residual |theta - lo ro|^2 (TF32 error squared); without one from
    # |theta|^2 - |C|^2 (TF32 error linear, ~1e-7)
    assert abs(disc - dref) < (1e-12 if prec == 0 else (1e-10 if cutoff > 0 else 2e-6))
    orth = lo.T @ lo if absorb == 0 else ro @ ro.T
    # split-TF32: the polar basis after its near-FP64 digit-Gram correction
    assert np.max(np.abs(orth - np.eye(keep))) < (1e-12 if prec == 0 else 2e-11)
    err = np.linalg.norm(lo @ ro - theta) ** 2 / np.sum(sv ** 2)
    assert abs(err - dref) < (1e-12 if prec == 0 else 1e-6)


@pytest.mark.parametrize("prec", [0, 1])
def test_subspace_route_growing_bond(prec):
    """A start with half the kept vectors (the bond grows): the other half is
    random, the basis stays orthonormal and the factorisation is consistent
    with its reported discarded weight, which stays close to the optimum."""
    m, n, k = 600, 600, 200
    sv = 0.96 ** np.arange(600)
    theta, U, V = _theta(m, n, sv, 9)
    eng = _eng("fp64" if prec == 0 else "tf32x3")
    start = V[:, :k // 2].T.copy()
    lo, ro, s, keep, disc = _subspace(eng, theta, k, start, k // 2, 0, 0.0, prec)
    assert keep == k
    # split-TF32: the polar basis after its near-FP64 Gram correction
    assert np.max(np.abs(lo.T @ lo - np.eye(keep))) < (1e-12 if prec == 0 else 2e-11)
    err = np.linalg.norm(lo @ ro - theta) ** 2 / np.sum(sv ** 2)
    assert abs(err - disc) < (1e-12 if prec == 0 else 1e-6)
    # one product with a half-random start: a NumPy model of the same step
    # (QR instead of the Ritz basis) captures the kept space to ~8x the
    # optimal discarded weight; sweeps then converge it
    _, dopt = O.truncate(sv, 0.0, k, 1)
    assert disc <= 20.0 * dopt + 1e-12


def test_sweeps_with_cutoff_keep_the_reference_counts():
    """FP64 and split-TF32 sweeps with the session default cutoff 1e-12 and
    maxdim 96 (S=1/2 Heisenberg, N=60, the subspace route taken from
    min(m, n) >= 128): central bonds reach maxdim, the others are bound by
    the cutoff.  For the two-site tensors of the last sweep the kept count
    and discarded weight are compared with the oracle's truncation of the
    same tensor (pyitensor/svd.py:108-151).
      FP64: exactly where maxdim binds, within one vector where the cutoff
      does; the discarded weight never below the optimal one and at most
      1e-11 (of the total weight) above it.
      split-TF32: a bond it decides itself keeps maxdim, which the oracle
      also keeps unless the weight beyond the TF32 subspace (which it
      reports) exceeds the optimal tail; every bond where the cutoff may bind
      is handed to the FP64 route and then matches as above.
    The FP64-refined energies of the two sweeps agree within 1e-9 per site
    (the split-TF32 states carry the ~1e-6 operator bias of split-TF32
    products, at a critical chain with bond dimensions that move with the
    cutoff)."""
    from golden_data import terms_heisenberg
    from dmrgpy_gb300 import engine as EG
    from dmrgpy_gb300 import mpo as M
    from dmrgpy_gb300 import mps as MP
    from dmrgpy_gb300.engine import Engine
    n = 60
    W, real = M.build_mpo([2] * n, terms_heisenberg(n))
    sched = [32, 64, 96, 96, 96]
    out = {}
    old = EG.SUBSPACE_MIN_DIM
    EG.SUBSPACE_MIN_DIM = 128
    try:
        for prec in ("fp64", "tf32x3"):
            eng = Engine(W, real=real, precision=prec)
            np.random.seed(3)
            A = eng.to_device(MP.random_arrays([2] * n, 8))
            eng.canonicalize_right_to_left_of(A)
            eng.dmrg(A, sched[:-1], 1e-12, 2)
            seen = []

            def hook(theta, cutoff, maxdim, keep, disc):
                # bonds of the subspace route (maxdim below min(m, n))
                if min(theta.shape) > 96:
                    seen.append((theta.detach().cpu().numpy().copy(), keep, disc))
            eng.theta_hook = hook
            eng.sweep(A, sched[-1], 1e-12, 2)
            eng.theta_hook = None
            dims = [a.shape[2] for a in A[:-1]]
            out[prec] = (eng.energy_fp64(A), seen[::2], eng.stats.fp64_truncations, dims)
    finally:
        EG.SUBSPACE_MIN_DIM = old
    e64, seen64, _, dims64 = out["fp64"]
    e32, seen32, nfp64, dims32 = out["tf32x3"]
    assert abs(e32 - e64) / n <= 1e-9, (e32, e64)
    assert nfp64 > 0
    # maxdim binds in the middle of the chain, the cutoff elsewhere
    for dims in (dims64, dims32):
        assert max(dims) == 96 and min(d for d in dims[10:50]) < 96, dims
    nbind = 0
    for prec, seen in (("fp64", seen64), ("tf32x3", seen32)):
        assert len(seen) >= 5
        for th, keep, disc in seen:
            _, S, _, kref, dref = O.svd_truncated(th, 1e-12, 96, 1)
            nbind += kref == 96
            if prec == "tf32x3" and keep == 96 and disc > 1e-11:
                # decided in split-TF32: maxdim kept because the weight beyond
                # its subspace exceeds the cutoff; never fewer than the oracle
                assert kref <= 96 and disc >= dref * (1 - 1e-6), (keep, kref, disc, dref)
                continue
            assert abs(keep - kref) <= (0 if kref == 96 else 1), (prec, keep, kref)
            # the subspace of one product with the previous basis falls short
            # of the optimal one by a few 1e-12 of the total weight at this
            # critical chain (never better than it)
            # (one vector more than the oracle keeps lowers it by that
            # vector's weight; the oracle's own Gram weights carry ~1e-14)
            extra = float(np.sum(S[kref:keep] ** 2) / np.sum(S ** 2)) if keep > kref else 0.0
            assert dref - extra - 2e-14 <= disc <= dref + 1e-11, (prec, disc, dref)
    assert nbind > 0
