"""GPU parity of the FP64 path against the reference (tests/golden) and the
CPU oracle, through the C ABI.

Tolerances: FP64 matvec / environments 1e-12 relative (the bar the reference
sets for its own alternative matvec kernels, examples/pyitensor/
selftest_kernels.py:50-88); converged energies |dE|/N <= 1e-10 against the
reference python backend and its ED; entropies within 1e-8."""
import numpy as np
import pytest

import oracle as O
from golden_data import fixtures, meta, terms_heisenberg, terms_xxz

pytestmark = pytest.mark.gpu

FX = fixtures()
META = meta()


def _torch():
    import torch
    return torch


def _engine(W, real):
    from dmrgpy_gb300.engine import Engine
    return Engine(W, real=real)


def _dev(eng, a):
    return eng.to_device([a])[0]


def _relerr(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("tag", ["mv_heis", "mv_edge", "mv_s1", "mv_hub"])
def test_two_site_matvec_matches_reference(tag):
    eng = _engine([FX[tag + "_Wi"], FX[tag + "_Wj"]], real=False)
    L, R, th = (_dev(eng, FX[tag + k]) for k in ("_L", "_R", "_theta"))
    h = eng.heff2(L, eng.W[0], eng.W[1], R, th.shape)
    y = eng.apply(h, th).cpu().numpy()
    assert _relerr(y, FX[tag + "_y"]) < 1e-12


@pytest.mark.parametrize("tag", ["mv_heis", "mv_edge", "mv_s1", "mv_hub"])
def test_real_arithmetic_matvec_matches_oracle(tag):
    """Same operator with the real MPO of the product compiler's form: take
    the real parts of environments/MPO and compare against the oracle."""
    L, Wi, Wj, R, th = (np.ascontiguousarray(FX[tag + k].real) for k in ("_L", "_Wi", "_Wj", "_R", "_theta"))
    ref = O.heff2_matvec(L, Wi, Wj, R, th)
    eng = _engine([Wi, Wj], real=True)
    h = eng.heff2(_dev(eng, L), eng.W[0], eng.W[1], _dev(eng, R), th.shape)
    y = eng.apply(h, _dev(eng, th)).cpu().numpy()
    assert _relerr(y, ref) < 1e-12


@pytest.mark.parametrize("tag", ["mv_heis", "mv_s1", "mv_hub"])
def test_environments_and_one_site_matvec_match_reference(tag):
    eng = _engine([FX[tag + "_Wi"], FX[tag + "_Wj"]], real=False)
    Lnext = eng.env_left(_dev(eng, FX[tag + "_L"]), eng.W[0], _dev(eng, FX[tag + "_Ai"])).cpu().numpy()
    assert _relerr(Lnext, FX[tag + "_Lnext"]) < 1e-12
    Rprev = eng.env_right(_dev(eng, FX[tag + "_R"]), eng.W[1], _dev(eng, FX[tag + "_Aj"])).cpu().numpy()
    assert _relerr(Rprev, FX[tag + "_Rprev"]) < 1e-12
    A1 = _dev(eng, FX[tag + "_A1"])
    h = eng.heff1(_dev(eng, FX[tag + "_Lnext"]), eng.W[1], _dev(eng, FX[tag + "_R"]), A1.shape)
    assert _relerr(eng.apply(h, A1).cpu().numpy(), FX[tag + "_y1"]) < 1e-12
    # zero-site operator against the oracle
    Ln, Rn = FX[tag + "_Lnext"], FX[tag + "_Rprev"]
    if Ln.shape[1] == Rn.shape[1]:
        C = np.random.default_rng(0).standard_normal((Ln.shape[0], Rn.shape[0])) + 0j
        h0 = eng.heff0(_dev(eng, Ln), _dev(eng, Rn), C.shape)
        assert _relerr(eng.apply(h0, _dev(eng, C)).cpu().numpy(), O.heff0_matvec(Ln, Rn, C)) < 1e-12


@pytest.mark.parametrize("tag,cut,md", [("a", 1e-12, None), ("b", 1e-8, 30), ("c", 0.0, 10)])
@pytest.mark.parametrize("absorb", [0, 1])
def test_truncated_svd_matches_reference(tag, cut, md, absorb):
    M = FX["svd_M"]
    eng = _engine([np.zeros((1, 2, 2, 1))], real=False)
    lo, ro, s, keep, disc = eng.svd(_dev(eng, M), cut, md or 0, 1, absorb)
    Sref = FX["svd_%s_S" % tag]
    assert keep == len(Sref)
    # the reference takes small singular values from the Gram matrix
    # (pyitensor/svd.py:108-151), accurate only to ~eps*s_max^2/s; the
    # one-sided Jacobi values are more accurate, so compare within that bound
    assert np.all(np.abs(s[:keep] - Sref) < 1e-13 + 1e-15 / Sref)
    assert abs(disc - FX["svd_%s_trunc" % tag][0]) < 1e-13
    rec = lo.cpu().numpy() @ ro.cpu().numpy()
    # the reference forms Vh = W^H M / S (pyitensor/svd.py:140-146), which
    # amplifies its Gram-route error on the smallest kept values; compare
    # both reconstructions with the input matrix instead
    tail = np.sum(Sref[keep:] ** 2) if keep < len(Sref) else 0.0
    ref_err = np.max(np.abs(FX["svd_%s_rec" % tag] - M))
    assert np.max(np.abs(rec - M)) <= max(1e-12, 2 * ref_err, 2 * np.sqrt(tail) + 1e-12)
    if absorb == 0:
        U = lo.cpu().numpy()
        assert np.max(np.abs(U.conj().T @ U - np.eye(keep))) < 1e-12
    else:
        # the orthonormal factor is formed as Y/sigma, accurate to ~eps*s_max/s
        V = ro.cpu().numpy()
        assert np.max(np.abs(V @ V.conj().T - np.eye(keep))) < 1e-13 * max(1.0, s[0] / s[keep - 1])


@pytest.mark.parametrize("shape", [(40, 60), (60, 40), (3, 50), (50, 3), (1, 7), (128, 128), (300, 200)])
def test_svd_shapes_real(shape):
    rng = np.random.default_rng(sum(shape))
    M = rng.standard_normal(shape)
    eng = _engine([np.zeros((1, 2, 2, 1))], real=True)
    lo, ro, s, keep, disc = eng.svd(_dev(eng, M), 0.0, 0, 1, 0)
    ref = np.linalg.svd(M, compute_uv=False)
    assert np.max(np.abs(s - ref)) < 1e-12 * ref[0]
    assert np.max(np.abs(lo.cpu().numpy() @ ro.cpu().numpy() - M)) < 1e-12 * ref[0]


def test_lanczos_matches_dense_ground_state():
    tag = "mv_heis"
    L, Wi, Wj, R, th = (FX[tag + k] for k in ("_L", "_Wi", "_Wj", "_R", "_theta"))
    n = th.size
    dense = np.column_stack([O.heff2_matvec(L, Wi, Wj, R, e.reshape(th.shape)).reshape(-1)
                             for e in np.eye(n, dtype=complex)])
    e0 = np.linalg.eigvalsh((dense + dense.conj().T) / 2)[0]
    eng = _engine([Wi, Wj], real=False)
    x = _dev(eng, th).contiguous()
    h = eng.heff2(_dev(eng, L), eng.W[0], eng.W[1], _dev(eng, R), th.shape)
    e, k = eng.ground(h, x, 200)
    assert abs(e - e0) < 1e-10 * max(1, abs(e0))
    v = x.cpu().numpy().reshape(-1)
    assert abs(np.linalg.norm(v) - 1) < 1e-12
    r = dense @ v - e * v
    assert np.linalg.norm(r) < 1e-5


def _gs(types, terms, maxm, nsweeps, seed):
    from dmrgpy_gb300 import Chain
    np.random.seed(seed)
    c = Chain(types)
    c.set_sweep_params(maxm, nsweeps, 1e-12, 0.0)
    c.set_hamiltonian(terms)
    e = c.gs_energy()
    return e, c


@pytest.mark.parametrize("tag", ["heis12_chi64", "tfim4", "hub4_chi32", "spinless8_chi32", "s1_heis10_chi32",
                                 "s1_heis8_chi81"])
def test_ground_state_energy_matches_reference_and_ed(tag):
    r = META["ground_states"][tag]
    if tag == "heis12_chi64":
        types, terms = [2] * 12, terms_heisenberg(12)
    elif tag == "tfim4":
        types = [2] * 4
        terms = [(-1.0 + 0j, [("Sz", i), ("Sz", i + 1)]) for i in range(1, 4)] + \
                [(1.0 + 0j, [("Sx", i)]) for i in range(1, 5)]
    elif tag == "s1_heis10_chi32":
        types, terms = [3] * 10, terms_heisenberg(10)
    elif tag == "s1_heis8_chi81":
        types, terms = [3] * 8, terms_heisenberg(8)
    else:
        key = {"hub4_chi32": "hubbard4", "spinless8_chi32": "spinless8"}[tag]
        types, terms = META["types"][key], META["terms"][key]
    e, c = _gs(types, terms, r["maxm"], r["nsweeps"], r["seed"])
    n = len(types)
    assert abs(e - r["E"]) / n <= 1e-10
    if "E_ed" in r:
        assert abs(e - r["E_ed"]) / n <= 1e-10
    if "S_vN" in r:
        # observables are compared where the bond dimension is exact (no
        # truncation): at a truncating chi two independent DMRG runs agree
        # in energy to second order but in observables only to first order
        exact = r["maxm"] >= max(np.prod([c.dims[0]] * (n // 2)), 1) or tag == "heis12_chi64"
        tol = 1e-8 if exact else 1e-6
        assert abs(c.bond_entropy(c.gs_wavefunction(), n // 2) - r["S_vN"]) < tol
        szsz = c.vev([(1.0 + 0j, [("Sz", 1), ("Sz", n)])], c.gs_wavefunction()).real
        assert abs(szsz - r["szsz_1N"]) < tol


def test_config1_heisenberg32_chi64_matches_reference():
    r = META["ground_states"]["heis32_chi64"]
    e, c = _gs([2] * 32, terms_heisenberg(32), 64, 10, 0)
    assert abs(e - r["E"]) / 32 <= 1e-10
    assert abs(c.bond_entropy(c.gs_wavefunction(), 16) - r["S_vN"]) < 1e-8
    szsz = c.vev([(1.0 + 0j, [("Sz", 1), ("Sz", 32)])], c.gs_wavefunction()).real
    assert abs(szsz - r["szsz_1N"]) < 1e-8


@pytest.mark.parametrize("nc", [2, 1])
def test_tdvp_matches_reference(nc):
    from dmrgpy_gb300.engine import Engine
    from dmrgpy_gb300 import mpo as M
    n = 8
    W, _ = M.build_mpo([2] * n, terms_xxz(n, 0.5))
    eng = Engine(W, real=False)
    A = []
    for i in range(n):
        a = np.zeros((1, 2, 1), dtype=complex)
        a[0, i % 2, 0] = 1.0
        A.append(a)
    A = eng.to_device(A)
    if nc == 1:
        eng.tdvp_step(A, 0.1, 1e-12, 16, 50, 2)
    for step in range(3):
        eng.tdvp_step(A, 0.05, 1e-12, 16, 50, nc)
        v = O.mps_to_dense(eng.to_host(A))
        ref = FX["tdvp%d_step%d" % (nc, step)]
        assert abs(abs(np.vdot(v, ref)) - 1.0) < 1e-9
        assert np.max(np.abs(v - ref)) < 1e-7
