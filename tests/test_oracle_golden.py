"""Pin the CPU oracle against outputs of the reference itself
(tests/golden, produced by tests/golden/make_golden.py) and against the
reference test-suite's own golden values."""
import numpy as np
import pytest

import oracle as O
from golden_data import fixtures, meta, terms_heisenberg, terms_xxz

FX = fixtures()
META = meta()


@pytest.mark.parametrize("tag", ["mv_heis", "mv_edge", "mv_s1", "mv_hub"])
def test_heff2_matvec_matches_reference(tag):
    y = O.heff2_matvec(FX[tag + "_L"], FX[tag + "_Wi"], FX[tag + "_Wj"], FX[tag + "_R"], FX[tag + "_theta"])
    ref = FX[tag + "_y"]
    assert np.max(np.abs(y - ref)) / np.max(np.abs(ref)) < 1e-12


@pytest.mark.parametrize("tag", ["mv_heis", "mv_edge", "mv_s1", "mv_hub"])
def test_environment_and_one_site_matvec_match_reference(tag):
    Lnext = O.extend_left(FX[tag + "_L"], FX[tag + "_Wi"], FX[tag + "_Ai"])
    ref = FX[tag + "_Lnext"]
    assert np.max(np.abs(Lnext - ref)) <= 1e-12 * np.max(np.abs(ref))
    Rprev = O.extend_right(FX[tag + "_R"], FX[tag + "_Wj"], FX[tag + "_Aj"])
    ref = FX[tag + "_Rprev"]
    assert np.max(np.abs(Rprev - ref)) <= 1e-12 * np.max(np.abs(ref))
    y1 = O.heff1_matvec(FX[tag + "_Lnext"], FX[tag + "_Wj"], FX[tag + "_R"], FX[tag + "_A1"])
    ref = FX[tag + "_y1"]
    assert np.max(np.abs(y1 - ref)) <= 1e-12 * np.max(np.abs(ref))


def test_random_mps_reproduces_reference_draw():
    np.random.seed(7)
    psi = O.random_mps([2] * 6, 8)
    for i in range(6):
        ref = FX["rmps_A%d" % (i + 1)]
        assert psi.A[i].shape == ref.shape
        assert np.max(np.abs(psi.A[i] - ref)) < 1e-12


@pytest.mark.parametrize("tag,cut,md", [("a", 1e-12, None), ("b", 1e-8, 30), ("c", 0.0, 10)])
def test_truncated_svd_matches_reference(tag, cut, md):
    M = FX["svd_M"]
    U, S, Vh, keep, disc = O.svd_truncated(M, cut, md, 1)
    Sref = FX["svd_%s_S" % tag]
    assert keep == len(Sref)
    assert np.max(np.abs(S[:keep] - Sref)) < 1e-13
    assert abs(disc - FX["svd_%s_trunc" % tag][0]) < 1e-13
    rec = (U * S[None, :keep]) @ Vh
    assert np.max(np.abs(rec - FX["svd_%s_rec" % tag])) < 1e-12


def test_truncate_rule_edge_cases():
    s = np.array([1.0, 0.5, 0.1, 1e-7, 1e-9])
    assert O.truncate(s, 1e-12, None, 1)[0] == 3
    assert O.truncate(s, 1e-16, None, 1)[0] == 4
    assert O.truncate(s, 1e-12, 2, 1)[0] == 2
    assert O.truncate(s, 0.5, None, 3)[0] == 3      # mindim floor
    assert O.truncate(np.zeros(4), 1e-12, None, 1) == (1, 0.0)
    keep, disc = O.truncate(s, 1e-2, None, 1)
    p = s ** 2 / np.sum(s ** 2)
    assert keep == 2 and abs(disc - p[2:].sum()) < 1e-15


def test_lanczos_matches_reference():
    A, v0 = FX["lz_A"], FX["lz_v0"]
    e, v, k = O.lanczos_ground_state(lambda x: A @ x, v0, niter=200)
    assert abs(e - FX["lz_E"][0]) < 1e-10
    assert abs(abs(np.vdot(v, FX["lz_v"])) - 1) < 1e-8
    assert abs(e - np.linalg.eigvalsh(A)[0]) < 1e-10


@pytest.mark.parametrize("key", ["hubbard4", "spinless8", "heis6", "heis_s1_5", "tfim6", "xxz8"])
def test_term_compiler_matches_reference_dense(key):
    types = META["types"][key]
    terms = META["terms"][key]
    dense = O.dense_hamiltonian(types, terms)
    ref = FX["mpo_dense_" + key]
    assert np.max(np.abs(dense - ref)) < 1e-12
    W = O.build_mpo(types, terms)
    assert np.max(np.abs(O.mpo_to_dense(W) - ref)) < 1e-10 * max(1.0, np.abs(ref).max())
    assert [w.shape[0] for w in W] + [W[-1].shape[3]] == list(FX["mpo_wdims_" + key])


def _gs(types, terms, maxm, nsweeps, seed):
    np.random.seed(seed)
    dims = [O.site_dim(c) for c in types]
    W = O.build_mpo(types, terms)
    psi = O.random_mps(dims, maxm)
    e = O.dmrg(psi.A, W, [maxm] * nsweeps, 1e-12, 2)
    psi.center = 1
    return e, psi


@pytest.mark.parametrize("tag", ["heis12_chi64", "tfim4", "hub4_chi32", "spinless8_chi32", "s1_heis10_chi32",
                                 "s1_heis8_chi81"])
def test_ground_state_energies_match_reference(tag):
    r = META["ground_states"][tag]
    key = {"heis12_chi64": None, "tfim4": None, "hub4_chi32": "hubbard4",
           "spinless8_chi32": "spinless8", "s1_heis10_chi32": None, "s1_heis8_chi81": None}[tag]
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
        types, terms = META["types"][key], META["terms"][key]
    e, psi = _gs(types, terms, r["maxm"], r["nsweeps"], r["seed"])
    n = len(types)
    assert abs(e - r["E"]) / n < 1e-10
    if "E_ed" in r:
        assert abs(e - r["E_ed"]) / n < 1e-10
    if "S_vN" in r:
        b = n // 2
        assert abs(O.bond_entropy(psi, b) - r["S_vN"]) < 1e-8


def test_reference_suite_golden_values():
    """tests/test_spin_chain.py:45-66 (TFIM N=4) and tests/reference_data.py:15-17
    (Heisenberg N=10 DMRG / ED) of the reference repository."""
    types = [2] * 4
    terms = [(-1.0 + 0j, [("Sz", i), ("Sz", i + 1)]) for i in range(1, 4)] + \
            [(1.0 + 0j, [("Sx", i)]) for i in range(1, 5)]
    e, _ = _gs(types, terms, 16, 6, 0)
    assert abs(e - (-2.0941996592125895)) < 1e-8
    e, _ = _gs([2] * 10, terms_heisenberg(10), 30, 8, 0)
    assert abs(e - (-4.258035207282873)) < 1e-8
    assert abs(e - (-4.25803520681935)) < 1e-6
    e, _ = _gs([2] * 2, terms_heisenberg(2), 8, 2, 0)
    assert abs(e - (-0.75)) < 1e-10


@pytest.mark.parametrize("nc", [2, 1])
def test_tdvp_matches_reference(nc):
    n = 8
    W = O.build_mpo([2] * n, terms_xxz(n, 0.5))
    A = []
    for i in range(n):
        a = np.zeros((1, 2, 1), dtype=complex)
        a[0, i % 2, 0] = 1.0
        A.append(a)
    if nc == 1:
        O.tdvp_step(A, W, 0.1, 1e-12, 16, 50, 2)
    for step in range(3):
        O.tdvp_step(A, W, 0.05, 1e-12, 16, 50, nc)
        v = O.mps_to_dense(A)
        ref = FX["tdvp%d_step%d" % (nc, step)]
        assert abs(abs(np.vdot(v, ref)) - 1.0) < 1e-9
        assert np.max(np.abs(v - ref)) < 1e-7


def test_config1_heisenberg32_matches_reference():
    r = META["ground_states"]["heis32_chi64"]
    e, psi = _gs([2] * 32, terms_heisenberg(32), 64, 10, 0)
    assert abs(e - r["E"]) / 32 < 1e-10
    assert abs(O.bond_entropy(psi, 16) - r["S_vN"]) < 1e-8
