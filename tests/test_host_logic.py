"""Host-side logic of the product: the term -> MPO compiler, the initial
state draw, the dmrgpy registration tag.  Checked against the reference's
own outputs (tests/golden) and the oracle."""
import numpy as np
import pytest

import oracle as O
from golden_data import fixtures, meta, terms_heisenberg, terms_tfim
from dmrgpy_gb300 import mpo as M
from dmrgpy_gb300 import mps as MP
from dmrgpy_gb300 import sites as S
from dmrgpy_gb300.backend import BACKEND_TAG

FX = fixtures()
META = meta()


@pytest.mark.parametrize("key", ["hubbard4", "spinless8", "heis6", "heis_s1_5", "tfim6", "xxz8"])
def test_mpo_compiler_reproduces_reference_hamiltonian(key):
    W, real = M.build_mpo(META["types"][key], META["terms"][key])
    assert real, "these Hamiltonians compile to a real MPO"
    assert np.max(np.abs(M.mpo_to_dense(W) - FX["mpo_dense_" + key])) < 1e-12


def test_mpo_bond_dimensions_are_optimal_for_nearest_neighbour_models():
    W, _ = M.build_mpo([2] * 10, terms_heisenberg(10))
    assert max(w.shape[3] for w in W) == 5
    W, _ = M.build_mpo([2] * 10, terms_tfim(10))
    assert max(w.shape[3] for w in W) == 3
    W, _ = M.build_mpo(META["types"]["hubbard4"], META["terms"]["hubbard4"])
    assert max(w.shape[3] for w in W) == 6


def test_complex_hamiltonian_stays_complex_and_long_range_is_compressed():
    n = 6
    terms = [(0.3 + 0j, [("Sy", 2)]), (1.0 + 0j, [("Sx", 1), ("Sz", 3)])]
    W, real = M.build_mpo([2] * n, terms)
    assert not real
    assert np.max(np.abs(M.mpo_to_dense(W) - O.dense_hamiltonian([2] * n, terms))) < 1e-12
    rng = np.random.default_rng(1)
    terms = [(complex(rng.normal()), [("Sz", i), ("Sz", j)]) for i in range(1, 11) for j in range(i + 1, 11)]
    W, real = M.build_mpo([2] * 10, terms)
    assert real
    assert np.max(np.abs(M.mpo_to_dense(W) - O.dense_hamiltonian([2] * 10, terms))) < 1e-10
    assert max(w.shape[3] for w in W) <= 12


def test_site_operators_match_reference_algebra():
    for code in (2, 3, 4, 5, 6):
        sx, sy, sz = S.op(code, "Sx"), S.op(code, "Sy"), S.op(code, "Sz")
        s = (S.dim(code) - 1) / 2
        assert np.allclose(sx @ sx + sy @ sy + sz @ sz, s * (s + 1) * np.eye(S.dim(code)))
        assert np.allclose(sx @ sy - sy @ sx, 1j * sz)
    for code, names in ((1, ("Cup", "Cdn", "Aup", "Adn", "F", "Fup", "Nup", "Ndn", "Sz", "Sp")),
                        (0, ("C", "Cdag", "A", "Adag", "N", "F"))):
        for nm in names:
            assert np.allclose(S.op(code, nm), O.site_op(code, nm).T), (code, nm)
    with pytest.raises(ValueError):
        S.op(2, "Cup")


def test_random_initial_state_uses_the_reference_draws():
    np.random.seed(7)
    arrays = MP.random_arrays([2] * 6, 8)
    psi = O.OracleMPS(arrays, center=1)
    psi.position(6)
    psi.normalize()
    for i in range(6):
        assert np.max(np.abs(psi.A[i] - FX["rmps_A%d" % (i + 1)])) < 1e-12


def test_backend_tag_routes_like_python_but_registers_separately():
    assert BACKEND_TAG == "python"
    assert BACKEND_TAG in (2, 3, "python")
    reg = {"python": "py"}
    reg[BACKEND_TAG] = "gb300"
    assert reg["python"] == "py" and reg[BACKEND_TAG] == "gb300"


def test_host_bond_entropy_matches_oracle():
    np.random.seed(3)
    psi = O.random_mps([2] * 8, 6)
    for b in (2, 4, 6):
        assert abs(MP.bond_entropy(psi.A, b) - O.bond_entropy(psi, b)) < 1e-10
