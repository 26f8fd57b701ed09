"""Host-side checks of the coupling map behind the energy gradients: the
automaton MPO is affine in the term coefficients, and the block that the map
names for term t is exactly dH/dc_t (compared as dense matrices with the
oracle's own term-by-term Hamiltonian, oracle.dense_hamiltonian)."""
import numpy as np

from dmrgpy_gb300 import mpo as M
from golden_data import terms_heisenberg, terms_tfim, terms_xxz
from oracle import dmrg_oracle as O


def _dense(W):
    return M.mpo_to_dense(W)


def _cases():
    rng = np.random.default_rng(5)
    n = 5
    xxz = terms_xxz(n, 0.5, fields=list(rng.uniform(-0.1, 0.1, n)))
    dm = [(0.3 + 0j, [("Sx", 1), ("Sy", 2)]), (-0.3 + 0j, [("Sy", 1), ("Sx", 2)])]  # DM term: complex MPO
    hub = [(complex(-1.0), [("Cdagup", i), ("Cup", i + 1)]) for i in range(1, 3)]
    hub += [(complex(-1.0), [("Cdagup", i + 1), ("Cup", i)]) for i in range(1, 3)]
    hub += [(complex(4.0), [("Nup", i), ("Ndn", i)]) for i in range(1, 4)]
    return [([2] * n, xxz), ([2] * 6, terms_tfim(6, 1.0, 0.7)), ([3] * 4, terms_heisenberg(4)),
            ([2] * 3, terms_heisenberg(3) + dm), ([1] * 3, hub)]


def test_map_blocks_are_term_derivatives():
    for types, terms in _cases():
        W, real, cmap = M.build_mpo(types, terms, coupling_map=True)
        H = _dense(W)
        assert np.allclose(H, O.dense_hamiltonian(types, terms), atol=1e-12)
        for t, (coef, factors) in enumerate(terms):
            site, ls, rs, Mt, factor = cmap[t]
            c2 = [c for c, _ in terms]
            c2[t] = c2[t] + 1.0
            W2, _, _ = M.build_mpo(types, [(c, f) for c, (_, f) in zip(c2, terms)], coupling_map=True)
            dH = _dense(W2) - H
            want = O.dense_hamiltonian(types, [(1.0 + 0j, factors)])
            assert np.allclose(dH, want, atol=1e-12), (types, t)
            # the map's block is the only change
            diff = [np.asarray(w2, dtype=complex) - np.asarray(w, dtype=complex) for w, w2 in zip(W, W2)]
            for i, dd in enumerate(diff):
                blk = np.zeros_like(dd)
                if i == site:
                    blk[ls, :, :, rs] = factor * Mt if not real else (factor * Mt).real
                assert np.allclose(dd, blk, atol=1e-13), (types, t, i)


def test_zero_coefficients_keep_their_block():
    terms = terms_tfim(4, 1.0, 0.0)
    W, real, cmap = M.build_mpo([2] * 4, terms, coupling_map=True)
    assert all(e is not None for e in cmap)
    W0, _ = M.build_mpo([2] * 4, terms)
    assert np.allclose(_dense(W), _dense(W0), atol=1e-13)
