"""Batched sweeps of many chains with uneven bond dimensions (grouped
launches, graph-replayed Lanczos) against the single-chain FP64 engine from
the same seeded states, against exact diagonalisation (oracle dense
Hamiltonians), and the dE/dh of every chain through the adjoint pass against
finite differences of exact energies."""
import numpy as np
import pytest

from golden_data import terms_tfim
from oracle import dmrg_oracle as O

pytestmark = pytest.mark.gpu


def _chains(n, count, seed):
    rng = np.random.default_rng(seed)
    hs = rng.uniform(0.5, 1.5, count)
    chis = rng.choice([4, 8, 16, 32], count)
    return hs, chis


def _batch(n, hs, chis, sweeps, use_graphs=True):
    from dmrgpy_gb300 import mpo as M
    from dmrgpy_gb300.batch import BatchEngine
    Ws = [M.build_mpo([2] * n, terms_tfim(n, 1.0, h))[0] for h in hs]
    be = BatchEngine(Ws, real=True, use_graphs=use_graphs)
    As = be.random_states([2] * n, 4, seeds=[100 + i for i in range(len(hs))])
    be.canonicalize(As)
    e = be.dmrg(As, [int(c) for c in chis], sweeps)
    return be, As, e


def _single(n, h, chi, seed, sweeps):
    from dmrgpy_gb300 import mpo as M
    from dmrgpy_gb300 import mps as MP
    from dmrgpy_gb300.engine import Engine
    W, real = M.build_mpo([2] * n, terms_tfim(n, 1.0, h))
    eng = Engine(W, real=real)
    np.random.seed(seed)
    A = eng.to_device(MP.random_arrays([2] * n, 4))
    eng.canonicalize_right_to_left_of(A)
    return eng.dmrg(A, [chi] * sweeps, 0.0), eng.energy_fp64(A)


def test_batch_matches_single_chain_engine():
    n, sweeps = 12, 6
    hs, chis = _chains(n, 6, 3)
    be, As, e = _batch(n, hs, chis, sweeps)
    for p in range(len(hs)):
        e1, _ = _single(n, hs[p], int(chis[p]), 100 + p, sweeps)
        assert abs(e[p] - e1) < 1e-9 * n, (p, e[p], e1)
        assert max(a.shape[2] for a in As[p][:-1]) <= chis[p]


def test_batch_reaches_exact_ground_states_and_graphs_change_nothing():
    n, sweeps = 10, 8
    hs = np.array([0.6, 0.9, 1.0, 1.3])
    chis = np.array([32, 32, 32, 32])
    _, _, e_graph = _batch(n, hs, chis, sweeps, use_graphs=True)
    _, _, e_plain = _batch(n, hs, chis, sweeps, use_graphs=False)
    for p, h in enumerate(hs):
        e0 = np.linalg.eigvalsh(O.dense_hamiltonian([2] * n, terms_tfim(n, 1.0, h)))[0]
        assert abs(e_graph[p] - e0) / n < 1e-10
        assert abs(e_graph[p] - e_plain[p]) < 1e-12 * n


def test_batch_field_gradients_match_finite_differences():
    from dmrgpy_gb300.gradients import CouplingProblem
    n, sweeps = 8, 8
    hs = np.array([0.55, 0.8, 1.2])
    chis = np.array([16, 16, 16])
    be, As, e = _batch(n, hs, chis, sweeps)
    delta = 1e-5
    for p, h in enumerate(hs):
        prob = CouplingProblem([2] * n, terms_tfim(n, 1.0, h))
        _, g = prob.gradient(As[p])
        nf = n
        dedh = sum(g[-nf:]).real

        def e0(hh):
            return np.linalg.eigvalsh(O.dense_hamiltonian([2] * n, terms_tfim(n, 1.0, hh)))[0]
        fd = (e0(h + delta) - e0(h - delta)) / (2 * delta)
        assert abs(dedh - fd) < 1e-6 * max(1.0, abs(fd)), (p, dedh, fd)
