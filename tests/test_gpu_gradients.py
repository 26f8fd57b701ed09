"""Energy gradients with respect to Hamiltonian couplings through the adjoint
of the environment chain (dmrg_env_gradient), against:
  * the contraction identity sum G_i . W_i = <psi|H|psi> at every site,
  * <h_t> on the exact ground state (Hellmann-Feynman, dense ED via the oracle),
  * central finite differences (delta = 1e-5) of exact ground-state energies,
  * torch.autograd through CouplingEnergy.
The reference has no derivative features, so these are the oracle."""
import numpy as np
import pytest

from golden_data import terms_heisenberg, terms_tfim
from oracle import dmrg_oracle as O

pytestmark = pytest.mark.gpu


def _ground(types, terms, chi, seed, sweeps=8):
    from dmrgpy_gb300 import mps as MP
    from dmrgpy_gb300.gradients import CouplingProblem
    prob = CouplingProblem(types, terms)
    eng = prob.engine
    np.random.seed(seed)
    A = eng.to_device(MP.random_arrays([O.site_dim(t) for t in types], min(chi, 8)))
    eng.canonicalize_right_to_left_of(A)
    e = prob.ground_state(A, [chi] * sweeps, [1e-14] * sweeps)
    return prob, A, e


def _ed(types, terms):
    H = O.dense_hamiltonian(types, terms)
    w, v = np.linalg.eigh(H)
    return w[0], v[:, 0]


def test_contraction_identity_every_site_real_and_complex():
    import torch
    from dmrgpy_gb300 import mps as MP
    from dmrgpy_gb300.gradients import CouplingProblem
    n = 7
    dm = [(0.3 + 0j, [("Sx", i), ("Sy", i + 1)]) for i in range(1, n)]
    dm += [(-0.3 + 0j, [("Sy", i), ("Sx", i + 1)]) for i in range(1, n)]
    for terms in (terms_heisenberg(n), terms_heisenberg(n) + dm):
        prob = CouplingProblem([2] * n, terms)
        eng = prob.engine
        np.random.seed(3)
        A = eng.to_device(MP.random_arrays([2] * n, 6))
        e, G = eng.mpo_gradients(A)
        for g, w in zip(G, eng.W):
            assert abs(complex(torch.sum(g * w).item()) - e) < 1e-12 * max(1.0, abs(e))
        psi = MP.MPS(eng.to_host(A), center=1)
        dense = O.mps_to_dense(psi.tensors)
        H = O.dense_hamiltonian([2] * n, terms)
        want = np.vdot(dense, H @ dense).real / np.vdot(dense, dense).real
        assert abs(e - want) < 1e-12 * abs(want)


@pytest.mark.parametrize("case", ["tfim", "heis_random_j"])
def test_term_gradients_match_ed_expectations(case):
    rng = np.random.default_rng(7)
    n = 10
    if case == "tfim":
        types, terms = [2] * n, terms_tfim(n, 1.0, 0.8)
    else:
        js = rng.uniform(0.5, 1.5, n - 1)
        types = [2] * n
        terms = [(complex(js[i - 1]), [(op, i), (op, i + 1)]) for i in range(1, n) for op in ("Sx", "Sy", "Sz")]
    prob, A, e = _ground(types, terms, 32, 1)
    e_fp, grad = prob.gradient(A)
    e0, v0 = _ed(types, terms)
    assert abs(e_fp - e0) / n < 1e-10
    for t, (c, f) in enumerate(terms):
        ht = O.dense_hamiltonian(types, [(1.0 + 0j, f)])
        want = np.vdot(v0, ht @ v0)
        # a derivative at a converged DMRG state is first order in the state
        # error (the energy is second order), hence the looser bar
        assert abs(grad[t] - want) < 1e-6, (t, grad[t], want)


def test_field_gradient_matches_finite_differences_and_autograd():
    import torch
    from dmrgpy_gb300.gradients import CouplingEnergy
    n, h = 10, 0.9
    types = [2] * n

    def terms_of(hh):
        return terms_tfim(n, 1.0, hh)

    prob, A, e = _ground(types, terms_of(h), 32, 2)
    nfield = n
    field_idx = list(range(len(terms_of(h)) - nfield, len(terms_of(h))))
    _, grad = prob.gradient(A)
    dedh = sum(grad[t] for t in field_idx).real
    delta = 1e-5
    fd = (_ed(types, terms_of(h + delta))[0] - _ed(types, terms_of(h - delta))[0]) / (2 * delta)
    assert abs(dedh - fd) < 1e-6 * max(1.0, abs(fd)), (dedh, fd)
    # autograd: E(c(h)) with c linear in h
    c0 = torch.tensor([c.real for c, _ in terms_of(h)], dtype=torch.float64)
    hh = torch.tensor(h, dtype=torch.float64, requires_grad=True)
    mask = torch.zeros_like(c0)
    mask[field_idx] = 1.0
    c = c0 * (1 - mask) + hh * mask
    E = CouplingEnergy.apply(c, prob, A)
    E.backward()
    assert abs(E.item() - _ed(types, terms_of(h))[0]) / n < 1e-10
    assert abs(hh.grad.item() - dedh) < 1e-12 * max(1.0, abs(dedh))


def test_chain_session_gradient():
    from dmrgpy_gb300.chain import Chain
    n = 8
    terms = terms_tfim(n, 1.0, 1.1)
    ch = Chain([2] * n)
    ch.set_sweep_params(16, 8, 1e-14, 0.0)
    ch.set_hamiltonian(terms)
    np.random.seed(4)
    g = ch.gs_energy_gradient()
    e0, v0 = _ed([2] * n, terms)
    assert abs(ch.gs_energy(skip_dmrg=True) - e0) / n < 1e-10
    for t, (c, f) in enumerate(terms):
        ht = O.dense_hamiltonian([2] * n, [(1.0 + 0j, f)])
        assert abs(g[t] - np.vdot(v0, ht @ v0)) < 1e-6
