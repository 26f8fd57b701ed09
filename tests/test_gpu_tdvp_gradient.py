"""Gradients of a time-evolved observable through TDVP (the continuous
adjoint in gradients.tdvp_observable_gradient) and the transition
environments behind it.  The reference has no derivative features; the
oracle is exact time evolution of the dense Hamiltonian (oracle
dense_hamiltonian) with central finite differences in the couplings.  The
adjoint differentiates the exact dynamics, TDVP integrates it with an
O(dt^2) error at fixed time, so gradients are compared at the integrator's
accuracy (stated below), the transition contractions exactly."""
import numpy as np
import pytest
from scipy.linalg import expm

from golden_data import terms_xxz
from oracle import dmrg_oracle as O

pytestmark = pytest.mark.gpu

N = 6
T_FINAL = 0.2
# The adjoint differentiates the exact dynamics; TDVP integrates it with an
# O(dt^2) error at fixed time (measured: 2.6e-6, 6.4e-7, 1.6e-7 for dt =
# 0.04, 0.02, 0.01 over all term gradients of this chain).
GRAD_TOL = 5e-6                # absolute, at dt = 0.02
VALUE_TOL = 1e-6


def _neel(n):
    out = []
    for i in range(n):
        a = np.zeros((1, 2, 1), dtype=complex)
        a[0, i % 2, 0] = 1.0
        out.append(a)
    return out


def _exact(terms, psi0, site, t):
    H = O.dense_hamiltonian([2] * N, terms)
    v = expm(-1j * t * H) @ psi0
    Sz = O.dense_hamiltonian([2] * N, [(1.0 + 0j, [("Sz", site)])])
    return float(np.vdot(v, Sz @ v).real)


def test_transition_gradients_match_dense_contractions():
    import torch
    from dmrgpy_gb300 import mps as MP
    from dmrgpy_gb300.gradients import CouplingProblem
    rng = np.random.default_rng(3)
    terms = terms_xxz(N, 0.5, fields=list(rng.uniform(-0.1, 0.1, N)))
    prob = CouplingProblem([2] * N, terms, complex_=True)
    eng = prob.engine
    np.random.seed(5)
    bra = MP.random_arrays([2] * N, 3)
    np.random.seed(6)
    ket = MP.random_arrays([2] * N, 4)
    Bd, Kd = eng.to_device(bra), eng.to_device(ket)
    val, G = eng.transition_gradients(Bd, Kd)
    vb, vk = O.mps_to_dense(bra), O.mps_to_dense(ket)
    H = O.dense_hamiltonian([2] * N, terms)
    want = np.vdot(vb, H @ vk)
    assert abs(val - want) < 1e-12 * max(1.0, abs(want))
    for g, w in zip(G, eng.W):
        assert abs(complex(torch.sum(g * w).item()) - want) < 1e-12 * max(1.0, abs(want))
    per_term = prob.term_values(G)
    for t, (c, f) in enumerate(terms):
        ht = O.dense_hamiltonian([2] * N, [(1.0 + 0j, f)])
        assert abs(per_term[t] - np.vdot(vb, ht @ vk)) < 1e-12 * max(1.0, abs(want))


def _gradient_errors(dt):
    from dmrgpy_gb300.gradients import tdvp_observable_gradient
    rng = np.random.default_rng(9)
    delta, fields = 0.5, list(rng.uniform(-0.1, 0.1, N))
    site = 3
    terms = terms_xxz(N, delta, fields=fields)
    psi0 = _neel(N)
    nsteps = int(round(T_FINAL / dt))
    val, grad = tdvp_observable_gradient([2] * N, terms, psi0, site, "Sz", dt, nsteps, maxdim=8)
    v0 = O.mps_to_dense(psi0)
    value_err = abs(val - _exact(terms, v0, site, T_FINAL))
    # d/dDelta: every Sz Sz coupling; d/dh_i: the field terms
    zz = [k for k, (c, f) in enumerate(terms) if len(f) == 2 and f[0][0] == "Sz"]
    field = list(range(len(terms) - N, len(terms)))
    eps = 1e-5

    def shifted(idx, sgn):
        out = list(terms)
        for k in idx:
            c, f = out[k]
            out[k] = (c + sgn, f)
        return out

    def fd(idx):
        return (_exact(shifted(idx, eps), v0, site, T_FINAL) - _exact(shifted(idx, -eps), v0, site, T_FINAL)) / (2 * eps)
    errs = [abs(sum(grad[k] for k in zz) - fd(zz))]
    errs += [abs(grad[k] - fd([k])) for k in field]
    return value_err, max(errs)


def test_tdvp_observable_gradient_matches_exact_finite_differences():
    v2, e2 = _gradient_errors(0.02)
    v4, e4 = _gradient_errors(0.04)
    assert v2 < VALUE_TOL
    assert e2 < GRAD_TOL, e2
    # second-order convergence to the exact derivative
    assert e2 < 0.4 * e4, (e2, e4)
