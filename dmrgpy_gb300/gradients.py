"""Derivatives of energies with respect to Hamiltonian couplings.

dmrgpy has no derivative features; this module adds them on top of the same
term lists.  A Hamiltonian H = sum_t c_t h_t is compiled with
``mpo.build_mpo(..., coupling_map=True)``, which keeps the automaton affine
in the coefficients: term t adds ``factor_t * c_t * M_t`` to one block
W[site_t][ls_t, :, :, rs_t].  The reverse pass over the environment chain
(``Engine.mpo_gradients``, kernel ``dmrg_env_gradient``) gives
G_i = dE/dW_i for every site at once, and

    dE/dc_t = factor_t * sum_{s,s'} G_{site_t}[ls_t, s, s', rs_t] M_t[s, s'].

At a converged ground state the state is stationary, so these are the
derivatives of the ground-state energy (Hellmann-Feynman); the checks are
central finite differences of ground-state energies and <h_t> measured on
the state (the reference's ``vev``, ``pyitensor/chain.py:277-287``).

``CouplingEnergy`` wraps the pass as a ``torch.autograd.Function`` so a
coupling vector (or anything differentiable that produces it) can be
back-propagated through.
"""
import numpy as np

from . import mpo as _mpo
from .engine import Engine


def _torch():
    import torch
    return torch


class CouplingProblem:
    """A term structure whose coefficients are the differentiable inputs.

    types: site type codes; terms: dmrgpy term list [(coef, [(op, site), ...])]
    (the coefficients give the initial coupling vector).
    """

    def __init__(self, types, terms, precision="fp64", device="cuda:0", complex_=False):
        self.types = [int(t) for t in types]
        self.structure = [list(f) for _, f in terms]
        self.coefs = np.array([complex(c) for c, _ in terms])
        W, real, cmap = _mpo.build_mpo(self.types, self.terms(self.coefs), coupling_map=True)
        self.real = real
        self.cmap = cmap
        self.engine = Engine(W, real=real and not complex_, precision=precision, device=device)

    def terms(self, coefs):
        return [(complex(c), f) for c, f in zip(coefs, self.structure)]

    def set_coefs(self, coefs):
        coefs = np.asarray(coefs, dtype=complex)
        W, real, cmap = _mpo.build_mpo(self.types, self.terms(coefs), coupling_map=True)
        if real != self.real:
            raise ValueError("the new couplings change the MPO's element type")
        self.engine.set_mpo(W)
        self.coefs = coefs
        self.cmap = cmap

    def term_values(self, G):
        """Per-term contractions factor_t <G_site, M_t> of a list of
        MPO-tensor gradients G_i (= <bra|h_t|ket> for transition gradients)."""
        Gh = [g.detach().cpu().numpy() for g in G]
        out = np.zeros(len(self.cmap), dtype=complex)
        for t, entry in enumerate(self.cmap):
            if entry is None:
                continue
            site, ls, rs, M, factor = entry
            out[t] = factor * np.sum(Gh[site][ls, :, :, rs] * M)
        return out

    def gradient(self, A):
        """(E, dE/dc_t for every term) at the state A (device tensors)."""
        e, G = self.engine.mpo_gradients(A)
        return e, self.term_values(G)

    def ground_state(self, A, maxdims, cutoffs, niters=2):
        """DMRG on the current couplings, in place on A; returns the energy."""
        return self.engine.dmrg(A, maxdims, cutoffs, niters)


class CouplingEnergy:
    """torch.autograd.Function: E(c) at a fixed state, backward = adjoint pass.

    ``CouplingEnergy.apply(c, problem, A)`` with c a real float64 tensor of
    the couplings returns the energy as a 0-d tensor; its gradient with
    respect to c is Re(dE/dc_t) from ``CouplingProblem.gradient``.
    """

    _fn = None

    @classmethod
    def apply(cls, c, problem, A):
        if cls._fn is None:
            torch = _torch()

            class _F(torch.autograd.Function):
                @staticmethod
                def forward(ctx, coefs, prob, state):
                    prob.set_coefs(coefs.detach().cpu().numpy().astype(complex))
                    e, g = prob.gradient(state)
                    ctx.save_for_backward(torch.as_tensor(g.real, dtype=coefs.dtype, device=coefs.device))
                    return torch.tensor(e, dtype=coefs.dtype, device=coefs.device)

                @staticmethod
                def backward(ctx, gout):
                    (g,) = ctx.saved_tensors
                    return gout * g, None, None

            cls._fn = _F
        return cls._fn.apply(c, problem, A)


def _overlap(eng, Bra, Ket):
    """<bra|ket> by transition environments with the identity MPO."""
    torch = _torch()
    L = eng.edge
    for b, a in zip(Bra, Ket):
        d = a.shape[1]
        ident = torch.eye(d, dtype=eng.tdtype, device=eng.device).reshape(1, d, d, 1).contiguous()
        L = eng.env_mixed(0, L, ident, b, a)
    return complex(L.reshape(-1)[0].item())


def tdvp_observable_gradient(types, terms, psi0, site, opname, dt, nsteps, maxdim, cutoff=1e-12, niter=50,
                             num_center=2, device="cuda:0"):
    """<O(t)> after nsteps TDVP steps of dt from psi0, and d<O(t)>/dc_t for
    every term of H = sum_t c_t h_t, by the continuous-time adjoint:

        d<O(t)>/dc_t = 2 Re[-i int_0^t <chi(s)| h_t |psi(s)> ds],
        |psi(s)> = exp(-iHs) |psi0>,   |chi(s)> = exp(+iH(t-s)) O |psi(t)>.

    The forward pass keeps the state after every step (the checkpoints); the
    backward pass applies O to the final state, evolves that costate back in
    time with the same TDVP integrator (dt -> -dt) and, at every checkpoint,
    evaluates <chi|h_t|psi> for all terms at once by one transition adjoint
    pass (dmrg_env_gradient_mixed), recomputing the environments from the
    checkpoint; the time integral is the trapezoid rule on the step grid.
    The error is that of the TDVP integrator (O(dt^2) over a fixed time) and
    of the truncation; the reference has no derivative features, so the
    checks are finite differences of exactly evolved observables.

    psi0: host site tensors (chi_l, d, chi_r); site: 1-based; opname: a site
    operator name of the site type (e.g. "Sz").  Returns (<O(t)>, grad).
    """
    from . import sites as _sites
    torch = _torch()
    prob = CouplingProblem(types, terms, device=device, complex_=True)
    eng = prob.engine
    A = eng.to_device(psi0)
    eng.right_canonicalize(A)
    A[0] = (A[0] / torch.linalg.vector_norm(A[0])).contiguous()
    states = [[a.clone() for a in A]]
    for _ in range(nsteps):
        eng.tdvp_step(A, dt, cutoff, maxdim, niter, num_center)
        states.append([a.clone() for a in A])
    j = int(site) - 1
    op = torch.as_tensor(np.asarray(_sites.op(prob.types[j], opname), dtype=np.complex128), device=eng.device)
    chi = [a.clone() for a in A]
    chi[j] = torch.einsum("st,atb->asb", op, chi[j]).contiguous()
    value = _overlap(eng, A, chi)
    eng.right_canonicalize(chi)
    acc = np.zeros(len(prob.cmap), dtype=complex)
    for k in range(nsteps, -1, -1):
        _, G = eng.transition_gradients(chi, states[k])
        w = 0.5 if k in (0, nsteps) else 1.0
        acc += w * prob.term_values(G)
        if k > 0:
            eng.tdvp_step(chi, -dt, cutoff, maxdim, niter, num_center)
    grad = 2.0 * np.real(-1j * dt * acc)
    return value.real, grad
