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

    def __init__(self, types, terms, precision="fp64", device="cuda:0"):
        self.types = [int(t) for t in types]
        self.structure = [list(f) for _, f in terms]
        self.coefs = np.array([complex(c) for c, _ in terms])
        W, real, cmap = _mpo.build_mpo(self.types, self.terms(self.coefs), coupling_map=True)
        self.real = real
        self.cmap = cmap
        self.engine = Engine(W, real=real, precision=precision, device=device)

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

    def gradient(self, A):
        """(E, dE/dc_t for every term) at the state A (device tensors)."""
        e, G = self.engine.mpo_gradients(A)
        Gh = [g.detach().cpu().numpy() for g in G]
        out = np.zeros(len(self.cmap), dtype=complex)
        for t, entry in enumerate(self.cmap):
            if entry is None:
                continue
            site, ls, rs, M, factor = entry
            out[t] = factor * np.sum(Gh[site][ls, :, :, rs] * M)
        return e, out

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
