"""Chain: the session object of the GB300 backend.

Mirrors the method surface and semantics of dmrgpy's python-backend session
(``pyitensor/chain.py:142-1448``, itself a transcription of
``mpscpp3/bindings.cc``) for the sweep path: dmrgpy's glue code calls these
methods with the same arguments (``groundstate.py:21-85``,
``timedependent.py:52-248``, ``vev.py:23-36``, ``entropy.py:29-35``).  The
sweep itself runs on the GPU (:mod:`dmrgpy_gb300.engine`); errors follow the
reference (``RuntimeError`` for misuse, ``ValueError`` for unknown operator
names).

Differences, all numerical-path only: the MPO is compiled by the automaton
builder of :mod:`dmrgpy_gb300.mpo` (real arithmetic whenever the Hamiltonian
allows); the right environments of a sweep are reused from the previous
right-to-left pass instead of being rebuilt; truncations take the
reference's Gram-matrix route on the GPU (blocked-Jacobi eigensolver) or,
on large bonds where maxdim binds, a subspace + Rayleigh-Ritz form of it.
"""
import numpy as np

from . import mpo as _mpo
from . import mps as _mps
from . import sites as _sites
from .engine import Engine


class Operator:
    """Compiled MPO handle (what build_operator returns)."""

    def __init__(self, W, real):
        self.W = W
        self.real = real

    def copy(self):
        return Operator([w.copy() for w in self.W], self.real)


class Chain:
    def __init__(self, site_types, precision="fp64"):
        self.site_types = [int(t) for t in site_types]
        self.dims = [_sites.dim(t) for t in self.site_types]
        self.H = None
        self.have_H = False
        self.wf0 = None
        self._wf0_energy = None
        self.maxm = 30
        self.nsweeps = 15
        self.cutoff = 1e-12
        self.noise = 1e-1
        self.mpomaxm = 5000
        self.verbose = False
        self.precision = precision
        self.last_stats = None

    # ---------------------------------------------------------------- setup
    def num_sites(self):
        return len(self.site_types)

    def site_dim(self, site):
        return self.dims[site - 1]

    def set_sweep_params(self, maxm, nsweeps, cutoff, noise):
        self.maxm = maxm
        self.nsweeps = nsweeps
        self.cutoff = cutoff
        self.noise = noise

    def set_mpomaxm(self, mpomaxm):
        self.mpomaxm = mpomaxm

    def set_verbose(self, verbose):
        self.verbose = verbose

    def set_precision(self, precision):
        self.precision = precision

    def build_operator(self, terms):
        W, real = _mpo.build_mpo(self.site_types, terms)
        return Operator(W, real)

    def set_hamiltonian(self, terms):
        self.H = self.build_operator(terms)
        self.H_terms = list(terms)
        self.have_H = True
        self._wf0_energy = None

    # ---------------------------------------------------------------- states
    def _engine(self, op, complex_=False):
        real = op.real and not complex_
        prec = self.precision if real else "fp64"
        return Engine(op.W, real=real, precision=prec)

    def _default_mps(self, eng=None):
        """pyitensor/chain.py:1175 -> randomMPS(sites, maxm)."""
        arrays = _mps.random_arrays(self.dims, self.maxm)
        if eng is None:
            eng = self._engine(self.H if self.H is not None else Operator(
                [np.zeros((1, d, d, 1)) for d in self.dims], True))
        A = eng.to_device(arrays)
        eng.canonicalize_right_to_left_of(A)
        return _mps.MPS(eng.to_host(A), center=len(A))

    def random_mps(self):
        return self._default_mps()

    def _make_sweeps(self):
        """pyitensor/chain.py:1188-1199: constant maxdim, niter 2 (the
        Lanczos floor of 200 applies inside the solver)."""
        return [self.maxm] * self.nsweeps, [self.cutoff] * self.nsweeps, [2] * self.nsweeps

    def gs_energy(self, skip_dmrg=False):
        if not self.have_H:
            raise RuntimeError("Chain.gs_energy called before set_hamiltonian")
        if skip_dmrg and self.wf0 is not None and self._wf0_energy is not None:
            return self._wf0_energy
        eng = self._engine(self.H)
        if self.wf0 is None:
            self.wf0 = self._default_mps(eng)
        A = eng.to_device(self.wf0.tensors)
        maxdims, cutoffs, niters = self._make_sweeps()
        energy = eng.dmrg(A, maxdims, cutoffs, niters)
        self.wf0 = _mps.MPS(eng.to_host(A), center=1)
        self._wf0_energy = energy
        self.last_stats = eng.stats
        return energy

    def gs_energy_gradient(self):
        """dE/dc_t for every term t of the Hamiltonian (as given to
        set_hamiltonian) at the current ground state, from one adjoint pass
        over the environments (:mod:`dmrgpy_gb300.gradients`).  Runs
        gs_energy first if needed.  Returns a complex NumPy array; for a
        Hermitian pair of terms with a real coupling the sum is real."""
        from .gradients import CouplingProblem
        if not self.have_H:
            raise RuntimeError("Chain.gs_energy_gradient called before set_hamiltonian")
        if self.wf0 is None or self._wf0_energy is None:
            self.gs_energy()
        prob = CouplingProblem(self.site_types, self.H_terms)
        A = prob.engine.to_device(self.wf0.tensors)
        _, grad = prob.gradient(A)
        return grad

    def gs_wavefunction(self):
        if self.wf0 is None:
            raise RuntimeError("Chain.gs_wavefunction called before gs_energy")
        return self.wf0

    def set_wavefunction(self, wf):
        self.wf0 = wf
        self._wf0_energy = None

    # ---------------------------------------------------------------- measurements
    # Contracted on the device in FP64 (Engine.transition / bond_spectrum);
    # the state crosses to the device once per call.
    def _measure_engine(self, W, real, wfs):
        real = real and not any(np.iscomplexobj(t) for wf in wfs for t in wf.tensors)
        return Engine(W, real=real, precision="fp64")

    def vev(self, terms, wf, npow=1):
        """pyitensor/chain.py:277-287: <psi|A^npow|psi>/<psi|psi>; A^npow is
        formed exactly as an MPO power (bond dimension w^npow) rather than
        by npow-1 truncated applications."""
        op = self.build_operator(terms)
        W = _mpo_power(op.W, int(npow))
        eng = self._measure_engine(W, op.real, [wf])
        A = eng.to_device(wf.tensors)
        num = eng.transition(eng.W, A, A)
        den = eng.transition(eng.identity_mpo(self.dims), A, A)
        return num / den.real

    def overlap(self, wf1, wf2):
        eng = self._measure_engine([np.eye(d).reshape(1, d, d, 1) for d in self.dims], True, [wf1, wf2])
        return eng.transition(eng.W, eng.to_device(wf1.tensors), eng.to_device(wf2.tensors))

    def overlap_aMb(self, wf1, terms, wf2):
        op = self.build_operator(terms)
        return self.overlap_aMb_operator(wf1, op, wf2)

    def overlap_aMb_operator(self, wf1, A, wf2):
        eng = self._measure_engine(A.W, A.real, [wf1, wf2])
        return eng.transition(eng.W, eng.to_device(wf1.tensors), eng.to_device(wf2.tensors))

    def bond_entropy(self, wf, b):
        """pyitensor/chain.py:468-480: -sum p log p over the Schmidt weights
        p > 1e-12 across bond (b, b+1)."""
        eng = self._measure_engine([np.eye(d).reshape(1, d, d, 1) for d in self.dims], True, [wf])
        s = eng.bond_spectrum(eng.to_device(wf.tensors), int(b))
        p = s ** 2
        p = p / p.sum()
        p = p[p > 1e-12]
        return float(-np.sum(p * np.log(p)))

    # ---------------------------------------------------------------- time evolution
    def tdvp_step(self, H, wf, dt, num_center=2):
        """pyitensor/chain.py:397-420 (note the (H, wf, dt) order); wf is
        copied, the evolved state returned."""
        eng = self._engine(H, complex_=True)
        A = eng.to_device([t.astype(complex) for t in wf.tensors])
        eng.tdvp_step(A, dt, self.cutoff, self.maxm, niter=50, num_center=num_center)
        return _mps.MPS(eng.to_host(A), center=1)

    def evolve_and_measure_tdvp(self, terms_h, terms_op, wf, nt, dt):
        """pyitensor/chain.py:544-564: measure <A> then step, nt times."""
        H = self.build_operator(terms_h)
        Aop = self.build_operator(terms_op)
        eng = self._engine(H, complex_=True)
        A = eng.to_device([t.astype(complex) for t in wf.tensors])
        out = []
        for _ in range(nt):
            host = eng.to_host(A)
            out.append(_mps.expect(host, Aop.W, host))
            eng.tdvp_step(A, dt, self.cutoff, self.maxm, niter=50)
        return out, _mps.MPS(eng.to_host(A), center=1)

    def quench_tdvp(self, terms_h, terms_i, terms_j, nt, dt):
        """pyitensor/chain.py:520-542."""
        if self.wf0 is None:
            self.gs_energy()
        H = self.build_operator(terms_h)
        egs = (_mps.expect(self.wf0.tensors, H.W, self.wf0.tensors)
               / _mps.inner(self.wf0.tensors, self.wf0.tensors)).real
        Hshift = self.build_operator(list(terms_h) + [(-egs + 0j, [("Id", 1)])])
        A1 = self.build_operator(terms_i)
        A2 = self.build_operator(terms_j)
        psi1 = _apply_mpo_exact(A1.W, self.wf0.tensors)
        psi2 = _apply_mpo_exact(A2.W, self.wf0.tensors)
        norm0 = np.sqrt(_mps.inner(psi1, psi1).real)
        eng = self._engine(Hshift, complex_=True)
        A = eng.to_device([t.astype(complex) for t in psi1])
        out = []
        for _ in range(nt):
            host = eng.to_host(A)
            out.append(_mps.inner(psi2, host))
            eng.tdvp_step(A, dt, self.cutoff, self.maxm, niter=50)
            nrm = _torch_norm(A)
            A[0] = A[0] * (norm0 / nrm)
        return out, _mps.MPS(eng.to_host(A), center=1)


def _mpo_power(W, k):
    """The MPO of A^k (k >= 1) for A given as (w_l, d_in, d_out, w_r) site
    tensors, without truncation: per site the product of k copies, bond
    dimension w^k."""
    if k < 1:
        raise ValueError("npow must be >= 1")
    out = [np.asarray(w) for w in W]
    for _ in range(k - 1):
        nxt = []
        for p, w in zip(out, W):
            # apply w after p: (pl, wl, din, dout, pr, wr)
            x = np.einsum("aimb,cmoe->acio be".replace(" ", ""), p, np.asarray(w))
            pl, wl, d, _, pr, wr = x.shape
            nxt.append(x.reshape(pl * wl, d, d, pr * wr))
        out = nxt
    return out


def _torch_norm(A):
    """Norm of an MPS whose sites 2..N are right-orthonormal (the state after
    a TDVP step): the norm of the first tensor."""
    import torch
    return float(torch.linalg.vector_norm(A[0]).item())


def _apply_mpo_exact(W, A):
    """W|A> without truncation (bond dims multiply); host-side helper for
    the quench set-up."""
    out = []
    for w, a in zip(W, A):
        x = np.tensordot(a, w, axes=([1], [1]))          # (al, ar, wl, dout, wr)
        x = x.transpose(2, 0, 3, 4, 1)                   # (wl, al, dout, wr, ar)
        wl, al, d, wr, ar = x.shape
        out.append(x.reshape(wl * al, d, wr * ar))
    return out
