"""The GB300 backend as a session of dmrgpy's own type.

dmrgpy's glue drives a session object through some 54 methods
(``pyitensor/chain.py:142-1448``) and hands back opaque wavefunction and
operator handles, which for the python backend are pyitensor ``MPS`` /
``MPO`` objects that other session methods then do algebra on
(``mpsalgebra.py:125-131``, ``manybodychain.py:289``).  The session class
here therefore *is* a python-backend session: a subclass of
``dmrgpy.pyitensor.chain.Chain`` whose handles stay pyitensor objects, so
every method keeps the reference's behaviour, and whose sweep methods run on
the GPU:

  gs_energy                the two-site DMRG sweeps (:mod:`.engine`), from
                           the reference's own random initial state
                           (``_default_mps``: the same ``np.random`` draws);
  tdvp_step, quench_tdvp,  the two-/one-site TDVP steps on the device,
  evolve_and_measure_tdvp  measured with the reference's ``inner`` between
                           steps like ``pyitensor/chain.py:520-564``.

At the boundary a pyitensor MPS becomes (chi_l, d, chi_r) arrays with
``_mps_arrays_lpr`` (``pyitensor/chain.py:41-60``) and comes back with fresh
``Link`` indices on the session's own site indices; an MPO becomes
(w_l, d_in, d_out, w_r) arrays ordered against its site index and its
primed copy.  The ground-state sweep uses the real MPO compiled from the
same terms by :mod:`.mpo`.

Requires dmrgpy to be importable; ``precision`` "fp64" or "tf32x3" selects
the contraction precision of the ground-state sweeps.
"""
import numpy as np

from . import mpo as _mpo
from .engine import Engine

_CLASSES = {}


def _py():
    from dmrgpy.pyitensor import chain as pychain
    from dmrgpy.pyitensor.index import Index
    from dmrgpy.pyitensor.mpscontainer import MPS, _link_at
    from dmrgpy.pyitensor.mpsalgebra import inner
    from dmrgpy.pyitensor.tensor import ITensor
    return pychain, Index, MPS, _link_at, inner, ITensor


def mps_to_arrays(psi):
    """(chi_l, d, chi_r) arrays of a pyitensor MPS (length-1 edge links)."""
    pychain = _py()[0]
    return pychain._mps_arrays_lpr(psi)


def arrays_to_mps(arrays, sites, center=1):
    """A pyitensor MPS on the session's site indices from (chi_l, d, chi_r)
    arrays, with freshly minted Link indices."""
    _, Index, MPS, _, _, ITensor = _py()
    n = len(arrays)
    links = [Index(int(arrays[k].shape[2]), tags="Link,l={}".format(k + 1)) for k in range(n - 1)]
    tensors = []
    for i, a in enumerate(arrays):
        a = np.asarray(a)
        inds = ([links[i - 1]] if i > 0 else []) + [sites.si(i + 1)] + ([links[i]] if i < n - 1 else [])
        shape = tuple(ind.dim for ind in inds)
        tensors.append(ITensor(tuple(inds), np.ascontiguousarray(a.reshape(shape), dtype=complex)))
    psi = MPS(tensors)
    psi.center = center
    return psi


def mpo_to_arrays(H):
    """(w_l, d_in, d_out, w_r) arrays of a pyitensor MPO, d_in being the
    unprimed site index (the one a ket's site index contracts with)."""
    _, _, _, _link_at, _, _ = _py()
    n = H.length()
    out = []
    for i in range(1, n + 1):
        T = H.A(i)
        s = next(ind for ind in T.inds if ind.hastags("Site") and ind.plev == 0)
        sp = s.prime(1)
        left = _link_at(H, i, i - 1)
        right = _link_at(H, i, i + 1)
        order = [x for x in (left, s, sp, right) if x is not None]
        a = T.transpose_to(order)
        out.append(np.ascontiguousarray(a.reshape(left.dim if left else 1, s.dim, s.dim,
                                                  right.dim if right else 1)))
    return out


def session_class(precision="fp64"):
    """The session class for one contraction precision (cached)."""
    if precision not in ("fp64", "tf32x3"):
        raise ValueError("precision must be 'fp64' or 'tf32x3'")
    if precision in _CLASSES:
        return _CLASSES[precision]
    pychain, _, _, _, inner, _ = _py()

    class GB300Session(pychain.Chain):
        """dmrgpy python-backend session whose sweeps run on the GB300."""
        contraction_precision = precision

        def __init__(self, site_types):
            super().__init__(site_types)
            self._site_types = [int(t) for t in site_types]
            self._gb_H = None
            self.last_stats = None

        def set_hamiltonian(self, terms):
            super().set_hamiltonian(terms)
            self._gb_H = _mpo.build_mpo(self._site_types, terms)

        def gs_energy(self, skip_dmrg=False):
            """pyitensor/chain.py:209-219 with the sweeps on the device."""
            if not self.have_H:
                raise RuntimeError("Chain.gs_energy called before set_hamiltonian")
            if skip_dmrg and self.wf0 is not None and self._wf0_energy is not None:
                return self._wf0_energy
            if self.wf0 is None:
                self.wf0 = self._default_mps()
            W, real = self._gb_H
            eng = Engine(W, real=real, precision=self.contraction_precision if real else "fp64")
            A = eng.to_device(mps_to_arrays(self.wf0))
            n = int(self.nsweeps)
            energy = eng.dmrg(A, [self.maxm] * n, [self.cutoff] * n, [2] * n)
            self.wf0 = arrays_to_mps(eng.to_host(A), self.sites, center=1)
            self._wf0_energy = energy
            self.last_stats = eng.stats
            return energy

        def _device_tdvp(self, H):
            return Engine(mpo_to_arrays(H), real=False, precision="fp64")

        def tdvp_step(self, H, wf, dt, num_center=2):
            """pyitensor/chain.py:397-420 (the (H, wf, dt) order): wf is left
            untouched, the evolved state returned."""
            eng = self._device_tdvp(H)
            A = eng.to_device(mps_to_arrays(wf))
            eng.tdvp_step(A, dt, self.cutoff, self.maxm, niter=50, num_center=num_center)
            return arrays_to_mps(eng.to_host(A), self.sites, center=1)

        def quench_tdvp(self, terms_h, terms_i, terms_j, nt, dt):
            """pyitensor/chain.py:520-542: the correlator <psi2|psi1(t)> of
            psi1 = A_i|gs>, psi2 = A_j|gs> under H - E_gs, measured before
            each step, psi1 renormalised to its initial norm after it."""
            if self.wf0 is None:
                self.gs_energy()
            H = self.build_operator(terms_h)
            egs = inner(self.wf0, H, self.wf0).real / inner(self.wf0, self.wf0).real
            Hshift = self.build_operator(list(terms_h) + [(-egs + 0j, [("Id", 1)])])
            A1 = self.build_operator(terms_i)
            A2 = self.build_operator(terms_j)
            psi1 = self._apply_mpo(A1, self.wf0)
            psi2 = self._apply_mpo(A2, self.wf0)
            norm0 = complex(np.sqrt(inner(psi1, psi1)))
            eng = self._device_tdvp(Hshift)
            A = eng.to_device(mps_to_arrays(psi1))
            correlator = []
            for _ in range(int(nt)):
                cur = arrays_to_mps(eng.to_host(A), self.sites, center=1)
                correlator.append(inner(psi2, cur))
                eng.tdvp_step(A, dt, self.cutoff, self.maxm, niter=50)
                # after a step the orthogonality centre is the first site
                nrm = float(np.linalg.norm(A[0].cpu().numpy()))
                A[0] = A[0] * (norm0 / nrm)
            return correlator, arrays_to_mps(eng.to_host(A), self.sites, center=1)

        def evolve_and_measure_tdvp(self, terms_h, terms_op, wf, nt, dt):
            """pyitensor/chain.py:544-564: <psi(t)|A|psi(t)> measured before
            each step; wf itself is left untouched."""
            H = self.build_operator(terms_h)
            Aop = self.build_operator(terms_op)
            eng = self._device_tdvp(H)
            A = eng.to_device(mps_to_arrays(wf))
            correlator = []
            for _ in range(int(nt)):
                cur = arrays_to_mps(eng.to_host(A), self.sites, center=1)
                correlator.append(inner(cur, Aop, cur))
                eng.tdvp_step(A, dt, self.cutoff, self.maxm, niter=50)
            return correlator, arrays_to_mps(eng.to_host(A), self.sites, center=1)

    GB300Session.__name__ = "GB300Session_" + precision
    _CLASSES[precision] = GB300Session
    return GB300Session
