"""Many independent chains swept together on one GPU.

Every chain has its own MPO, state and bond-dimension cap, but all chains have
the same length and are swept in lock step: at each bond, the two-site
merges, the Lanczos ground states, the truncated SVDs and the environment
extensions of all chains are single grouped launches (``dmrg_batch_*`` in
``include/dmrg_gb300.h``), whatever their bond dimensions.  The Lanczos
blocks are replayed from captured CUDA graphs.  The per-chain algorithm is
the single-chain sweep of :class:`dmrgpy_gb300.engine.Engine` (the reference
sweep ``pyitensor/dmrg.py:355-398``) in FP64.
"""
import ctypes

import numpy as np

from . import _lib
from . import mps as _mps
from .engine import LANCZOS_TOL, Workspace


def _torch():
    import torch
    return torch


def _arr(ctype, values):
    return (ctype * len(values))(*values)


def _ptrs(tensors):
    return (ctypes.c_void_p * len(tensors))(*[t.data_ptr() for t in tensors])


def partition_chains(costs, nparts):
    """Assigns independent chains to nparts ranks (GPUs) so that their summed
    costs balance, e.g. chi^3 d^2 w per chain for the matvec-dominated
    sweep: longest first, each chain to the rank with the least cost so far
    (ties to the lower rank).  Deterministic, so every rank computes the same
    assignment without communication; the ranks then sweep their shares with
    no collective.  Returns one ascending list of chain indices per rank."""
    if nparts < 1:
        raise ValueError("nparts must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i))
    load = [0.0] * nparts
    parts = [[] for _ in range(nparts)]
    for i in order:
        r = min(range(nparts), key=lambda j: (load[j], j))
        parts[r].append(i)
        load[r] += float(costs[i])
    return [sorted(p) for p in parts]


class BatchEngine:
    """Lock-step sweeps of len(Ws) chains.

    Ws: one MPO (list of (wl, d, d, wr) arrays) per chain, all of the same
    length; real: element type of every MPO.  niter_cap bounds the Krylov
    dimension per bond (the batch keeps all bases resident).
    """

    def __init__(self, Ws, real=True, device="cuda:0", niter_cap=48, use_graphs=True):
        torch = _torch()
        if not torch.cuda.is_available():
            raise RuntimeError("dmrgpy_gb300 needs a CUDA device (GB300); no CPU fallback exists")
        self.lib = _lib.load()
        self.device = torch.device(device)
        self.real = bool(real)
        self.tdtype = torch.float64 if self.real else torch.complex128
        self.cdtype = _lib.REAL64 if self.real else _lib.COMPLEX128
        npdt = np.float64 if self.real else np.complex128
        self.nchains = len(Ws)
        self.n = len(Ws[0])
        if any(len(W) != self.n for W in Ws):
            raise ValueError("all chains of a batch must have the same number of sites")
        self.W = [[torch.as_tensor(np.ascontiguousarray(w, dtype=npdt), device=self.device) for w in W] for W in Ws]
        self.ws = Workspace(self.device)
        self.edge = torch.ones((1, 1, 1), dtype=self.tdtype, device=self.device)
        self.niter_cap = int(niter_cap)
        self.use_graphs = bool(use_graphs)
        self.lanczos_iters = []

    @property
    def stream(self):
        return ctypes.c_void_p(_torch().cuda.current_stream(self.device).cuda_stream)

    # ------------------------------------------------------------ batched primitives
    def merge(self, As, Bs):
        torch = _torch()
        m = [a.shape[0] * a.shape[1] for a in As]
        k = [a.shape[2] for a in As]
        nn = [b.shape[1] * b.shape[2] for b in Bs]
        out = [torch.empty((a.shape[0], a.shape[1], b.shape[1], b.shape[2]), dtype=self.tdtype, device=self.device)
               for a, b in zip(As, Bs)]
        c = self.nchains
        need = self.lib.dmrg_batch_gemm_workspace_bytes(c)
        ptr, size = self.ws.get(need)
        _lib.check("dmrg_batch_gemm", self.lib.dmrg_batch_gemm(
            self.cdtype, c, _arr(ctypes.c_int, m), _arr(ctypes.c_int, k), _arr(ctypes.c_int, nn), _ptrs(As),
            _ptrs(Bs), _ptrs(out), ptr, size, self.stream))
        return out

    def _env(self, side, Es, Ws, As):
        torch = _torch()
        cl = [a.shape[0] for a in As]
        d = [a.shape[1] for a in As]
        cr = [a.shape[2] for a in As]
        wl = [w.shape[0] for w in Ws]
        wr = [w.shape[3] for w in Ws]
        if side == 0:
            out = [torch.empty((a.shape[2], w.shape[3], a.shape[2]), dtype=self.tdtype, device=self.device)
                   for a, w in zip(As, Ws)]
        else:
            out = [torch.empty((a.shape[0], w.shape[0], a.shape[0]), dtype=self.tdtype, device=self.device)
                   for a, w in zip(As, Ws)]
        args = [_arr(ctypes.c_int, v) for v in (cl, d, cr, wl, wr)]
        c = self.nchains
        need = self.lib.dmrg_batch_env_workspace_bytes(side, self.cdtype, c, *args)
        ptr, size = self.ws.get(need)
        _lib.check("dmrg_batch_env_extend", self.lib.dmrg_batch_env_extend(
            side, self.cdtype, c, *args, _ptrs(Es), _ptrs(Ws), _ptrs(As), _ptrs(out), ptr, size, self.stream))
        return out

    def env_left(self, Ls, Ws, As):
        return self._env(0, Ls, Ws, As)

    def env_right(self, Rs, Ws, Bs):
        return self._env(1, Rs, Ws, Bs)

    def ground(self, Ls, Wis, Wjs, Rs, thetas):
        """Lowest eigenpairs of every chain's H_eff; thetas overwritten."""
        c = self.nchains
        ops = (_lib.HeffDesc * c)()
        keep = []
        for p in range(c):
            h = ops[p]
            cl, d1, d2, cr = thetas[p].shape
            h.kind, h.dtype, h.precision = 2, self.cdtype, _lib.PREC_FP64
            h.chil, h.d1, h.d2, h.chir = cl, d1, d2, cr
            h.wl, h.wm, h.wr = Wis[p].shape[0], Wis[p].shape[3], Wjs[p].shape[3]
            h.L, h.W1, h.W2, h.R = Ls[p].data_ptr(), Wis[p].data_ptr(), Wjs[p].data_ptr(), Rs[p].data_ptr()
            keep.append((Ls[p], Wis[p], Wjs[p], Rs[p]))
        kmax = int(min(self.niter_cap, max(int(t.numel()) for t in thetas)))
        need = self.lib.dmrg_batch_lanczos_workspace_bytes(c, ops, kmax)
        if need == 0:
            raise _lib.DmrgError("dmrg_batch_lanczos_workspace_bytes", _lib.DMRG_ERR_ARG, "invalid operator")
        ptr, size = self.ws.get(need)
        e = (ctypes.c_double * c)()
        it = (ctypes.c_int * c)()
        _lib.check("dmrg_batch_lanczos_ground", self.lib.dmrg_batch_lanczos_ground(
            c, ops, _ptrs(thetas), kmax, LANCZOS_TOL, int(self.use_graphs), e, it, ptr, size, self.stream))
        del keep
        self.lanczos_iters.append(list(it))
        return np.array(e[:])

    def svd(self, Ms, cutoff, maxdims, absorb, mindim=1):
        """Truncated SVD of every chain's 2-D matrix -> (lefts, rights, keeps)."""
        torch = _torch()
        c = self.nchains
        m = _arr(ctypes.c_int, [x.shape[0] for x in Ms])
        n = _arr(ctypes.c_int, [x.shape[1] for x in Ms])
        need = self.lib.dmrg_batch_svd_workspace_bytes(self.cdtype, c, m, n)
        ptr, size = self.ws.get(need)
        keep = (ctypes.c_int * c)()
        disc = (ctypes.c_double * c)()
        st = self.lib.dmrg_batch_svd_factor(self.cdtype, c, m, n, _ptrs(Ms), float(cutoff),
                                            _arr(ctypes.c_int, [int(x) for x in maxdims]), int(mindim), int(absorb),
                                            keep, disc, None, 0, ptr, size, self.stream)
        if st not in (_lib.DMRG_OK, _lib.DMRG_ERR_NOCONV):
            _lib.check("dmrg_batch_svd_factor", st)
        lefts = [torch.empty((x.shape[0], keep[p]), dtype=self.tdtype, device=self.device) for p, x in enumerate(Ms)]
        rights = [torch.empty((keep[p], x.shape[1]), dtype=self.tdtype, device=self.device) for p, x in enumerate(Ms)]
        _lib.check("dmrg_batch_svd_output", self.lib.dmrg_batch_svd_output(
            self.cdtype, c, m, n, keep, int(absorb), _ptrs(lefts), _ptrs(rights), ptr, size, self.stream))
        return lefts, rights, list(keep)

    # ------------------------------------------------------------ states
    def to_device(self, states):
        torch = _torch()
        npdt = np.float64 if self.real else np.complex128
        out = []
        for arrays in states:
            chain = []
            for a in arrays:
                a = np.asarray(a)
                if self.real and np.iscomplexobj(a):
                    a = a.real
                chain.append(torch.as_tensor(np.ascontiguousarray(a, dtype=npdt), device=self.device))
            out.append(chain)
        return out

    def random_states(self, dims, chi, seeds):
        """One seeded random MPS per chain (the reference's randomMPS draws,
        pyitensor/mpsalgebra.py:315-353, each chain from its own seed)."""
        states = []
        for sd in seeds:
            np.random.seed(int(sd))
            states.append(_mps.random_arrays(dims, chi))
        return self.to_device(states)

    def canonicalize(self, As):
        """Lossless left-to-right SVD pass with the centre carried to the
        last site and normalised, for every chain (as Engine.canonicalize_right_to_left_of)."""
        torch = _torch()
        for i in range(self.n - 1):
            Ms = [A[i].reshape(A[i].shape[0] * A[i].shape[1], A[i].shape[2]) for A in As]
            lo, ro, keep = self.svd(Ms, 0.0, [0] * self.nchains, 0)
            nxt = self.merge([r.view(r.shape[0], 1, r.shape[1]) for r in ro], [A[i + 1] for A in As])
            for p, A in enumerate(As):
                cl, d, cr = A[i].shape
                A[i] = lo[p].reshape(cl, d, keep[p])
                # the carried centre is renormalised at every step (its scale
                # grows along the chain and is irrelevant)
                x = nxt[p].reshape(keep[p], A[i + 1].shape[1], A[i + 1].shape[2])
                A[i + 1] = (x / torch.linalg.vector_norm(x)).contiguous()
        for A in As:
            A[-1] = (A[-1] / torch.linalg.vector_norm(A[-1])).contiguous()
        return As

    # ------------------------------------------------------------ sweeps
    def _column(self, store, i):
        return [s[i] for s in store]

    def sweep(self, As, maxdims, cutoff, renv=None):
        """One left-to-right and right-to-left two-site sweep of every chain
        (A modified in place); returns the energies of the last bond."""
        c, n = self.nchains, self.n
        W = self.W
        edge = [self.edge] * c
        if renv is None:
            renv = {n + 1: edge}
            for i in range(n, 1, -1):
                renv[i] = self.env_right(renv[i + 1], [W[p][i - 1] for p in range(c)], [A[i - 1] for A in As])
        lenv = {0: edge}
        energies = None
        for i in range(1, n):
            energies = self._bond(lenv[i - 1], renv[i + 2], As, i - 1, maxdims, cutoff, 0)
            lenv[i] = self.env_left(lenv[i - 1], [W[p][i - 1] for p in range(c)], [A[i - 1] for A in As])
        renv = {n + 1: edge}
        for i in range(n - 1, 0, -1):
            energies = self._bond(lenv[i - 1], renv[i + 2], As, i - 1, maxdims, cutoff, 1)
            renv[i + 1] = self.env_right(renv[i + 2], [W[p][i] for p in range(c)], [A[i] for A in As])
        return energies, renv

    def _bond(self, Ls, Rs, As, i, maxdims, cutoff, absorb):
        c = self.nchains
        thetas = self.merge([A[i] for A in As], [A[i + 1] for A in As])
        energies = self.ground(Ls, [self.W[p][i] for p in range(c)], [self.W[p][i + 1] for p in range(c)], Rs, thetas)
        Ms = [t.view(t.shape[0] * t.shape[1], t.shape[2] * t.shape[3]) for t in thetas]
        lo, ro, keep = self.svd(Ms, cutoff, maxdims, absorb)
        for p, A in enumerate(As):
            cl, d1, d2, cr = thetas[p].shape
            A[i] = lo[p].view(cl, d1, keep[p])
            A[i + 1] = ro[p].view(keep[p], d2, cr)
        return energies

    def dmrg(self, As, maxdims, nsweeps, cutoff=0.0):
        """nsweeps lock-step sweeps with per-chain bond caps maxdims."""
        renv = None
        energies = None
        for _ in range(nsweeps):
            energies, renv = self.sweep(As, maxdims, cutoff, renv)
        return energies
