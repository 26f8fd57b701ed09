"""Device-resident two-site DMRG / TDVP sweep driven through the C ABI.

The host loop mirrors the reference sweep structure
(``pyitensor/dmrg.py:355-398`` for DMRG, ``pyitensor/tdvp.py:220-368`` for
TDVP); every numerical step -- two-site merge, H_eff matvec, Lanczos /
Krylov-exponential loops, truncated SVD, environment extension -- runs as
CUDA kernels of libdmrg_gb300.so on tensors that stay in HBM.  PyTorch only
provides device memory and the stream.  There is no CPU fallback: without a
CUDA device the engine refuses to start.
"""
import ctypes
import time

import numpy as np

from . import _lib

LANCZOS_TOL = 1e-12          # pyitensor/dmrg.py:95
# The split-TF32 operator is a fixed (slightly biased, ~1e-7 relative)
# operator, so its Ritz values converge as smoothly as in FP64 and the same
# relative test applies; the bias is removed by the FP64 energy refinement.
LANCZOS_TOL_TF32 = 1e-12
TF32_MIN_CHI = 32            # bonds with a smaller chi stay on the FP64 path
# bonds where maxdim binds factorise theta by warm-started subspace
# iteration plus Rayleigh-Ritz once min(m, n) reaches this size (split-TF32
# products in tf32x3 sweeps, FP64 products in fp64 sweeps and on every
# split-TF32 bond where the cutoff may bind); smaller bonds take the full
# Gram-matrix route of dmrg_svd_truncate
SUBSPACE_MIN_DIM = 256
LANCZOS_NITER_FLOOR = 200    # pyitensor/dmrg.py:315-330
KRYLOV_ERRGOAL = 1e-10       # pyitensor/tdvp.py:79
KRYLOV_TOL = 1e-12           # pyitensor/tdvp.py:82


def _torch():
    import torch
    return torch


class Workspace:
    """One growing device scratch buffer shared by all entry points (calls
    are stream-ordered, so reuse is safe)."""

    def __init__(self, device):
        self.device = device
        self.buf = None

    def get(self, nbytes):
        torch = _torch()
        nbytes = int(max(nbytes, 256))
        if self.buf is None or self.buf.numel() < nbytes:
            self.buf = None
            self.buf = torch.empty(int(nbytes * 1.25) + 4096, dtype=torch.uint8, device=self.device)
        return self.buf.data_ptr(), self.buf.numel()


class SweepStats:
    def __init__(self):
        self.records = []
        self.t = {"lanczos": 0.0, "svd": 0.0, "env": 0.0, "merge": 0.0}
        self.matvecs = 0
        self.matvec_flops = 0.0
        self.fp64_truncations = 0   # split-TF32 bonds whose cutoff the FP64 route decided

    def add(self, **kw):
        self.records.append(kw)


class Engine:
    """Sweeps over an MPO held on the device.

    W: list of (w_left, d, d, w_right) numpy arrays; real: element type.
    precision: "fp64" or "tf32x3" (split-TF32 contractions, real only).
    """

    def __init__(self, W, real=True, precision="fp64", device="cuda:0", krylov_budget_bytes=32 << 30):
        torch = _torch()
        if not torch.cuda.is_available():
            raise RuntimeError("dmrgpy_gb300 needs a CUDA device (GB300); no CPU fallback exists")
        self.lib = _lib.load()
        self.device = torch.device(device)
        self.real = bool(real)
        self.tdtype = torch.float64 if self.real else torch.complex128
        self.cdtype = _lib.REAL64 if self.real else _lib.COMPLEX128
        self.esize = 8 if self.real else 16
        if precision not in ("fp64", "tf32x3"):
            raise ValueError("precision must be 'fp64' or 'tf32x3'")
        if precision == "tf32x3" and not self.real:
            raise ValueError("tf32x3 contractions are built for real MPOs only")
        self.precision = precision
        self.prec = _lib.PREC_FP64 if precision == "fp64" else _lib.PREC_TF32X3
        self.W = [torch.as_tensor(np.ascontiguousarray(w, dtype=np.float64 if self.real else np.complex128),
                                  device=self.device) for w in W]
        self.n = len(W)
        self.ws = Workspace(self.device)
        self.edge = torch.ones((1, 1, 1), dtype=self.tdtype, device=self.device)
        self.krylov_budget = krylov_budget_bytes
        self.stats = SweepStats()
        self._renv = None  # right environments valid for the current MPS (after a RL pass)
        self.subspace_iters = 1     # subspace iterations per fixed-rank truncation
        # optional callable(theta (m x n device matrix), cutoff, maxdim, keep,
        # discarded) run after every bond truncation (tests inspect the
        # two-site tensors of a sweep with it)
        self.theta_hook = None
        self.last_spectrum = None
        # split-TF32 subspace truncations also return the Ritz values of the
        # kept problem (an FP32 Jacobi per bond); off in sweeps by default
        self.want_spectra = False
        self.lanczos_tol_tf32 = LANCZOS_TOL_TF32

    # ------------------------------------------------------------ plumbing
    @property
    def stream(self):
        return ctypes.c_void_p(_torch().cuda.current_stream(self.device).cuda_stream)

    def to_device(self, arrays):
        torch = _torch()
        out = []
        for a in arrays:
            a = np.asarray(a)
            if self.real:
                a = a.real if np.iscomplexobj(a) else a
                a = np.ascontiguousarray(a, dtype=np.float64)
            else:
                a = np.ascontiguousarray(a, dtype=np.complex128)
            out.append(torch.as_tensor(a, device=self.device))
        return out

    def to_host(self, tensors):
        return [t.detach().cpu().numpy() for t in tensors]

    def prec_for(self, cl, cr):
        """Split-TF32 for the bulk bonds, FP64 for the small edge bonds."""
        if self.prec == _lib.PREC_TF32X3 and min(cl, cr) >= TF32_MIN_CHI:
            return _lib.PREC_TF32X3
        return _lib.PREC_FP64

    def _heff(self, kind, L, W1, W2, R, cl, d1, d2, cr, wl, wm, wr):
        h = _lib.HeffDesc()
        h.kind, h.dtype = kind, self.cdtype
        h.precision = self.prec_for(cl, cr) if kind == 2 else _lib.PREC_FP64
        h.chil, h.d1, h.d2, h.chir = cl, d1, d2, cr
        h.wl, h.wm, h.wr = wl, wm, wr
        h.L = L.data_ptr()
        h.R = R.data_ptr()
        h.W1 = W1.data_ptr() if W1 is not None else None
        h.W2 = W2.data_ptr() if W2 is not None else None
        # the descriptor holds raw device pointers: keep the tensors alive
        # for as long as the descriptor is
        h._keep = (L, W1, W2, R)
        return h

    def heff2(self, L, Wi, Wj, R, theta_shape):
        cl, d1, d2, cr = theta_shape
        return self._heff(2, L, Wi, Wj, R, cl, d1, d2, cr, Wi.shape[0], Wi.shape[3], Wj.shape[3])

    def heff1(self, L, W, R, a_shape):
        cl, d, cr = a_shape
        return self._heff(1, L, W, None, R, cl, d, 1, cr, W.shape[0], W.shape[3], W.shape[3])

    def heff0(self, L, R, c_shape):
        cl, cr = c_shape
        w = L.shape[1]
        return self._heff(0, L, None, None, R, cl, 1, 1, cr, w, w, w)

    def apply(self, h, x):
        """y = H_eff x (one matvec; used by tests and the benchmark)."""
        torch = _torch()
        y = torch.empty_like(x)
        need = self.lib.dmrg_heff_workspace_bytes(ctypes.byref(h))
        ptr, size = self.ws.get(need)
        _lib.check("dmrg_heff_apply", self.lib.dmrg_heff_apply(ctypes.byref(h), x.data_ptr(), y.data_ptr(),
                                                                 ptr, size, self.stream))
        return y

    def _kcap(self, n, niter):
        cap = max(8, int(self.krylov_budget // max(1, n * self.esize)))
        return int(min(niter, cap))

    def ground(self, h, x, niter):
        """Lowest eigenpair of H_eff; x (contiguous) is overwritten by the
        normalised eigenvector."""
        k = self._kcap(x.numel(), max(niter, LANCZOS_NITER_FLOOR))
        need = self.lib.dmrg_lanczos_workspace_bytes(ctypes.byref(h), k)
        ptr, size = self.ws.get(need)
        e = ctypes.c_double(0.0)
        it = ctypes.c_int(0)
        tol = self.lanczos_tol_tf32 if h.precision == _lib.PREC_TF32X3 else LANCZOS_TOL
        _lib.check("dmrg_lanczos_ground", self.lib.dmrg_lanczos_ground(
            ctypes.byref(h), x.data_ptr(), k, tol, ctypes.byref(e), ctypes.byref(it), ptr, size, self.stream))
        return e.value, it.value

    def expm(self, h, x, coeff, niter):
        k = self._kcap(x.numel(), niter)
        need = self.lib.dmrg_expm_workspace_bytes(ctypes.byref(h), k)
        ptr, size = self.ws.get(need)
        it = ctypes.c_int(0)
        coeff = complex(coeff)
        _lib.check("dmrg_krylov_expm", self.lib.dmrg_krylov_expm(
            ctypes.byref(h), x.data_ptr(), coeff.real, coeff.imag, k, KRYLOV_TOL, KRYLOV_ERRGOAL,
            ctypes.byref(it), ptr, size, self.stream))
        return it.value

    def gemm(self, A2, B2):
        """C = A2 @ B2 for 2-D contiguous device tensors."""
        torch = _torch()
        m, k = A2.shape
        k2, n = B2.shape
        assert k == k2
        C = torch.empty((m, n), dtype=self.tdtype, device=self.device)
        prec = self.prec_for(min(m, n), k)
        need = self.lib.dmrg_gemm_workspace_bytes(self.cdtype, prec, m, k, n)
        ptr, size = self.ws.get(need)
        _lib.check("dmrg_gemm", self.lib.dmrg_gemm(self.cdtype, prec, m, k, n, A2.data_ptr(), B2.data_ptr(),
                                                   C.data_ptr(), ptr, size, self.stream))
        return C

    def merge(self, Ai, Aj):
        cl, d1, cm = Ai.shape
        _, d2, cr = Aj.shape
        return self.gemm(Ai.reshape(cl * d1, cm), Aj.reshape(cm, d2 * cr)).reshape(cl, d1, d2, cr)

    def svd(self, M2, cutoff, maxdim, mindim=1, absorb=0):
        """Truncated SVD of a 2-D device matrix -> (left, right, s, keep, disc)."""
        torch = _torch()
        m, n = M2.shape
        cap = min(m, n) if not maxdim or maxdim <= 0 else min(m, n, maxdim)
        lo = torch.empty(m * cap, dtype=self.tdtype, device=self.device)
        ro = torch.empty(cap * n, dtype=self.tdtype, device=self.device)
        s = np.zeros(min(m, n), dtype=np.float64)
        keep = ctypes.c_int(0)
        disc = ctypes.c_double(0.0)
        need = self.lib.dmrg_svd_workspace_bytes(self.cdtype, m, n)
        ptr, size = self.ws.get(need)
        st = self.lib.dmrg_svd_truncate(self.cdtype, m, n, M2.data_ptr(), float(cutoff),
                                        int(maxdim) if maxdim else 0, int(mindim), int(absorb),
                                        lo.data_ptr(), ro.data_ptr(),
                                        s.ctypes.data_as(_lib.P_double), ctypes.byref(keep), ctypes.byref(disc),
                                        ptr, size, self.stream)
        _lib.check("dmrg_svd_truncate", st)
        k = keep.value
        return lo[:m * k].view(m, k), ro[:k * n].view(k, n), s, k, disc.value

    def subspace_split(self, M2, k, start, kstart, absorb, cutoff=0.0, mindim=1, prec=None):
        """Truncation of a 2-D device matrix to at most k vectors by
        warm-started subspace iteration plus Rayleigh-Ritz, with the cutoff
        rule: -> (left, right, s, keep, disc).  prec: the engine's precision
        by default; split-TF32 raises DmrgError(DMRG_ERR_PRECISION) where
        its weights cannot decide the cutoff.  s holds the singular-value
        estimates (FP64 route) or, with want_spectra, the FP32-accurate
        Ritz values (split-TF32 route); else None."""
        torch = _torch()
        m, n = M2.shape
        if prec is None:
            prec = self.prec if self.prec == _lib.PREC_TF32X3 else _lib.PREC_FP64
        lo = torch.empty(m * k, dtype=self.tdtype, device=self.device)
        ro = torch.empty(k * n, dtype=self.tdtype, device=self.device)
        disc = ctypes.c_double(0.0)
        keep = ctypes.c_int(0)
        want = prec == _lib.PREC_FP64 or self.want_spectra
        s = np.zeros(k, dtype=np.float64) if want else None
        need = self.lib.dmrg_subspace_truncate_ex_workspace_bytes(prec, m, n, k)
        ptr, size = self.ws.get(need)
        st = self.lib.dmrg_subspace_truncate_ex(prec, m, n, k, M2.data_ptr(),
                                                start.data_ptr() if start is not None else None,
                                                int(kstart), int(absorb), int(self.subspace_iters), float(cutoff),
                                                int(mindim), lo.data_ptr(), ro.data_ptr(),
                                                s.ctypes.data_as(_lib.P_double) if s is not None else None,
                                                ctypes.byref(keep), ctypes.byref(disc), ptr, size, self.stream)
        _lib.check("dmrg_subspace_truncate_ex", st)
        kp = keep.value
        return lo[:m * kp].view(m, kp), ro[:kp * n].view(kp, n), s, kp, disc.value

    def use_subspace(self, m, n, cutoff, maxdim, absorb=0):
        """Real sweeps on a large bond use the subspace route (split-TF32 or
        FP64 products by the engine's precision) where maxdim binds, and
        where the full rank min(m, n) is kept but the kept side is more than
        twice that (a Gram matrix of the kept side would be oversized; with
        the other side's tensor as the start the subspace is then exact);
        split-TF32 sweeps without a cutoff take it for every full-rank bond."""
        if not (self.real and maxdim and maxdim > 0):
            return False
        c = min(m, n)
        if self.prec == _lib.PREC_TF32X3 and cutoff <= 0.0 and maxdim >= c:
            # the full rank is kept: the subspace is exact at any size
            return True
        if c < SUBSPACE_MIN_DIM:
            return False
        if maxdim < c:
            return True
        kept = m if absorb == 0 else n
        return kept > 2 * c

    def use_identity_split(self, m, n, cutoff, maxdim, absorb):
        """Split-TF32 sweeps that keep the whole kept side with no cutoff:
        the identity is an exact orthonormal basis and theta the other
        factor, so nothing is factorised."""
        if not (self.prec == _lib.PREC_TF32X3 and self.real and cutoff <= 0.0 and maxdim and maxdim > 0):
            return False
        rank = min(maxdim, m, n)
        return (absorb == 0 and rank == m) or (absorb == 1 and rank == n)

    def env_left(self, L, W, A, fp64=False):
        torch = _torch()
        cl, d, cr = A.shape
        wl, wr = W.shape[0], W.shape[3]
        out = torch.empty((cr, wr, cr), dtype=self.tdtype, device=self.device)
        prec = self.prec_for(cl, cr) if fp64 is False else _lib.PREC_FP64
        need = self.lib.dmrg_env_workspace_bytes(self.cdtype, prec, cl, d, cr, wl, wr)
        ptr, size = self.ws.get(need)
        _lib.check("dmrg_env_extend_left", self.lib.dmrg_env_extend_left(
            self.cdtype, prec, cl, d, cr, wl, wr, L.data_ptr(), W.data_ptr(), A.data_ptr(), out.data_ptr(),
            ptr, size, self.stream))
        return out

    def env_right(self, R, W, B, fp64=False):
        torch = _torch()
        cl, d, cr = B.shape
        wl, wr = W.shape[0], W.shape[3]
        out = torch.empty((cl, wl, cl), dtype=self.tdtype, device=self.device)
        prec = self.prec_for(cl, cr) if fp64 is False else _lib.PREC_FP64
        need = self.lib.dmrg_env_workspace_bytes(self.cdtype, prec, cl, d, cr, wl, wr)
        ptr, size = self.ws.get(need)
        _lib.check("dmrg_env_extend_right", self.lib.dmrg_env_extend_right(
            self.cdtype, prec, cl, d, cr, wl, wr, R.data_ptr(), W.data_ptr(), B.data_ptr(), out.data_ptr(),
            ptr, size, self.stream))
        return out

    def env_gradient(self, L, A, R, wl, wr):
        """d<psi|H|psi>/dW for one site: (wl, d, d, wr), FP64."""
        torch = _torch()
        cl, d, cr = A.shape
        out = torch.empty((wl, d, d, wr), dtype=self.tdtype, device=self.device)
        need = self.lib.dmrg_env_gradient_workspace_bytes(self.cdtype, cl, d, cr, wl, wr)
        ptr, size = self.ws.get(need)
        _lib.check("dmrg_env_gradient", self.lib.dmrg_env_gradient(
            self.cdtype, cl, d, cr, wl, wr, L.data_ptr(), A.data_ptr(), R.data_ptr(), out.data_ptr(),
            ptr, size, self.stream))
        return out

    # ------------------------------------------------------------ transition forms
    def env_mixed(self, side, E, W, B, A):
        """Transition environment with bra B and ket A (side 0: left, 1: right), FP64."""
        torch = _torch()
        clb, d, crb = B.shape
        clk, _, crk = A.shape
        wl, wr = W.shape[0], W.shape[3]
        shape = (crb, wr, crk) if side == 0 else (clb, wl, clk)
        out = torch.empty(shape, dtype=self.tdtype, device=self.device)
        need = self.lib.dmrg_env_mixed_workspace_bytes(side, self.cdtype, clb, crb, clk, crk, d, wl, wr)
        ptr, size = self.ws.get(need)
        _lib.check("dmrg_env_extend_mixed", self.lib.dmrg_env_extend_mixed(
            side, self.cdtype, clb, crb, clk, crk, d, wl, wr, E.data_ptr(), W.data_ptr(), B.data_ptr(),
            A.data_ptr(), out.data_ptr(), ptr, size, self.stream))
        return out

    def transition_gradients(self, Bra, Ket):
        """<bra|H|ket> and G_i = d<bra|H|ket>/dW_i for every site (FP64, no
        normalisation): the adjoint pass of mpo_gradients with two states."""
        torch = _torch()
        n = len(Ket)
        R = {n + 1: self.edge}
        for i in range(n, 1, -1):
            R[i] = self.env_mixed(1, R[i + 1], self.W[i - 1], Bra[i - 1], Ket[i - 1])
        L = self.edge
        grads = []
        for i in range(n):
            W = self.W[i]
            B, A = Bra[i], Ket[i]
            clb, d, crb = B.shape
            clk, _, crk = A.shape
            wl, wr = W.shape[0], W.shape[3]
            G = torch.empty((wl, d, d, wr), dtype=self.tdtype, device=self.device)
            need = self.lib.dmrg_env_gradient_mixed_workspace_bytes(self.cdtype, clb, crb, clk, crk, d, wl, wr)
            ptr, size = self.ws.get(need)
            _lib.check("dmrg_env_gradient_mixed", self.lib.dmrg_env_gradient_mixed(
                self.cdtype, clb, crb, clk, crk, d, wl, wr, L.data_ptr(), B.data_ptr(), A.data_ptr(),
                R[i + 2].data_ptr(), G.data_ptr(), ptr, size, self.stream))
            grads.append(G)
            L = self.env_mixed(0, L, W, B, A)
        return complex(L.reshape(-1)[0].item()), grads

    # ------------------------------------------------------------ measurements
    def transition(self, W, bra, ket):
        """<bra|W|ket> on the device in FP64 (pyitensor/mpsalgebra.py:66-106,
        inner with an MPO): the left transition environment carried across
        the chain.  W: device MPO tensors of the engine's dtype (self.W for
        the engine's own operator); bra, ket: device site tensors."""
        L = self.edge
        for w, b, a in zip(W, bra, ket):
            L = self.env_mixed(0, L, w, b, a)
        return complex(L.reshape(-1)[0].item())

    def identity_mpo(self, dims):
        torch = _torch()
        return [torch.eye(d, dtype=self.tdtype, device=self.device).reshape(1, d, d, 1).contiguous() for d in dims]

    def bond_spectrum(self, A, b):
        """Schmidt values across bond (b, b+1), 1-based, of the device MPS A
        (descending, host array): a copy is brought into mixed canonical
        form by lossless device factorisations from both ends and the
        two-site tensor across the bond factorised (the measurement of
        pyitensor/chain.py:468-480)."""
        A = [a.clone() for a in A]
        n = len(A)
        for i in range(b - 1):
            cl, d, cr = A[i].shape
            lo, ro, _, k, _ = self.svd(A[i].reshape(cl * d, cr), -1.0, 0, 1, 0)
            A[i] = lo.reshape(cl, d, k)
            nxt = A[i + 1]
            A[i + 1] = self.gemm(ro, nxt.reshape(cr, -1)).reshape(k, nxt.shape[1], nxt.shape[2])
        for i in range(n - 1, b, -1):
            cl, d, cr = A[i].shape
            lo, ro, _, k, _ = self.svd(A[i].reshape(cl, d * cr), -1.0, 0, 1, 1)
            A[i] = ro.reshape(k, d, cr)
            prv = A[i - 1]
            A[i - 1] = self.gemm(prv.reshape(-1, cl), lo).reshape(prv.shape[0], prv.shape[1], k)
        theta = self.merge(A[b - 1].contiguous(), A[b].contiguous())
        cl, d1, d2, cr = theta.shape
        _, _, s, _, _ = self.svd(theta.reshape(cl * d1, d2 * cr), -1.0, 0, 1, 2)
        return np.asarray(s, dtype=np.float64)

    def right_canonicalize(self, A):
        """Lossless right-to-left SVD pass: A[1:] right-orthonormal, the
        norm carried into A[0] (the gauge the TDVP sweep starts from)."""
        for i in range(len(A) - 1, 0, -1):
            cl, d, cr = A[i].shape
            lo, ro, _, k, _ = self.svd(A[i].reshape(cl, d * cr), 0.0, 0, 1, 1)
            A[i] = ro.reshape(k, d, cr)
            prv = A[i - 1]
            A[i - 1] = self.gemm(prv.reshape(-1, cl), lo).reshape(prv.shape[0], prv.shape[1], k)
        return A

    def set_mpo(self, W):
        """Replace the MPO tensors (same shapes), e.g. after a change of couplings."""
        torch = _torch()
        if len(W) != self.n or any(tuple(w.shape) != tuple(v.shape) for w, v in zip(W, self.W)):
            raise ValueError("set_mpo needs tensors of the current MPO's shapes")
        self.W = [torch.as_tensor(np.ascontiguousarray(w, dtype=np.float64 if self.real else np.complex128),
                                  device=self.device) for w in W]
        self.invalidate()

    def mpo_gradients(self, A):
        """Energy and its adjoint at a fixed state, all in FP64:
        E = <psi|H|psi>/<psi|psi> and G_i = dE/dW_i for every site.

        One right-to-left pass stores the right environments; a left-to-right
        pass carries the left (and norm) environment and evaluates
        dmrg_env_gradient at each site, so the cost is three environment
        sweeps for the gradient with respect to every MPO tensor at once."""
        torch = _torch()
        n = len(A)
        R = {n + 1: self.edge}
        for i in range(n, 1, -1):
            R[i] = self.env_right(R[i + 1], self.W[i - 1], A[i - 1], fp64=True)
        L = self.edge
        Nn = self.edge
        grads = []
        for i in range(n):
            W = self.W[i]
            grads.append(self.env_gradient(L, A[i], R[i + 2], W.shape[0], W.shape[3]))
            d = A[i].shape[1]
            ident = torch.eye(d, dtype=self.tdtype, device=self.device).reshape(1, d, d, 1).contiguous()
            L = self.env_left(L, W, A[i], fp64=True)
            Nn = self.env_left(Nn, ident, A[i], fp64=True)
            if i + 2 in R and i + 2 <= n:
                del R[i + 2]
        nrm = Nn.reshape(-1)[0].real
        e = L.reshape(-1)[0] / nrm
        grads = [g / nrm for g in grads]
        return float(e.real.item()), grads

    def right_envs(self, A):
        n = len(A)
        env = {n + 1: self.edge}
        for i in range(n, 1, -1):
            env[i] = self.env_right(env[i + 1], self.W[i - 1], A[i - 1])
        return env

    def left_envs(self, A):
        n = len(A)
        env = {0: self.edge}
        for i in range(1, n):
            env[i] = self.env_left(env[i - 1], self.W[i - 1], A[i - 1])
        return env

    # ------------------------------------------------------------ DMRG
    @staticmethod
    def heff2_flops(cl, d1, d2, cr, wl, wm, wr, complex_=False):
        """Algorithmic FLOPs of one two-site matvec (2 per real MAC; complex
        MACs count 4 real MACs)."""
        macs = cl * wl * cl * d1 * d2 * cr + cl * d1 * wm * wl * d1 * d2 * cr \
            + cl * d1 * d2 * wr * wm * d2 * cr + cl * d1 * d2 * cr * wr * cr
        return 2.0 * macs * (4 if complex_ else 1)

    def _bond_update(self, L, Wi, Wj, R, Ai, Aj, niter, cutoff, maxdim, absorb, record):
        torch = _torch()
        t0 = time.perf_counter()
        theta = self.merge(Ai, Aj).contiguous()
        t1 = time.perf_counter()
        h = self.heff2(L, Wi, Wj, R, theta.shape)
        energy, iters = self.ground(h, theta, niter)
        t2 = time.perf_counter()
        cl, d1, d2, cr = theta.shape
        m, n = cl * d1, d2 * cr
        rank = min(maxdim, m, n) if maxdim and maxdim > 0 else min(m, n)
        if self.use_identity_split(m, n, cutoff, maxdim, absorb):
            # nothing to truncate on the kept side: the identity is an exact
            # orthonormal basis of it and theta itself the other factor
            eye = torch.eye(rank, dtype=self.tdtype, device=self.device)
            tm = theta.view(m, n)
            lo, ro = (eye, tm) if absorb == 0 else (tm, eye)
            s, keep, disc = None, rank, 0.0
        elif self.use_subspace(m, n, cutoff, maxdim, absorb):
            # warm start: the orthonormal tensor on the other side of the bond
            # (right-canonical A_j in a left-to-right pass, left-canonical A_i
            # in a right-to-left pass)
            if absorb == 0:
                start = Aj.reshape(Aj.shape[0], n)
                kx = min(start.shape[0], rank)
                start = start[:kx].contiguous()
            else:
                start = Ai.reshape(m, Ai.shape[2])
                kx = min(start.shape[1], rank)
                start = start[:, :kx].contiguous()
            try:
                try:
                    lo, ro, s, keep, disc = self.subspace_split(theta.view(m, n), rank, start, kx, absorb, cutoff)
                except _lib.DmrgError as ex:
                    if ex.status != _lib.DMRG_ERR_PRECISION:
                        raise
                    # the cutoff may bind here: the FP64 route decides it
                    self.stats.fp64_truncations += 1
                    lo, ro, s, keep, disc = self.subspace_split(theta.view(m, n), rank, start, kx, absorb, cutoff,
                                                                prec=_lib.PREC_FP64)
            except _lib.DmrgError as ex:
                if ex.status != _lib.DMRG_ERR_NOCONV:
                    raise
                # the basis could not be made orthonormal: the full FP64
                # truncation
                lo, ro, s, keep, disc = self.svd(theta.view(m, n), cutoff, maxdim, 1, absorb)
        else:
            lo, ro, s, keep, disc = self.svd(theta.view(m, n), cutoff, maxdim, 1, absorb)
        t3 = time.perf_counter()
        if self.theta_hook is not None:
            self.theta_hook(theta.view(m, n), cutoff, maxdim, keep, disc)
        st = self.stats
        st.t["merge"] += t1 - t0
        st.t["lanczos"] += t2 - t1
        st.t["svd"] += t3 - t2
        st.matvecs += iters
        st.matvec_flops += iters * self.heff2_flops(cl, d1, d2, cr, Wi.shape[0], Wi.shape[3], Wj.shape[3],
                                                    not self.real)
        if record:
            st.add(energy=energy, iters=iters, keep=keep, disc=disc, chil=cl, chir=cr)
        self.last_spectrum = None if s is None else np.asarray(s[:keep], dtype=np.float64).copy()
        return energy, lo.view(cl, d1, keep), ro.view(keep, d2, cr), s, keep, disc

    def sweep(self, A, maxdim, cutoff, niter=2, record=False):
        """One left-to-right then right-to-left two-site sweep on the list of
        device site tensors A (modified in place); returns the last bond's
        eigenvalue (pyitensor/dmrg.py:355-382)."""
        n = len(A)
        W = self.W
        renv = self._renv if self._renv is not None else self.right_envs(A)
        lenv = {0: self.edge}
        energy = None
        for i in range(1, n):
            energy, A[i - 1], A[i], _, _, _ = self._bond_update(
                lenv[i - 1], W[i - 1], W[i], renv[i + 2], A[i - 1], A[i], niter, cutoff, maxdim, 0, record)
            t0 = time.perf_counter()
            lenv[i] = self.env_left(lenv[i - 1], W[i - 1], A[i - 1])
            self.stats.t["env"] += time.perf_counter() - t0
        renv = {n + 1: self.edge}
        for i in range(n - 1, 0, -1):
            energy, A[i - 1], A[i], _, _, _ = self._bond_update(
                lenv[i - 1], W[i - 1], W[i], renv[i + 2], A[i - 1], A[i], niter, cutoff, maxdim, 1, record)
            t0 = time.perf_counter()
            renv[i + 1] = self.env_right(renv[i + 2], W[i], A[i])
            self.stats.t["env"] += time.perf_counter() - t0
        # the right environments now match A exactly (every A[i], i >= 2, was
        # finalised before its environment was built), so the next sweep
        # reuses them instead of rebuilding (pyitensor/dmrg.py:365 rebuilds)
        self._renv = renv
        return energy

    def dmrg(self, A, maxdims, cutoffs, niters=2, record=False):
        """pyitensor/dmrg.py:385-398 with one (maxdim, cutoff, niter) per sweep."""
        nsw = len(maxdims)
        cutoffs = list(cutoffs) if isinstance(cutoffs, (list, tuple)) else [cutoffs] * nsw
        niters = list(niters) if isinstance(niters, (list, tuple)) else [niters] * nsw
        self._renv = None
        energy = None
        for s in range(nsw):
            energy = self.sweep(A, maxdims[s], cutoffs[s], niters[s], record)
        return energy

    def invalidate(self):
        self._renv = None

    def energy_fp64(self, A):
        """FP64 refinement of the energy: <psi|H|psi> / <psi|psi> with every
        environment recomputed in FP64 (used after split-TF32 sweeps)."""
        torch = _torch()
        L = self.edge
        N = self.edge
        for i, a in enumerate(A):
            d = a.shape[1]
            ident = torch.eye(d, dtype=self.tdtype, device=self.device).reshape(1, d, d, 1)
            L = self.env_left(L, self.W[i], a, fp64=True)
            N = self.env_left(N, ident.contiguous(), a, fp64=True)
        return float(L.reshape(-1)[0].real.item() / N.reshape(-1)[0].real.item())

    # ------------------------------------------------------------ initial state
    def canonicalize_right_to_left_of(self, A):
        """Lossless left-to-right SVD pass (centre ends at the last site) and
        normalisation: pyitensor/mpsalgebra.py:347-352 (position(n), normalize)."""
        torch = _torch()
        n = len(A)
        for i in range(n - 1):
            cl, d, cr = A[i].shape
            lo, ro, s, keep, _ = self.svd(A[i].reshape(cl * d, cr), 0.0, 0, 1, 0)
            A[i] = lo.reshape(cl, d, keep)
            nxt = self.gemm(ro, A[i + 1].reshape(cr, -1))
            # the carried centre grows by ~|A| per site (1e100 and more over a
            # long chain); its scale is irrelevant because the state is
            # normalised at the end, so keep it O(1)
            nxt = nxt / torch.linalg.vector_norm(nxt)
            A[i + 1] = nxt.reshape(keep, A[i + 1].shape[1], A[i + 1].shape[2])
        nrm = float(_torch().linalg.vector_norm(A[n - 1]).item())
        A[n - 1] = A[n - 1] / nrm
        return A

    # ------------------------------------------------------------ TDVP
    def _evolve2(self, L, Wi, Wj, R, theta, coeff, niter):
        h = self.heff2(L, Wi, Wj, R, theta.shape)
        self.expm(h, theta, coeff, niter)
        return theta

    def _evolve1(self, L, W, R, A, coeff, niter):
        A = A.contiguous().clone()
        h = self.heff1(L, W, R, A.shape)
        self.expm(h, A, coeff, niter)
        return A

    def _evolve0(self, L, R, C, coeff, niter):
        C = C.contiguous().clone()
        h = self.heff0(L, R, C.shape)
        self.expm(h, C, coeff, niter)
        return C

    def tdvp_step(self, A, dt, cutoff, maxdim, niter=50, num_center=2):
        """One step exp(-i dt H): two half sweeps of dt/2 (pyitensor/tdvp.py:350-368)."""
        if self.real:
            raise ValueError("real-time TDVP needs a complex engine (real=False)")
        tau = dt / 2.0
        n = len(A)
        W = self.W
        self._renv = None
        if num_center == 1:
            renv = self.right_envs(A)
            lenv = {0: self.edge}
            for i in range(1, n + 1):
                Anew = self._evolve1(lenv[i - 1], W[i - 1], renv[i + 1], A[i - 1], -1j * tau, niter)
                if i == n:
                    A[i - 1] = Anew
                    continue
                cl, d, cr = Anew.shape
                Q, C, _, k, _ = self.svd(Anew.reshape(cl * d, cr), -1.0, 0, 1, 0)
                A[i - 1] = Q.reshape(cl, d, k)
                lenv[i] = self.env_left(lenv[i - 1], W[i - 1], A[i - 1])
                Cev = self._evolve0(lenv[i], renv[i + 1], C, 1j * tau, niter)
                nxt = A[i]
                A[i] = self.gemm(Cev, nxt.reshape(cr, -1)).reshape(k, nxt.shape[1], nxt.shape[2])
            lenv = self.left_envs(A)
            renv = {n + 1: self.edge}
            for i in range(n, 0, -1):
                Anew = self._evolve1(lenv[i - 1], W[i - 1], renv[i + 1], A[i - 1], -1j * tau, niter)
                if i == 1:
                    A[0] = Anew
                    continue
                cl, d, cr = Anew.shape
                C, V, _, k, _ = self.svd(Anew.reshape(cl, d * cr), -1.0, 0, 1, 1)
                A[i - 1] = V.reshape(k, d, cr)
                renv[i] = self.env_right(renv[i + 1], W[i - 1], A[i - 1])
                Cev = self._evolve0(lenv[i - 1], renv[i], C, 1j * tau, niter)
                prv = A[i - 2]
                A[i - 2] = self.gemm(prv.reshape(-1, cl), Cev).reshape(prv.shape[0], prv.shape[1], k)
            return A
        # two-site
        renv = self.right_envs(A)
        lenv = {0: self.edge}
        for i in range(1, n):
            theta = self.merge(A[i - 1], A[i]).contiguous()
            theta = self._evolve2(lenv[i - 1], W[i - 1], W[i], renv[i + 2], theta, -1j * tau, niter)
            cl, d1, d2, cr = theta.shape
            U, C, _, k, _ = self.svd(theta.view(cl * d1, d2 * cr), cutoff, maxdim, 1, 0)
            A[i - 1] = U.reshape(cl, d1, k)
            A[i] = C.reshape(k, d2, cr)
            lenv[i] = self.env_left(lenv[i - 1], W[i - 1], A[i - 1])
            if i < n - 1:
                A[i] = self._evolve1(lenv[i], W[i], renv[i + 2], A[i], 1j * tau, niter)
        lenv = self.left_envs(A)
        renv = {n + 1: self.edge}
        for i in range(n - 1, 0, -1):
            theta = self.merge(A[i - 1], A[i]).contiguous()
            theta = self._evolve2(lenv[i - 1], W[i - 1], W[i], renv[i + 2], theta, -1j * tau, niter)
            cl, d1, d2, cr = theta.shape
            C, V, _, k, _ = self.svd(theta.view(cl * d1, d2 * cr), cutoff, maxdim, 1, 1)
            A[i] = V.reshape(k, d2, cr)
            A[i - 1] = C.reshape(cl, d1, k)
            renv[i + 1] = self.env_right(renv[i + 2], W[i], A[i])
            if i > 1:
                A[i - 1] = self._evolve1(lenv[i - 1], W[i - 1], renv[i + 1], A[i - 1], 1j * tau, niter)
        return A
