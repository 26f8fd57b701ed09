"""MPS handle returned by the GB300 session, plus host-side measurements.

The handle is opaque to dmrgpy's glue code (``mps.py:8-21`` of dmrgpy only
ever calls ``copy()`` on it); it holds the site tensors as (chi_left, d,
chi_right) arrays with explicit dimension-1 edge links.  When dmrgpy itself
is importable, :meth:`MPS.to_pyitensor` converts to the python backend's MPS
object so every non-hot-path method of that backend can consume it.

The measurement helpers here (norms, overlaps, <bra|W|ket>, bond entropy)
run in NumPy on the host: they are parity checks and observables outside
the sweep, not part of the device hot path.
"""
import numpy as np


class MPS:
    def __init__(self, tensors, center=None):
        self.tensors = [np.asarray(t) for t in tensors]
        self.center = center

    def length(self):
        return len(self.tensors)

    def copy(self):
        return MPS([t.copy() for t in self.tensors], self.center)

    def dims(self):
        return [t.shape[2] for t in self.tensors[:-1]]

    def to_pyitensor(self, sites):
        """Convert to a ``dmrgpy.pyitensor.mpscontainer.MPS`` on the given
        ``SiteX`` (requires dmrgpy)."""
        from dmrgpy.pyitensor.index import Index
        from dmrgpy.pyitensor.mpscontainer import MPS as PyMPS
        from dmrgpy.pyitensor.tensor import ITensor
        n = self.length()
        links = [Index(t.shape[2], tags="Link,l={}".format(i + 1)) for i, t in enumerate(self.tensors[:-1])]
        out = []
        for i, t in enumerate(self.tensors):
            inds = ([links[i - 1]] if i > 0 else []) + [sites.si(i + 1)] + ([links[i]] if i < n - 1 else [])
            arr = t.reshape(tuple(ind.dim for ind in inds))
            out.append(ITensor(tuple(inds), arr.astype(complex)))
        m = PyMPS(out)
        m.center = self.center
        return m


def _dt(*arrs):
    return np.result_type(*[a.dtype for a in arrs], np.float64)


def inner(A, B):
    """<A|B>."""
    E = np.ones((1, 1), dtype=_dt(*(A + B)))
    for a, b in zip(A, B):
        x = np.tensordot(E, b, axes=([1], [0]))
        E = np.tensordot(a.conj(), x, axes=([0, 1], [0, 1]))
    return complex(E.reshape(-1)[0])


def expect(bra, W, ket):
    """<bra|W|ket> with W an MPO (w_left, d_in, d_out, w_right)."""
    L = np.ones((1, 1, 1), dtype=_dt(*(bra + ket + W)))
    for a, w, b in zip(bra, W, ket):
        x = np.tensordot(L, b, axes=([2], [0]))
        x = np.tensordot(x, w, axes=([1, 2], [0, 1]))
        L = np.tensordot(a.conj(), x, axes=([0, 1], [0, 2])).transpose(0, 2, 1)
    return complex(L.reshape(-1)[0])


def bond_entropy(A, b, cutoff_p=1e-12):
    """von Neumann entropy across bond (b, b+1), 1-based, with the p > 1e-12
    filter of pyitensor/chain.py:468-480.  Brings a copy into mixed
    canonical form first (QR sweeps from both ends)."""
    A = [a.copy() for a in A]
    n = len(A)
    for i in range(b - 1):
        cl, d, cr = A[i].shape
        Q, R = np.linalg.qr(A[i].reshape(cl * d, cr))
        A[i] = Q.reshape(cl, d, -1)
        A[i + 1] = np.tensordot(R, A[i + 1], axes=([1], [0]))
    for i in range(n - 1, b, -1):
        cl, d, cr = A[i].shape
        Q, R = np.linalg.qr(A[i].reshape(cl, d * cr).conj().T)
        A[i] = Q.conj().T.reshape(-1, d, cr)
        A[i - 1] = np.tensordot(A[i - 1], R.conj().T, axes=([2], [0]))
    theta = np.tensordot(A[b - 1], A[b], axes=([2], [0]))
    cl, d1, d2, cr = theta.shape
    s = np.linalg.svd(theta.reshape(cl * d1, d2 * cr), compute_uv=False)
    p = s ** 2
    p = p / p.sum()
    p = p[p > cutoff_p]
    return float(-np.sum(p * np.log(p)))


def random_arrays(dims, m, rng=np.random):
    """Site tensors of pyitensor/mpsalgebra.py:315-346: bond dimensions
    min(prod d, m) from both ends, complex Gaussian entries drawn from the
    global NumPy generator site by site (same draws as the reference for the
    same seed).  Canonicalisation and normalisation happen on the device."""
    n = len(dims)
    left_cum = 1
    bond = []
    for d in dims[:-1]:
        left_cum = min(left_cum * d, m)
        bond.append(left_cum)
    right_cum = 1
    for k in range(n - 2, -1, -1):
        right_cum = min(right_cum * dims[k + 1], m)
        bond[k] = min(bond[k], right_cum)
    out = []
    for i in range(n):
        cl = bond[i - 1] if i > 0 else 1
        cr = bond[i] if i < n - 1 else 1
        shape = tuple(([cl] if i > 0 else []) + [dims[i]] + ([cr] if i < n - 1 else []))
        arr = rng.randn(*shape) + 1j * rng.randn(*shape)
        out.append(arr.reshape(cl, dims[i], cr))
    return out
