"""Generate tests/golden/reference_truncation.npz: truncated factorisations
of REAL matrices computed by dmrgpy's own pure-Python backend
(``pyitensor/svd.py``: ``svd`` with its Gram-matrix route and ``_truncate``
rule), the golden values of the Gram-matrix truncation route.

Run from the repository root with the reference checkout on disk:

    python tests/golden/make_golden_truncation.py /path/to/dmrgpy

Each case stores the matrix, the cutoff/maxdim, the kept singular values
and the truncation error of the reference.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_golden import _install_numba_stub  # noqa: E402


def cases(rng):
    """(tag, matrix, cutoff, maxdim): square and rectangular shapes, a
    spectrum spanning the cutoff, a rank-deficient matrix and degenerate
    singular values (the multiplets of a spin-symmetric state)."""
    out = []

    def spectral(m, n, sv):
        r = len(sv)
        U, _ = np.linalg.qr(rng.standard_normal((m, r)))
        V, _ = np.linalg.qr(rng.standard_normal((n, r)))
        return (U * sv) @ V.T

    A = spectral(40, 60, np.exp(-0.6 * np.arange(40)))
    out += [("r40x60_a", A, 1e-12, None), ("r40x60_b", A, 1e-8, 30), ("r40x60_c", A, 0.0, 10)]
    B = spectral(96, 64, np.exp(-0.25 * np.arange(64)))
    out += [("r96x64_a", B, 1e-12, None), ("r96x64_b", B, 1e-10, 48)]
    C = spectral(128, 128, np.exp(-0.15 * np.arange(128)))
    out += [("r128_a", C, 1e-12, None), ("r128_b", C, 1e-9, 100), ("r128_c", C, 0.0, 64)]
    # rank 20 of 64: a lossless split keeps the zero directions
    D = spectral(64, 64, np.exp(-0.3 * np.arange(20)))
    out += [("rank20_a", D, 1e-12, None)]
    # degenerate multiplets (values repeated 3 and 5 times)
    sv = np.repeat(np.exp(-0.4 * np.arange(30)), [1, 3, 5] * 10)[:90]
    E = spectral(90, 120, sv)
    out += [("multiplet_a", E, 1e-12, None), ("multiplet_b", E, 0.0, 40)]
    F = spectral(256, 192, np.exp(-0.1 * np.arange(192)))
    out += [("r256x192_a", F, 1e-10, None), ("r256x192_b", F, 1e-12, 128)]
    return out


def main(ref):
    sys.path.insert(0, os.path.join(ref, "src"))
    _install_numba_stub()
    from dmrgpy.pyitensor.index import Index
    from dmrgpy.pyitensor.tensor import ITensor
    from dmrgpy.pyitensor.svd import svd

    rng = np.random.default_rng(2024)
    arrays = {}
    tags = []
    for tag, M, cut, md in cases(rng):
        m, n = M.shape
        i1, i2 = Index(m, "Link"), Index(n, "Link")
        U, S, V, spec = svd(ITensor((i1, i2), M), [i1], cutoff=cut, maxdim=md)
        arrays[tag + "_M"] = M
        arrays[tag + "_cut"] = np.array([cut, md if md else 0], dtype=float)
        arrays[tag + "_S"] = np.array(spec.singular_values).real
        arrays[tag + "_trunc"] = np.array([spec.truncerr])
        tags.append(tag)
        print(tag, M.shape, cut, md, "keep", len(spec.singular_values), "trunc", spec.truncerr)
    arrays["tags"] = np.array(tags)
    np.savez_compressed(os.path.join(HERE, "reference_truncation.npz"), **arrays)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
