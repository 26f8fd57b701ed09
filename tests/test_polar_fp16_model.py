"""The FP16-split polar (Newton-Schulz) iteration of the subspace truncation
(subspace.cu), modelled in NumPy: operands held as FP16 hi/lo pairs of
power-of-two scaled values, products of the pairs (hi.hi + hi.lo + lo.hi,
exact in FP32) accumulated in FP32, 14 quintic steps X <- X B with
B = aI + A(bI + cA), then cubic steps to max|X^T X - I| < 5e-6; the iterate
is kept only as its FP16 pair, and the basis formed from it.  Checks
that the fixed scales keep every scaled operand inside the FP16 range
(|v| <= 65504) at every step, for inputs from an orthonormal start to a
spectrum spread below the ~5e-8 perturbation floor, that the iteration
converges within its step budget, and that the orthonormal basis keeps the
input's weight to ~1e-12: the FP32-class rounding of ~18 steps rotates the
basis by ~7e-7 along strong directions and ~2e-8 / s along one of relative
singular value s, which loses ~5e-13 of weight per strong direction and
~4e-16 per weak one -- far below the discarded weight of a truncation at
these bond dimensions."""
import numpy as np
import pytest

# the scales and coefficients of csrc/subspace.cu
SX, SA, SP, SB = 4096.0, 4096.0, 4096.0, 2048.0
A5, B5, C5 = 3.4445, -4.7750, 2.0315
FP16_MAX = 65504.0


def _pair(v, scale, peak):
    """FP16 hi/lo pair of v * scale; records the largest |v * scale|."""
    w = v * scale
    peak.append(float(np.max(np.abs(w))))
    hi = w.astype(np.float16)
    lo = (w - hi.astype(np.float64)).astype(np.float16)
    return hi.astype(np.float32), lo.astype(np.float32)


def _prod(a, b, scale):
    """a^T-free product of two pairs, A (rows x K) . B (K x cols), FP32 accumulation."""
    (ah, al), (bh, bl) = a, b
    return (ah @ bh + ah @ bl + al @ bh).astype(np.float64) / scale


def _polar(Z):
    m, k = Z.shape
    peak = []
    rng = np.random.default_rng(5)
    X = Z / np.linalg.norm(Z, axis=0) / np.sqrt(k)
    X = X + (1e-7 / np.sqrt(m)) * rng.uniform(-0.5, 0.5, X.shape)
    d = np.inf
    steps = 0
    for it in range(14 + 16):
        xs = _pair(X, SX, peak)
        A = _prod((xs[0].T, xs[1].T), xs, SX * SX)          # X^T X
        if it < 14:
            P = C5 * A + B5 * np.eye(k)                      # c A + b I
            Bm = _prod(_pair(A, SA, peak), _pair(P, SP, peak), SA * SP) + A5 * np.eye(k)
        else:
            d = np.max(np.abs(A - np.eye(k)))
            if d < 5e-6:
                break
            Bm = 1.5 * np.eye(k) - 0.5 * A
        X = _prod(xs, _pair(Bm, SB, peak), SX * SB)
        steps += 1
    # the iterate lives only as its FP16 pair; the basis is formed from it
    hi, lo = _pair(X, SX, peak)
    X = (hi.astype(np.float64) + lo.astype(np.float64)) / SX
    return X, d, max(peak), steps


@pytest.mark.parametrize("spread", [0.0, 1e-3, 1e-6, 1e-9])
def test_polar_fp16_scales_stay_in_range_and_converge(spread):
    rng = np.random.default_rng(3)
    m, k = 256, 48
    U = np.linalg.qr(rng.standard_normal((m, k)))[0]
    V = np.linalg.qr(rng.standard_normal((k, k)))[0]
    s = np.geomspace(1.0, spread, k) if spread > 0 else np.ones(k)
    Z = (U * s) @ V.T
    X, d, peak, steps = _polar(Z)
    assert peak < FP16_MAX / 2, peak        # a factor 2 of headroom
    assert d < 5e-6 and steps <= 14 + 16
    # weight of the input outside the basis (measured ~3e-12)
    lost = np.linalg.norm(Z - X @ (X.T @ Z)) ** 2 / np.linalg.norm(Z) ** 2
    assert lost < 1e-11, lost
