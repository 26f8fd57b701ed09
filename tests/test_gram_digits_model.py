"""The digit decomposition behind the tensor-core Gram matrix (gram.cu),
modelled in NumPy: columns scaled by powers of two, cut into three 8-bit
integer digits and a TF32 hi/lo tail; per K-slice of 32 the three digit
orders are summed (their partial sums are integer multiples of 2^-14,
2^-22, 2^-30 below 2^24 units, so an FP32 accumulator adds them without
rounding) and the 13 tail pairs in FP32.  Checks that invariant and the
error bound 1e-12 relative to |x_a| |x_b| against an extended-precision
Gram; the GPU test (test_gpu_gram.py) checks the kernel against the FP64
Gram with the same bound."""
import numpy as np
import pytest

SLICE = 32
# tail pairs summed in FP32 (operand order: D0, D1, D2, Th, Tl)
TAIL = [(1, 2), (2, 1), (0, 3), (3, 0), (0, 4), (4, 0), (2, 2), (1, 3), (3, 1), (2, 3), (3, 2), (1, 4), (4, 1)]


def _tf32(x):
    """Round to TF32 (10 explicit mantissa bits), ties away from zero."""
    b = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    b = (b + 0x1000) & 0xFFFFE000
    return b.astype(np.uint32).view(np.float32)


def _digits(X):
    """As digits_kernel: y = X / sigma as the FP32 pair yh + yl; the digits
    are those of yh (every FP32 step exact), the tail is the digits'
    remainder plus yl, rounded once to FP32 and split into a TF32 pair."""
    mx = np.abs(X).max(axis=0)
    sigma = np.where(mx > 0, 2.0 ** np.ceil(np.log2(np.where(mx > 0, mx, 1.0))), 1.0)
    y = X / sigma
    yh = y.astype(np.float32)
    yl = (y - yh.astype(np.float64)).astype(np.float32)
    f = np.float32
    d0 = np.rint(yh * f(128))
    r1 = yh * f(128) - d0
    d1 = np.rint(r1 * f(256))
    r2 = r1 * f(256) - d1
    d2 = np.rint(r2 * f(256))
    rem = r2 * f(256) - d2
    # the FP32 steps were exact: yh 2^23 = d0 2^16 + d1 2^8 + d2 + rem
    assert np.array_equal(yh.astype(np.float64) * 2.0 ** 23,
                          d0.astype(np.float64) * 2.0 ** 16 + d1.astype(np.float64) * 2.0 ** 8 + d2 + rem)
    tt = (rem.astype(np.float64) * 2.0 ** -23 + yl.astype(np.float64)).astype(np.float32)
    th = _tf32(tt)
    tl = _tf32(tt - th)
    D = [d0.astype(np.float64) / 128, d1.astype(np.float64) * 2.0 ** -15, d2.astype(np.float64) * 2.0 ** -23,
         th.astype(np.float64), tl.astype(np.float64)]
    return sigma, D, (d0, d1, d2, tt.astype(np.float64))


def _gram_model(X):
    m, k = X.shape
    sigma, D, (d0, d1, d2, tt) = _digits(X)
    assert max(np.abs(d0).max(), np.abs(d1).max(), np.abs(d2).max()) <= 128
    assert np.abs(tt).max() <= 1.5 * 2.0 ** -24
    acc = [np.zeros((k, k), np.int64) for _ in range(3)]
    tail = np.zeros((k, k), np.float32)
    units = (2.0 ** 14, 2.0 ** 22, 2.0 ** 30)
    for s in range(0, m, SLICE):
        a = [x[s:s + SLICE] for x in D]
        exact = (a[0].T @ a[0],
                 a[0].T @ a[1] + a[1].T @ a[0],
                 a[1].T @ a[1] + a[0].T @ a[2] + a[2].T @ a[0])
        for j, (p, u) in enumerate(zip(exact, units)):
            q = p * u
            # integer-valued and below 2^24: exact in an FP32 accumulator
            assert np.array_equal(q, np.rint(q)) and np.abs(q).max() < 2.0 ** 24
            acc[j] += np.rint(q).astype(np.int64)
        part = np.zeros((k, k), np.float32)
        for i, j in TAIL:
            part = (part + a[i].T.astype(np.float32) @ a[j].astype(np.float32)).astype(np.float32)
        tail = (tail + part).astype(np.float32)
    # int32 running sums in the kernel: stay below 2^31 for m <= 32768
    assert max(np.abs(x).max() for x in acc) < 2 ** 31
    g = acc[0] * 2.0 ** -14 + acc[1] * 2.0 ** -22 + acc[2] * 2.0 ** -30 + tail.astype(np.float64)
    return g * np.outer(sigma, sigma)


def _scaled_err(G, X):
    ref = X.astype(np.longdouble).T @ X.astype(np.longdouble)
    d = np.sqrt(np.abs(np.diag(ref)).astype(np.float64))
    den = np.outer(d, d)
    den[den == 0] = 1.0
    return float(np.max(np.abs(G - ref.astype(np.float64)) / den))


@pytest.mark.parametrize("kind", ["orthonormal", "scaled", "constant", "ragged"])
def test_digit_gram_model_error_bound(kind):
    rng = np.random.default_rng(11)
    if kind == "orthonormal":
        X = np.linalg.qr(rng.standard_normal((1536, 128)))[0]
    elif kind == "scaled":
        X = rng.standard_normal((640, 48)) * np.exp(rng.uniform(-18.0, 18.0, 48))
    elif kind == "constant":
        # coherent digits and tails (every row the same): the worst case for
        # the FP32 tail accumulation
        X = np.ones((1024, 24)) * np.linspace(0.3, 0.9, 24) / 32.0
    else:
        X = rng.standard_normal((333, 7))
        X[:, 3] = 0.0
    G = _gram_model(X)
    assert _scaled_err(G, X) < 1e-12
    # the split-TF32 class of error, for contrast: ~1e-7
    assert _scaled_err((X.astype(np.float32).T @ X.astype(np.float32)).astype(np.float64), X) > 1e-9
