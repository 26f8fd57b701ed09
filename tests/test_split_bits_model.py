"""The bit-pattern conversions of the split-TF32 kernels, modelled in NumPy
step for step (integer shifts and masks on the FP64/FP32 bit patterns, FP32
products and sums where the device uses them):

  widen  (common.cuh)   FP32 -> FP64, exact;
  narrow (common.cuh)   FP64 -> FP32, round half away from zero at 24 bits,
                        equal to IEEE round-to-nearest except at exact ties;
  split2 (tf32x3.cu)    FP64 -> TF32 pair (hi, lo): hi is x rounded to 11
                        significant bits, lo the remainder rounded to 11 bits,
                        |x - hi - lo| <= 2^-21 |x|.

The device forms replace FP64 arithmetic and FP64 <-> FP32 conversions,
which GB300 issues at a small fraction of the FP32 rate; values outside the
FP32 normal range take the conversion route on the device and are left out
here."""
import numpy as np


def _tf32(x):
    """cvt.rna.tf32.f32: 10 explicit mantissa bits, ties away from zero."""
    b = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    b = (b + 0x1000) & 0xFFFFE000
    return b.astype(np.uint32).view(np.float32)


def _hi_lo(x):
    b = np.asarray(x, np.float64).view(np.uint64)
    return (b >> 32).astype(np.uint64), (b & 0xFFFFFFFF).astype(np.uint64)


def widen(f):
    u = np.asarray(f, np.float32).view(np.uint32).astype(np.uint64)
    ef = (u >> 23) & 0xFF
    hi = (u & 0x80000000) | ((ef + 896) << 20) | ((u & 0x7FFFFF) >> 3)
    lo = (u << 29) & 0xFFFFFFFF
    out = ((hi << 32) | lo).view(np.float64)
    special = (ef == 0) | (ef == 0xFF)
    return np.where(special, np.asarray(f, np.float32).astype(np.float64), out)


def narrow(x):
    xh, xl = _hi_lo(x)
    e = ((xh >> 20) & 0x7FF).astype(np.int64)
    frac = ((xh & 0xFFFFF) << 3) | (xl >> 29)
    bits = (xh & 0x80000000) | ((((e - 896) << 23).astype(np.uint64) + frac + ((xl >> 28) & 1)) & 0xFFFFFFFF)
    out = bits.astype(np.uint32).view(np.float32)
    fallback = (e < 897) | (e > 1150)
    return np.where(fallback, np.asarray(x, np.float64).astype(np.float32), out), fallback


def split2(x):
    xh, xl = _hi_lo(x)
    e = ((xh >> 20) & 0x7FF).astype(np.int64)
    sgn = xh & 0x80000000
    mh = xh & 0xFFFFF
    up = (mh >> 9) & 1
    hb = sgn | ((((e - 896) << 23).astype(np.uint64) + (((mh >> 10) + up) << 13)) & 0xFFFFFFFF)
    hi = hb.astype(np.uint32).view(np.float32)
    rh = (mh & 0x3FF).astype(np.int64) - (up << 10).astype(np.int64)
    # fmaf(rh, 2^32, xl): the product is exact, one rounding of the sum
    r = (rh.astype(np.float64) * 2.0 ** 32 + xl.astype(np.float32).astype(np.float64)).astype(np.float32)
    scale = (((e - 884) << 23).astype(np.uint32)).view(np.float32)
    v = (r * np.float32(2.0 ** -64)).astype(np.float32) * scale
    lo = _tf32(np.where(sgn != 0, -v, v))
    inside = (e >= 897) & (e <= 1138)
    return hi, lo, inside


def _samples(n=200000, seed=0):
    rng = np.random.default_rng(seed)
    x = rng.standard_normal(n) * 10.0 ** rng.uniform(-30, 30, n)
    # values next to rounding boundaries: exact TF32 / FP32 ties and carries
    t = rng.standard_normal(2000).astype(np.float32).astype(np.float64)
    ties = np.concatenate([t * (1 + 2.0 ** -11), t * (1 - 2.0 ** -11), t * (1 + 2.0 ** -24), t, -t])
    return np.concatenate([x, ties, [1.0, -1.0, 0.5, 3.0, 2.0 ** 114, -(2.0 ** -125)]])


def test_widen_is_exact():
    rng = np.random.default_rng(1)
    f = (rng.standard_normal(200000) * 10.0 ** rng.uniform(-37, 37, 200000)).astype(np.float32)
    f = np.concatenate([f, np.float32([0.0, -0.0, 1.0, -2.5, 3.4e38, 1.2e-38])])
    assert np.array_equal(widen(f), f.astype(np.float64))


def test_narrow_rounds_to_nearest():
    x = _samples()
    y, fallback = narrow(x)
    ref = x.astype(np.float32)
    inside = ~fallback
    rel = np.abs(y[inside].astype(np.float64) - x[inside]) / np.abs(x[inside])
    assert rel.max() <= 2.0 ** -24
    # away from exact ties it is IEEE round-to-nearest
    assert np.mean(y[inside] == ref[inside]) > 0.999


def test_split2_pairs_hold_22_bits():
    x = _samples()
    hi, lo, inside = split2(x)
    x, hi, lo = x[inside], hi[inside], lo[inside]
    assert np.array_equal(_tf32(hi), hi) and np.array_equal(_tf32(lo), lo)
    err = np.abs(hi.astype(np.float64) + lo.astype(np.float64) - x) / np.abs(x)
    assert err.max() <= 2.0 ** -21
    # hi is x rounded to 11 significant bits: within half an ulp of TF32
    assert np.all(np.abs(hi.astype(np.float64) - x) <= np.abs(x) * 2.0 ** -11)
    # and it agrees with the conversion route (FP64 -> FP32 -> TF32) except
    # where that route's double rounding lands on the other side of a tie
    conv = _tf32(x.astype(np.float32))
    assert np.mean(conv == hi) > 0.999
