"""The index arithmetic of the tensor-core MPO step (mpo_step_mma_kernel in
csrc/tf32x3.cu), emulated in NumPy lane by lane: the input-offset and
output-offset tables, the m16n8k8 fragment ownership (A a0..a3, B b0/b1,
C c0..c3 with g = lane / 4, t = lane % 4), the guarded loads, the 3 x 4
tiles of a warp and the paired or single stores.  Exact arithmetic (no TF32
rounding), so the emulated step must equal the direct contraction
  X3[(a, s', t')][n chir + b] = sum_{s,t,k} W2[(s',t',n)][(s,t,k)] X1T[(a,k)][(s,t,b)]
exactly, and every offset it loads from or stores to must lie inside its
buffer, at the shapes the sweeps use (S=1/2 and S=1 bonds, chir not a
multiple of 32 and odd)."""
import numpy as np
import pytest

MMA_K = 48
RT_A = 8


def _kernel(X1T, W2, chil, d1, d2, chir, wl, wr, Kp, pair_stores, out_len):
    nst = d1 * d2
    in_cols, out_rows = nst * wl, nst * wr
    ldt = nst * chir
    # shared tables
    sOff = [(c % wl) * ldt + (c // wl) * chir if c < in_cols else -1 for c in range(MMA_K)]
    sOut = [(c // wr) * Kp + (c % wr) * chir if c < out_rows else -1 for c in range(MMA_K)]
    Wp = np.zeros((MMA_K, MMA_K))
    Wp[:out_rows, :in_cols] = W2.reshape(out_rows, in_cols)
    out = np.full(out_len, np.nan)
    touched = np.zeros(out_len, dtype=bool)
    grid_x, grid_y = (chir + 31) // 32, (chil + RT_A - 1) // RT_A
    for by in range(grid_y):
        for wi in range(RT_A):
            a = by * RT_A + wi
            if a >= chil:
                continue
            for bx in range(grid_x):
                b0 = bx * 32
                base = a * wl * ldt + b0
                acc = np.zeros((3, 4, 32, 4))
                for kt in range(MMA_K // 8):
                    # B fragments of all lanes, then the 8 x 8 tiles they form
                    Bt = np.zeros((4, 8, 8))
                    for lane in range(32):
                        g, t = lane >> 2, lane & 3
                        off0, off1 = sOff[8 * kt + t], sOff[8 * kt + t + 4]
                        for nt in range(4):
                            col = 8 * nt + g
                            ok = b0 + col < chir
                            for off, row in ((off0, t), (off1, t + 4)):
                                v = 0.0
                                if ok and off >= 0:
                                    idx = base + off + col
                                    assert 0 <= idx < X1T.size
                                    v = X1T.flat[idx]
                                Bt[nt, row, g] = v          # b0 = (t, g), b1 = (t + 4, g)
                    for mt in range(3):
                        At = np.zeros((16, 8))
                        for lane in range(32):
                            g, t = lane >> 2, lane & 3
                            r0, c0 = 16 * mt + g, 8 * kt + t
                            At[g, t] = Wp[r0, c0]               # a0
                            At[g + 8, t] = Wp[r0 + 8, c0]       # a1
                            At[g, t + 4] = Wp[r0, c0 + 4]       # a2
                            At[g + 8, t + 4] = Wp[r0 + 8, c0 + 4]   # a3
                        for nt in range(4):
                            D = At @ Bt[nt]
                            for lane in range(32):
                                g, t = lane >> 2, lane & 3
                                acc[mt, nt, lane] += (D[g, 2 * t], D[g, 2 * t + 1], D[g + 8, 2 * t], D[g + 8, 2 * t + 1])
                arow = a * nst * Kp
                for lane in range(32):
                    g, t = lane >> 2, lane & 3
                    for mt in range(3):
                        for half in range(2):
                            ro = sOut[16 * mt + g + 8 * half]
                            if ro < 0:
                                continue
                            for nt in range(4):
                                b = b0 + 8 * nt + 2 * t
                                if b >= chir:
                                    continue
                                o = arow + ro + b
                                v0, v1 = acc[mt, nt, lane, 2 * half], acc[mt, nt, lane, 2 * half + 1]
                                if pair_stores and b + 1 < chir:
                                    assert o % 2 == 0 and 0 <= o and o + 1 < out_len
                                    out[o], out[o + 1] = v0, v1
                                    touched[o:o + 2] = True
                                else:
                                    assert 0 <= o < out_len
                                    out[o] = v0
                                    touched[o] = True
                                    if b + 1 < chir:
                                        assert o + 1 < out_len
                                        out[o + 1] = v1
                                        touched[o + 1] = True
    return out, touched


@pytest.mark.parametrize("chil,chir,d,w", [(9, 40, 2, 5), (8, 45, 3, 5), (3, 64, 3, 5), (5, 33, 2, 4)])
def test_mpo_step_mma_index_arithmetic(chil, chir, d, w):
    rng = np.random.default_rng(chil * 100 + chir)
    wl = wr = w
    nst = d * d
    Kp = (wr * chir + 31) // 32 * 32
    X1T = rng.standard_normal((chil * wl, nst * chir))
    W2 = rng.standard_normal((nst * wr, nst * wl))
    # the launch's pairing rule: even chir and Kp (8-byte aligned bases)
    pair = int((chir | Kp) % 2 == 0)
    out_len = chil * nst * Kp
    out, touched = _kernel(X1T, W2, chil, d, d, chir, wl, wr, Kp, pair, out_len)
    # direct contraction in the same output layout
    X1 = X1T.reshape(chil, wl, nst, chir)                      # [a][k][st][b]
    W = W2.reshape(nst, wr, nst, wl)                           # [s't'][n][st][k]
    ref = np.einsum("pnsk,aksb->apnb", W, X1)                  # [a][s't'][n][b]
    expect = np.full((chil, nst, Kp), np.nan)
    expect[:, :, :wr * chir] = ref.reshape(chil, nst, wr * chir)
    expect = expect.reshape(-1)
    # every output element written exactly where the layout puts it, padding untouched
    assert np.array_equal(touched, ~np.isnan(expect))
    assert np.allclose(out[touched], expect[touched], rtol=1e-12, atol=1e-12)
