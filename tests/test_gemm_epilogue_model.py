"""The warp-to-accumulator mapping of the tcgen05 GEMM epilogue
(tf32x3_gemm_kernel in csrc/tf32x3.cu), emulated: eight epilogue warps
(warps 2..9 of the CTA) drain each K-slice TMEM buffer, a warp reaching only
the TMEM lane quarter warp % 4 (rows 32 q .. 32 q + 31, one row per lane) and
taking half of the tile's columns (warps 2..5 the first BNT / 2, warps 6..9
the rest).  With the merged MMA (A_hi.[B_hi; B_lo] as one N = 2 BNT MMA) a
buffer holds A_hi.B_hi + A_lo.B_hi in columns [0, BNT) and A_hi.B_lo in
[BNT, 2 BNT), and a warp adds both halves of its columns.  Checks that every
(row, output column) of a tile is accumulated by exactly one thread, from
exactly the TMEM columns that hold its products, for both tile widths and
both buffer layouts, and that each warp's lane quarter is the one its warp
index allows."""
import itertools

import pytest


@pytest.mark.parametrize("bnt,merge", [(128, True), (128, False), (64, True)])
def test_epilogue_warps_cover_each_output_once(bnt, merge):
    acc_cols = 2 * bnt if merge else bnt
    hb = bnt // 2
    owners = {}
    sources = {}
    for warp, lane in itertools.product(range(2, 10), range(32)):
        q = warp & 3                     # TMEM lane quarter this warp may access
        half = (warp - 2) >> 2
        row = q * 32 + lane
        assert 32 * q <= row < 32 * q + 32
        n0 = half * hb                   # first output column of this warp
        for grp in range(acc_cols // bnt):
            for j in range(hb):
                tcol = grp * bnt + half * hb + j      # TMEM column read
                assert 0 <= tcol < acc_cols
                key = (row, n0 + j)
                sources.setdefault(key, set()).add(tcol)
                owners.setdefault(key, set()).add((warp, lane))
    assert len(owners) == 128 * bnt
    for (row, col), who in owners.items():
        assert len(who) == 1
        # the products of output column col: column col, and col + BNT when merged
        assert sources[(row, col)] == ({col, col + bnt} if merge else {col})
