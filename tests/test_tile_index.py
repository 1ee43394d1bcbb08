"""CPU check of the x-pair tile's shared-memory index arithmetic (split_tile_x2
in csrc/gbf_split_tile.cuh), restated here for the three shapes the kernels
instantiate: 64x8 (single grids, ensembles), 32x16 and 48x10 (ensembles).

Per plane, every thread builds its own pair (box row ty + 1) and the first
2 * THX + 2 * HY threads one halo pair each (the interior pairs of the halo
rows 0 and HY - 1, then the left and right column pair of every row). The
update of a thread's pair reads the pair and its x, y neighbours in the plane
buffers. Checked: every element the updates read is built in the same plane,
no element is built twice, every index lies inside the buffer, and every TMA
box starts on a 16-byte boundary."""
import pytest


def shape(TXC, TY, NTB=256):
    THX = TXC // 2
    NT = THX * TY
    BX, HY = TXC + 8, TY + 2
    NP = (BX * HY + 31) // 32 * 32
    PCOLS = (TXC + 4) // 2
    return THX, NT, BX, HY, NP, PCOLS, NTB


@pytest.mark.parametrize("TXC,TY", [(64, 8), (32, 16), (48, 10)])
def test_halo_builds_cover_every_read_once(TXC, TY):
    THX, NT, BX, HY, NP, PCOLS, NTB = shape(TXC, TY)
    assert NT <= NTB and BX * HY <= NP
    built = []
    reads = set()
    for t in range(NTB):
        in_tile = t < NT
        tx, ty = t % THX, t // THX
        hc = (ty + 1) * BX + 2 * tx + 4
        if in_tile:  # slot 0: the own pair
            built += [hc, hc + 1]
            # 64-bit loads of the left, own and right pairs (cell a uses x-1,
            # cell b x+2 of the outer ones) and of the pairs above and below
            reads |= {hc - 2, hc - 1, hc, hc + 1, hc + 2, hc + 3}
            reads |= {hc - BX, hc - BX + 1, hc + BX, hc + BX + 1}
        q = t + NT  # slot 1
        if in_tile and q < PCOLS * HY:
            if q < NT + 2 * THX:
                h = q - NT
                r, c2 = (0 if h < THX else HY - 1), 2 + h % THX
            else:
                h = q - NT - 2 * THX
                r, c2 = h >> 1, (PCOLS if h & 1 else 1)
            built += [r * BX + 2 * c2, r * BX + 2 * c2 + 1]
    assert len(built) == len(set(built)), "an element built twice"
    assert all(0 <= e < NP for e in built) and all(0 <= e < NP for e in reads)
    missing = reads - set(built)
    assert not missing, sorted(missing)[:8]
    # the 64-bit shared accesses are 8-byte aligned: pairs start at even elements
    assert all(e % 2 == 0 for e in built[::2])


@pytest.mark.parametrize("TXC,TY", [(64, 8), (32, 16), (48, 10)])
def test_tma_boxes_start_on_16_bytes(TXC, TY):
    """FP32 boxes: the halo box at x0 - 4, the interior-row box at x0, with
    tiles at x0 = TXC * t (the mixed shape's 48-wide tile at x0 = 32 (q - 1)
    for nx = 32 q + 16, covering the row's last 48 cells); inner extents
    multiples of 16 bytes."""
    _, _, BX, _, _, _, _ = shape(TXC, TY)
    for t in range(8):
        x0 = TXC * t
        assert ((x0 - 4) * 4) % 16 == 0 and (x0 * 4) % 16 == 0
    for q in range(2, 6):  # mixed: the 48-wide tile ends the row of nx = 32 q + 16
        nx = 32 * q + 16
        x0 = (nx // 32 - 1) * 32
        assert x0 + 48 == nx and ((x0 - 4) * 4) % 16 == 0
    assert (BX * 4) % 16 == 0 and (TXC * 4) % 16 == 0
