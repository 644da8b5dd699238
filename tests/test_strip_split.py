"""CPU model of the strip engine's tile decoding (<pkg>/csrc/strips.cu: StripSplit::locate and
StripTiles::visit): a tile's global owned row gives its strip and local row by the
decomposition's arithmetic (the reference's make_strip, src/v4_mpi_cuda/decomposition.hpp:19-33:
strip k owns ny / S rows, the first ny % S strips one more), with the divisions done as the
device does them (multiply-high division by an invariant divisor, tests/cpp/fastdiv_test.cpp).
Checked against the cumulative layout of the strips for many lattice heights and strip counts.
"""

import pytest


def fastdiv(d):
    """The (m, s1, s2) of <pkg>/csrc/fastdiv.h for divisor d."""
    l = 0
    while l < 32 and (1 << l) < d:
        l += 1
    m = ((1 << 32) * ((1 << l) - d)) // d + 1
    return m & 0xFFFFFFFF, min(l, 1), max(l - 1, 0)


def fdiv(n, fd):
    m, s1, s2 = fd
    t = (m * n) >> 32
    return (t + ((n - t) >> s1)) >> s2


def locate(row, base, extra):
    split = extra * (base + 1)
    if row < split:
        k = fdiv(row, fastdiv(base + 1))
        return k, row - k * (base + 1)
    q = fdiv(row - split, fastdiv(base))
    return extra + q, row - split - q * base


@pytest.mark.parametrize("ny", [4, 5, 17, 64, 127, 128, 1000, 4096, 8191])
def test_locate_matches_layout(ny):
    for strips in range(1, min(ny // 2, 40) + 1):
        base, extra = divmod(ny, strips)
        n = [base + (1 if k < extra else 0) for k in range(strips)]
        y0 = [k * base + min(k, extra) for k in range(strips)]
        for k in range(strips):
            assert n[k] >= 2
            for r in range(n[k]):
                assert locate(y0[k] + r, base, extra) == (k, r)


@pytest.mark.parametrize("tw", [512, 1024, 2048])
def test_tile_rows(tw):
    for nx in (3, 511, 512, 513, 2048, 4100):
        tpr = (nx + tw - 1) // tw
        fd = fastdiv(tpr)
        for tile in range(0, 40 * tpr):
            row = fdiv(tile, fd)
            assert (row, tile - row * tpr) == divmod(tile, tpr)
