"""CPU model of the batched ensemble's ring tiling (<pkg>/csrc/batch.cu: build_table's tile
rule, build_plan's copies of each tile and the strip descriptors BatchFlatPolicy::issue writes
for the consumers).

The index arithmetic is restated here line by line and checked for every tile shape the
library accepts (consumer warps x passes: 8x2, 4x2, 4x1, 2x2), every storage width (FP32,
FP16/BF16, FP64), every row width 1..160 and a spread up to 4100, and several row counts:

- every cell of an instance is updated by exactly one lane of one consumer warp of one tile;
- for every cell and direction, the stage element the consumer reads (or the wrap value it
  substitutes at x = 0 / x = nx - 1) holds the pull source of the reference's streaming step,
  plane i at (x - c_x, y - c_y) with periodic wrap;
- the mask words a consumer reads (cells x - 1 .. x + 1 of rows y - 1 .. y + 1) are staged;
- every bulk copy starts and ends on 16-byte boundaries, stays inside its source row (plane
  rows within the pitch, mask rows within the row's words) and inside its stage region.
"""

import pytest

Q = 9
CX = [0, 1, 0, -1, 0, 1, -1, -1, 1]
CY = [0, 0, 1, 0, -1, 1, 1, -1, -1]
WRAP_LO = [1, 5, 8]  # wrap blocks 0..2: column nx - 1, planes with c_x = +1
WRAP_HI = [3, 6, 7]  # wrap blocks 3..5: column 0, planes with c_x = -1
MASK_PAD_WORDS = 80


def mask_row_words(nx):
    return ((nx + 31) // 32 + MASK_PAD_WORDS + 3) // 4 * 4


class Shape:
    """RingShape / FlatShape constants (step_ring.cuh, batch.cu)."""

    def __init__(self, elem, kw, kc):
        self.elem, self.kw, self.kc = elem, kw, kc
        self.H = 16 // elem
        self.LC = 2 if elem == 2 else 1
        self.SW = 32 * kc * self.LC
        self.WPS = self.SW // 32
        self.TW = kw * self.SW
        self.SROW = self.TW + 2 * self.H * kw
        self.MW = self.TW // 32 + 4
        self.mask_rows = kw * 3


def instance_tiles(sh, nx, ny):
    """build_table: strips per row, rows per tile (0: strip tiles) and the tile count."""
    spr = (nx + sh.SW - 1) // sh.SW
    rpt = sh.kw // spr if spr <= sh.kw else 0
    tiles = (ny + rpt - 1) // rpt if rpt else (spr * ny + sh.kw - 1) // sh.kw
    return spr, rpt, tiles


def check_instance(sh, nx, ny):
    pitch = (nx + 128 // sh.elem - 1) // (128 // sh.elem) * (128 // sh.elem)
    mw_row = mask_row_words(nx)
    spr, rpt, tiles = instance_tiles(sh, nx, ny)
    covered = [[0] * nx for _ in range(ny)]

    def src_row(i, y):
        return (y - CY[i]) % ny

    for t in range(tiles):
        stage = {}  # (plane, element) -> (row, x) of the source
        wrap = {}   # (segment, block, element) -> (row, x)
        masks = {}  # (stage mask row) -> (row, first word)

        def put(i, dst, row, xs, n):
            assert (xs * sh.elem) % 16 == 0 and (n * sh.elem) % 16 == 0, "16-byte aligned copy"
            assert 0 <= xs and xs + n <= pitch, "copy inside the source row"
            assert 0 <= dst and dst + n <= sh.SROW, "copy inside the plane's stage row"
            assert (dst * sh.elem) % 16 == 0
            for e in range(n):
                stage[(i, dst + e)] = (row, xs + e)

        descs = []
        if rpt:
            ya = t * rpt
            rn = min(rpt, ny - ya)
            for c in range(2 * Q):  # row_copy: plane i = c / 2, run c % 2
                i = c >> 1
                r0 = (ya - CY[i]) % ny
                len0 = min(rn, ny - r0)
                rs, ln = (0, rn - len0) if c & 1 else (r0, len0)
                if ln <= 0:
                    continue
                base = (len0 if c & 1 else 0) * pitch
                assert base + ln * pitch <= sh.SROW
                for r in range(ln):
                    put(i, base + r * pitch, rs + r, 0, pitch)
            for k in range(rn + 2):
                assert k < sh.mask_rows
                masks[k] = ((ya - 1 + k) % ny, 0)
                assert sh.MW <= mw_row
            for w in range(sh.kw):
                r, j = divmod(w, spr)
                if r >= rn:
                    continue
                x0 = j * sh.SW
                descs.append(dict(y=ya + r, x0=x0, lx0=r * pitch + x0, w0=x0 >> 5, sm_off=r, rows=True,
                                  seg=None))
        else:
            strips = spr * ny
            s0 = t * sh.kw
            s1 = min(s0 + sh.kw, strips)
            ya = s0 // spr
            nseg = (s1 - 1) // spr - ya + 1
            assert nseg <= sh.kw
            segs = []
            for g in range(nseg):
                y = ya + g
                row_s = y * spr
                j_lo = max(s0 - row_s, 0)
                j_hi = min(s1 - 1, row_s + spr - 1) - row_s
                w_first = row_s + j_lo - s0
                segs.append((y, j_lo, j_hi, w_first))
                x0 = j_lo * sh.SW
                xs = max(x0 - sh.H, 0)
                xe = min((j_hi + 1) * sh.SW + sh.H, pitch)
                for i in range(Q):
                    dst = w_first * sh.SW + 2 * g * sh.H + (xs - (x0 - sh.H))
                    put(i, dst, src_row(i, y), xs, xe - xs)
                wbase = ((x0 >> 5) & ~3)
                assert wbase + sh.MW <= mw_row, "mask copy inside the row's words"
                for r in range(3):
                    masks[g * 3 + r] = ((y - 1 + r) % ny, wbase)
                if j_lo == 0:
                    xb = (nx - 1) & ~(sh.H - 1)
                    for b, i in enumerate(WRAP_LO):
                        for e in range(sh.H):
                            wrap[(g, b, e)] = (src_row(i, y), xb + e)
                if j_hi == spr - 1:
                    for b, i in enumerate(WRAP_HI):
                        for e in range(sh.H):
                            wrap[(g, 3 + b, e)] = (src_row(i, y), e)
            for w in range(sh.kw):
                st = s0 + w
                if st >= s1:
                    continue
                y = st // spr
                j = st - y * spr
                g = y - ya
                j_lo = s0 - ya * spr if g == 0 else 0
                x0 = j * sh.SW
                descs.append(dict(y=y, x0=x0, lx0=w * sh.SW + (2 * g + 1) * sh.H,
                                  w0=(x0 >> 5) - (((j_lo * sh.SW) >> 5) & ~3), sm_off=g * 3, rows=False,
                                  seg=g))
        for d in descs:
            y = d["y"]
            for c in range(sh.kc):
                for lane in range(32):
                    for k in range(sh.LC):
                        x = d["x0"] + 32 * sh.LC * c + sh.LC * lane + k
                        if x >= nx:
                            continue
                        covered[y][x] += 1
                        lx = d["lx0"] + (x - d["x0"])
                        if sh.LC == 2:
                            assert (lx - k) % 2 == 0, "pairs read whole 32-bit words"
                        for i in range(Q):
                            want = (src_row(i, y), (x - CX[i]) % nx)
                            if d["rows"]:
                                r0 = lx - x
                                if x == 0 and CX[i] == 1:
                                    got = stage.get((i, r0 + nx - 1))
                                elif x == nx - 1 and CX[i] == -1:
                                    got = stage.get((i, r0))
                                else:
                                    got = stage.get((i, lx - CX[i]))
                            else:
                                if x == 0 and CX[i] == 1:
                                    got = wrap.get((d["seg"], WRAP_LO.index(i), (nx - 1) & (sh.H - 1)))
                                elif x == nx - 1 and CX[i] == -1:
                                    got = wrap.get((d["seg"], 3 + WRAP_HI.index(i), 0))
                                else:
                                    got = stage.get((i, lx - CX[i]))
                            assert got == want, (nx, ny, t, x, y, i, got, want)
                        # Mask bits of cells x - 1 .. x + 1 (bit x + 1 of a row is cell x): the
                        # absolute words (x >> 5) and (x >> 5) + 1 of rows y - 1, y, y + 1.
                        for r in range(3):
                            row, wbase = masks[d["sm_off"] + r]
                            assert row == (y - 1 + r) % ny
                            word = d["w0"] + (x - d["x0"]) // 32
                            assert wbase + word == x >> 5 and word + 1 < sh.MW
    assert all(v == 1 for row in covered for v in row), "every cell updated exactly once"


SHAPES = [(8, 2), (4, 2), (4, 1), (2, 2)]
WIDTHS = list(range(1, 161)) + [191, 255, 256, 257, 383, 511, 512, 513, 640, 767, 1000, 1023, 1024,
                                1025, 1500, 2047, 2049, 4100]


@pytest.mark.parametrize("elem", [4, 2, 8])
@pytest.mark.parametrize("kw,kc", SHAPES)
def test_batch_tiling_covers_and_stages_correctly(elem, kw, kc):
    sh = Shape(elem, kw, kc)
    for nx in WIDTHS:
        for ny in ((1, 2, 3, 7) if nx <= 160 else (3,)):
            check_instance(sh, nx, ny)


def test_whole_row_rule():
    # Rows that fit in a tile (at most kW strips) get whole-row tiles of kW / strips rows;
    # wider rows get strip tiles.
    sh = Shape(2, 8, 2)
    assert instance_tiles(sh, 1024, 10) == (8, 1, 10)
    assert instance_tiles(sh, 128, 10) == (1, 8, 2)
    assert instance_tiles(sh, 1025, 10)[1] == 0
