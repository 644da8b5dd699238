"""CPU restatement of the adjoint kernels' tile order (<pkg>/csrc/adjoint.cu: AdjTiles and
tile_pos).

The ring pipeline hands block k the grid-stride tiles k, k + G, k + 2G, ... (G blocks);
tile_pos maps the i-th of them to the i-th tile of the block's contiguous chunk
k q + min(k, r) .. (total = q G + r), mirrored on alternate steps. The kernels rely on this
being a bijection (every tile of every instance stepped once) whose per-block images are
contiguous (a block's tiles of one instance are consecutive, so its per-instance partial sums
are flushed once per launch).
"""

import pytest


def tile_pos(tile, total, grid, per_inst, per_row, tw, reverse):
    q, r = divmod(total, grid)
    i, k = divmod(tile, grid)
    lin = k * q + min(k, r) + i
    if reverse:
        lin = total - 1 - lin
    b, rem = divmod(lin, per_inst)
    y, t = divmod(rem, per_row)
    return lin, b, y, t * tw


@pytest.mark.parametrize("reverse", [0, 1])
@pytest.mark.parametrize("batch,ny,per_row", [(1, 1, 1), (1, 7, 3), (4, 5, 2), (32, 128, 1), (32, 128, 2),
                                              (3, 17, 5)])
def test_tile_order_is_a_bijection_with_contiguous_chunks(reverse, batch, ny, per_row):
    per_inst = ny * per_row
    total = batch * per_inst
    for grid in sorted({1, 2, 3, 7, 152, 304, 456, total, total + 5}):
        seen = set()
        for k in range(grid):
            lins = []
            for tile in range(k, total, grid):  # the pipeline's grid-stride sequence of block k
                lin, b, y, tx0 = tile_pos(tile, total, grid, per_inst, per_row, 256, reverse)
                assert 0 <= b < batch and 0 <= y < ny and 0 <= tx0 < per_row * 256
                assert (b * ny + y) * per_row + tx0 // 256 == lin
                lins.append(lin)
            step = -1 if reverse else 1
            assert all(b - a == step for a, b in zip(lins, lins[1:])), "a block's tiles are contiguous"
            seen.update(lins)
        assert seen == set(range(total)), "every tile exactly once"
