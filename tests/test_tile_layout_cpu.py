"""The tile step's work-item layout, restated on the host: every node of the
grid is written by exactly one lane of one work item (none on the rows the
finite-difference closure writes), for the one-node layout and the aligned
pair layout, over grid shapes the GPU tests do not reach (nx not a multiple
of 64, nx = 4, thin y/z) and every face mix the API accepts.

The restatement follows csrc/rr_inst.inc (make_tile_args, pair_layout) and
csrc/rr_kernels.cuh (pair_item, pair_row's keep, tile_decode, tile_item's
end-pair dispatch, tile_node's FDBC skip) and the edge-node list of
rr_create (csrc/rr_api.cu).  It checks the decode scheme, not the device
code; the GPU tests run the device code on the configuration sizes.
"""
import itertools

import numpy as np
import pytest

PERIODIC, WALL, WALL_BB, FDBC = 0, 1, 2, 3


def _cdiv(a, b):
    return (a + b - 1) // b


def coverage(nx, ny, nz, face, rows_group, pairs):
    """writes per node by the tile step (and the FDBC rows left to fdbc_kernel)"""
    nrows = ny * nz
    wallmask = sum(1 << f for f in range(6) if face[f] != PERIODIC)
    fdbc = (1 if face[2] == FDBC else 0) | (2 if face[3] == FDBC else 0)
    xends = (not pairs) or (wallmask & 3) != 0
    segs = _cdiv(nx, 64) if pairs else _cdiv(nx - 2, 32)
    xf_half = rows_group // 32 if xends else 0
    group_items = rows_group * segs + 2 * xf_half
    nmain = _cdiv(nrows, rows_group) * group_items
    edges = []
    if xends:
        for z in range(nz):
            for y in range(ny):
                yzw = ((face[2] != PERIODIC and y == 0) or (face[3] != PERIODIC and y == ny - 1) or
                       (face[4] != PERIODIC and z == 0) or (face[5] != PERIODIC and z == nz - 1))
                if yzw:
                    row = z * ny + y
                    edges += [row * nx, row * nx + nx - 1]
    nitems = nmain + _cdiv(len(edges), 32)
    nedge_items = nitems - nmain
    rot = (nz - 1) * ny
    yzwall = [face[2] != PERIODIC, face[3] != PERIODIC, face[4] != PERIODIC, face[5] != PERIODIC]

    count = np.zeros(nx * ny * nz, dtype=np.int64)

    def interior(y, z):
        return 1 <= y <= ny - 2 and 1 <= z <= nz - 2

    def tile_node(row, x, y, fast):
        # the finite-difference closure's wall rows: fdbc_kernel writes them
        if not fast and fdbc and (((fdbc & 1) and y == 0) or ((fdbc & 2) and y == ny - 1)):
            return
        count[row * nx + x] += 1

    def rotate(row):
        row += rot
        return row - nrows if row >= nrows else row

    for item in range(nitems):
        for lane in range(32):
            if pairs and item >= nedge_items:
                # pair_item
                mitem = item - nedge_items
                grp, sub = divmod(mitem, group_items)
                if sub < rows_group * segs:
                    rl = sub // segs
                    row = grp * rows_group + rl
                    if row >= nrows:
                        continue
                    row = rotate(row)
                    z, y = divmod(row, ny)
                    x = (sub - rl * segs) * 64 + 2 * lane
                    if x >= nx:
                        continue
                    if interior(y, z):
                        # pair_row: keep 0 for the end pairs of an x-walled row
                        if not (xends and (x == 0 or x + 2 == nx)):
                            count[row * nx + x] += 1
                            count[row * nx + x + 1] += 1
                    else:
                        for k in (0, 1):
                            if not xends or (x + k != 0 and x + k != nx - 1):
                                tile_node(row, x + k, y, False)
                    continue
            # tile_decode
            if item >= nedge_items:
                mitem = item - nedge_items
                grp, sub = divmod(mitem, group_items)
                xface = False
                if sub < rows_group * segs:
                    assert not pairs
                    rl = sub // segs
                    row = grp * rows_group + rl
                    x = 1 + (sub - rl * segs) * 32 + lane
                    fast = True
                    if x > nx - 2:
                        continue
                else:
                    xi = sub - rows_group * segs
                    lo = xi < xf_half
                    row = grp * rows_group + (xi if lo else xi - xf_half) * 32 + lane
                    x = 0 if lo else nx - 1
                    fast = False
                    xface = True
                if row >= nrows:
                    continue
                row = rotate(row)
                z, y = divmod(row, ny)
                yzw = ((yzwall[0] and y == 0) or (yzwall[1] and y == ny - 1) or
                       (yzwall[2] and z == 0) or (yzwall[3] and z == nz - 1))
                if xface and yzw:
                    continue
                fast = fast and interior(y, z)
            else:
                e = item * 32 + lane
                if e >= len(edges):
                    continue
                row, x = divmod(edges[e], nx)
                z, y = divmod(row, ny)
                fast = False
            if pairs and interior(y, z):
                # tile_item: an x-face node of a row off every y/z face takes
                # its end pair (xend_pair)
                x0 = 0 if x == 0 else nx - 2
                count[row * nx + x0] += 1
                count[row * nx + x0 + 1] += 1
                continue
            tile_node(row, x, y, fast)

    fdbc_rows = np.zeros((nz, ny, nx), dtype=bool)
    if fdbc & 1:
        fdbc_rows[:, 0, :] = True
    if fdbc & 2:
        fdbc_rows[:, ny - 1, :] = True
    return count, fdbc_rows.reshape(-1)


FACES = {
    "periodic": (PERIODIC,) * 6,
    "cavity": (WALL,) * 6,
    "channel": (PERIODIC, PERIODIC, WALL, WALL, PERIODIC, PERIODIC),
    "channel_bb": (PERIODIC, PERIODIC, WALL_BB, WALL_BB, PERIODIC, PERIODIC),
    "channel_fdbc": (PERIODIC, PERIODIC, FDBC, FDBC, PERIODIC, PERIODIC),
    "fdbc_one_side": (PERIODIC, PERIODIC, FDBC, WALL, PERIODIC, PERIODIC),
    "x_walls_only": (WALL, WALL, PERIODIC, PERIODIC, PERIODIC, PERIODIC),
    "laminar": (WALL, WALL, PERIODIC, PERIODIC, PERIODIC, PERIODIC),
    "duct": (PERIODIC, PERIODIC, WALL, WALL, WALL, WALL),
}


@pytest.mark.parametrize("faces", sorted(FACES))
@pytest.mark.parametrize("nx,ny,nz", [(4, 4, 4), (6, 5, 3), (30, 7, 4), (64, 4, 5), (66, 6, 4), (128, 3, 3),
                                      (130, 5, 6), (200, 4, 3), (60, 20, 2)])
def test_every_node_written_once(faces, nx, ny, nz):
    face = FACES[faces]
    if face[2] == FDBC and ny < 4:
        pytest.skip("the finite-difference closure needs ly >= 4")
    pairs_ok = nx % 2 == 0 and nx >= 4
    for rows_group, pairs in itertools.product((32, 64), (False, True)):
        if pairs and not pairs_ok:
            continue
        if not pairs and nx < 3:
            continue
        count, fdbc_rows = coverage(nx, ny, nz, face, rows_group, pairs)
        bad = np.flatnonzero(count != np.where(fdbc_rows, 0, 1))
        assert bad.size == 0, (faces, nx, ny, nz, rows_group, pairs, bad[:10], count[bad[:10]])


def test_pair_layout_has_no_x_items_when_x_is_periodic():
    """without x walls the pair layout's segments take every node: no x-face
    and no edge items (the uncoalesced one-row-per-lane items)"""
    nx, ny, nz = 128, 8, 8
    for face in (FACES["periodic"], FACES["channel"], FACES["duct"]):
        wallmask = sum(1 << f for f in range(6) if face[f] != PERIODIC)
        assert (wallmask & 3) == 0
        count, fdbc_rows = coverage(nx, ny, nz, face, 32, True)
        assert np.array_equal(count, np.where(fdbc_rows, 0, 1))
