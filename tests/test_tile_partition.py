"""Tile partition of the tile-scheduled sweeps (dfm2g_tile_partition, host
only; csrc/tiles.cu), on ILU patterns and level orders from the oracle.

Checked for both sweep directions: every row lies in exactly one tile; every
dependency of a row lies in a lower-numbered tile, or in the row's own tile
at a lower local level, the rule the sweep's freedom from deadlock rests on;
a row's local level is 1 + the highest local level of its dependencies in
the same tile (0 if none); tiles hold at most max_rows rows and max_width
rows per local level; tiles are numbered in the level order of their seeds.
On the natural ordering of a voxel mesh (nodes numbered z fastest, every
dependency on a lower neighbour) the tiles are columns of the node grid
(7 x 7 z lines, one segment deep) where the grid allows, for the FP64 and
the FP32 tile sizes."""
import ctypes as C

import numpy as np
import pytest


def _partition(lib, port, ind, col, dia, backward, max_rows, max_width):
    n = ind.size - 1
    tile_of = np.zeros(max(n, 1), np.uint32)
    level = np.zeros(max(n, 1), np.uint32)
    nt, m = C.c_uint(0), C.c_uint(0)
    u32 = lambda a: np.ascontiguousarray(a, np.uint32)
    _, order, _ = port.ilu_levels(ind, col, dia, backward)
    ind, col, dia, order = u32(ind), u32(col), u32(dia), u32(order)
    st = lib.dfm2g_tile_partition(n, ind.ctypes.data, col.ctypes.data, dia.ctypes.data, order.ctypes.data,
                                  int(backward), max_rows, max_width, tile_of.ctypes.data, level.ctypes.data,
                                  C.byref(nt), C.byref(m))
    assert st == 0
    return tile_of[:n], level[:n], nt.value, m.value, order


def _check(ind, col, dia, order, tile_of, level, nt, m, backward, max_rows, max_width):
    n = ind.size - 1
    assert tile_of.max() + 1 == nt
    counts = np.bincount(tile_of, minlength=nt)
    assert counts.min() >= 1 and counts.max() <= max_rows
    widths = {}
    most = 0
    for i in range(n):
        deps = col[dia[i]:ind[i + 1]] if backward else col[ind[i]:dia[i]]
        most = max(most, len(deps))
        want = 0
        for j in deps:
            assert tile_of[j] <= tile_of[i], (i, j)
            if tile_of[j] == tile_of[i]:
                assert level[j] < level[i], (i, j)
                want = max(want, int(level[j]) + 1)
        assert level[i] == want, (i, level[i], want)
        key = (int(tile_of[i]), int(level[i]))
        widths[key] = widths.get(key, 0) + 1
    assert max(widths.values()) <= max_width
    assert most == m
    # tiles are numbered in the level order of their seeds (the first row of the level order not in an
    # earlier tile): along the wavefront
    rank = np.empty(n, np.int64)
    rank[order] = np.arange(n)
    first = [int(rank[tile_of == t].min()) for t in range(nt)]
    assert first == sorted(first)


@pytest.mark.parametrize("rows,depths,full", [(1617, (20, 21), 4), (3185, (41,), 2)])
@pytest.mark.parametrize("backward", [False, True])
def test_voxel_mesh_tiles_are_columns(built_lib, port, backward, rows, depths, full):
    """With the sweep kernel's sizes (FP64: 1617 rows, 49 segments of 33 rows;
    FP32: 3185 rows, 49 segments of 65) the strands are the grid's z lines (41
    nodes: two segments of 21 + 20 rows, or one whole line) and the tiles are
    full boxes of them: 7 x 7 columns where the grid holds them, wider flat
    boxes at its edges."""
    import delfem2_gb300 as D
    nx, ny, nz = 16, 9, 40  # nodes 17 x 10 x 41
    a = D.voxel_problem_arrays(nx, ny, nz, 1.0 / nx, young=1.0)
    ind, psup = a["psup_ind"], a["psup"]
    col, dia = port.ilu_pattern0(ind, psup)
    tile_of, level, nt, m, order = _partition(built_lib, port, ind, col, dia, backward, rows, 49)
    _check(ind, col, dia, order, tile_of, level, nt, m, backward, rows, 49)
    assert m == 7
    # node (x, y, z) is row (x * (ny + 1) + y) * (nz + 1) + z
    x, y, z = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), np.arange(nz + 1), indexing="ij")
    x, y, z = x.ravel(), y.ravel(), z.ravel()
    columns = 0
    for t in range(nt):
        r = tile_of == t
        ext = [int(v[r].max() - v[r].min() + 1) for v in (x, y, z)]
        assert int(r.sum()) == ext[0] * ext[1] * ext[2], (t, ext)  # a full box
        assert ext[2] in depths and ext[0] * ext[1] <= 49, (t, ext)  # whole segments, at most 49
        assert int(level[r].max()) + 1 == ext[0] + ext[1] + ext[2] - 2  # a plane of the box per step
        columns += ext[:2] == [7, 7]
    assert columns == full  # 2 x 1 full columns of z lines in the 17 x 10 grid, per segment along z
    first = tile_of == 0
    d = max(depths)
    corner = (x >= nx + 1 - 7, y >= ny + 1 - 7, z >= nz + 1 - d) if backward else (x < 7, y < 7, z < d)
    assert np.array_equal(first, corner[0] & corner[1] & corner[2])  # the seed's column


@pytest.mark.parametrize("seed", [0, 1])
def test_random_pattern(built_lib, port, seed):
    rng = np.random.default_rng(seed)
    n = 600
    links = set()
    for i in range(1, n):
        if rng.random() < 0.8:
            links.add((i - 1, i))
    for i in range(n):
        for j in rng.integers(0, n, 2):
            if int(j) != i:
                links.add((min(i, int(j)), max(i, int(j))))
    nbr = [[] for _ in range(n)]
    for i, j in sorted(links):
        nbr[i].append(j)
        nbr[j].append(i)
    ind = np.zeros(n + 1, np.uint32)
    ind[1:] = np.cumsum([len(v) for v in nbr])
    psup = np.array([j for v in nbr for j in sorted(v)], np.uint32)
    col, dia = port.ilu_pattern0(ind, psup)
    for backward in (False, True):
        for max_rows, max_width in ((64, 10), (512, 50)):
            tile_of, level, nt, m, order = _partition(built_lib, port, ind, col, dia, backward, max_rows, max_width)
            _check(ind, col, dia, order, tile_of, level, nt, m, backward, max_rows, max_width)


@pytest.mark.parametrize("k", [1, 2])
def test_fill_in_patterns(built_lib, port, k):
    import delfem2_gb300 as D
    a = D.voxel_problem_arrays(6, 5, 4, 1.0 / 6, young=1.0)
    rs, col, dia = port.ilu_pattern_k(a["psup_ind"], a["psup"], k)
    for backward in (False, True):
        tile_of, level, nt, m, order = _partition(built_lib, port, rs, col, dia, backward, 512, 50)
        _check(rs, col, dia, order, tile_of, level, nt, m, backward, 512, 50)
        assert m > 7


@pytest.mark.parametrize("rows", [1617, 3185])
def test_sweep_sizes_on_cloth_and_fill_in_patterns(built_lib, port, rows):
    """The sweep's tile sizes (49 segments of at most 33 or 65 rows) on the
    cloth sheet's quad pattern and on ILU(1) of a voxel block whose z lines
    (41 rows) are cut in two at 33 rows and kept whole at 65: the partition's
    invariants hold in both directions."""
    import delfem2_gb300 as D
    from delfem2_gb300.cloth import SetClothShape_Square
    _, _, _, quad = SetClothShape_Square(20, 1.0)
    ind, psup = port.psup(quad, 4, 21 * 21)
    col, dia = port.ilu_pattern0(ind, psup)
    a = D.voxel_problem_arrays(3, 3, 40, 1.0 / 3, young=1.0)
    rs1, col1, dia1 = port.ilu_pattern_k(a["psup_ind"], a["psup"], 1)
    for rs_, col_, dia_ in ((np.asarray(ind), col, dia), (rs1, col1, dia1)):
        for backward in (False, True):
            tile_of, level, nt, m, order = _partition(built_lib, port, rs_, col_, dia_, backward, rows, 49)
            _check(rs_, col_, dia_, order, tile_of, level, nt, m, backward, rows, 49)


def test_empty_pattern_and_arguments(built_lib):
    z = np.zeros(1, np.uint32)
    nt, m = C.c_uint(7), C.c_uint(7)
    assert built_lib.dfm2g_tile_partition(0, z.ctypes.data, z.ctypes.data, z.ctypes.data, z.ctypes.data, 0, 512,
                                          50, z.ctypes.data, z.ctypes.data, C.byref(nt), C.byref(m)) == 0
    assert nt.value == 0 and m.value == 0
    assert built_lib.dfm2g_tile_partition(0, z.ctypes.data, z.ctypes.data, z.ctypes.data, z.ctypes.data, 0, 0,
                                          50, z.ctypes.data, z.ctypes.data, C.byref(nt), C.byref(m)) != 0
