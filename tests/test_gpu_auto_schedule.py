"""Which schedule the automatic sweep choice (DFM2G_SWEEP_AUTO, the default)
runs, read back with dfm2g_ilu_last_schedule, against its rule: the tile
schedule where the tile partition averages at least 20 rows per step, rows
have at most 8 dependency blocks and, in FP64, the partition has at least
half as many tiles as the GPU has SMs; the chain schedule otherwise, and
always for 1x1 and 2x2 blocks.

The partition's rows per step and tile count come from dfm2g_tile_partition
with the sweep's sizes (49 rows per step; tiles of 3185 rows in FP32, 1617 in
FP64) on the oracle's level order. Cases: voxel blocks of 32^3 cells (tiles in
FP32; 26 tiles, so the chains in FP64) and 48^3 (tiles in both), the cloth
sheet's quad pattern (9-11 rows per step: chains), ILU(1) of a 48^3 voxel
block (13 dependency blocks per row: chains, although its FP32 tiles of whole
z lines reach 25-27 rows per step), a scalar chain pattern (chains). An explicit schedule is the
one that runs, and the cluster schedule on a vector larger than shared
memory falls back to the automatic choice."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TILES, CHAINS, AUTO, CLUSTER = 6, 5, 7, 8


def _rule(lib, port, ilu, fp64):
    """Schedule the rule picks for each direction (forward, backward)."""
    import torch
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    rs = np.ascontiguousarray(ilu.row_start(), np.uint32)
    col, dia = (np.ascontiguousarray(a, np.uint32) for a in ilu.pattern())
    n = rs.size - 1
    rows = 1617 if fp64 else 3185
    out = []
    for backward in (False, True):
        _, order, _ = port.ilu_levels(rs, col, dia, backward)
        order = np.ascontiguousarray(order, np.uint32)
        tile_of, level = np.zeros(n, np.uint32), np.zeros(n, np.uint32)
        nt, m = C.c_uint(0), C.c_uint(0)
        assert lib.dfm2g_tile_partition(n, rs.ctypes.data, col.ctypes.data, dia.ctypes.data, order.ctypes.data,
                                        int(backward), rows, 49, tile_of.ctypes.data, level.ctypes.data,
                                        C.byref(nt), C.byref(m)) == 0
        nsteps = sum(int(level[tile_of == t].max()) + 1 for t in range(nt.value))
        tiles = n / nsteps >= 20.0 and m.value <= 8 and (not fp64 or 2 * nt.value >= sms)
        out.append(TILES if tiles else CHAINS)
    return out


def _sweep_both(ilu, fp64, n3):
    v = np.random.default_rng(1).standard_normal(n3)
    if fp64:
        ilu.ForwardSubstitution(v)
        ilu.BackwardSubstitution(v)
    else:
        ilu.SolvePrecond(v.astype(np.float32))
    return [ilu.last_schedule(fp64, False), ilu.last_schedule(fp64, True)]


def _voxel_ilu(nc, k=0):
    import delfem2_gb300 as D
    P = D.StaticElasticProblem(D.voxel_problem_arrays(nc, nc, nc, 1.0 / nc, seed=4, e_range=(0.1, 10.0)))
    b = P.assemble()
    ilu = D.CPreconditionerILU()
    if k:
        ilu.Initialize_ILUk(P.K, k)
    else:
        ilu.SetPattern0(P.K)
    ilu.CopyValue(P.K)
    assert ilu.Decompose()
    return ilu, b.size


def _pattern_ilu(ind, psup, ndim):
    import delfem2_gb300 as D
    n = ind.size - 1
    rng = np.random.default_rng(2)
    K = D.CMatrixSparse()
    K.Initialize(n, ndim, True)
    K.SetPattern(ind, psup)
    K.set_values(0.05 * rng.standard_normal(psup.size * ndim * ndim),
                 np.tile(np.eye(ndim).ravel(), n) * 4.0 + 0.05 * rng.standard_normal(n * ndim * ndim))
    ilu = D.CPreconditionerILU()
    ilu.SetPattern0(K)
    ilu.CopyValue(K)
    assert ilu.Decompose()
    return ilu, n * ndim


@pytest.mark.parametrize("nc,want32,want64", [(32, TILES, CHAINS), (48, TILES, TILES)])
def test_auto_on_voxel_blocks(gpu, port, nc, want32, want64):
    ilu, n3 = _voxel_ilu(nc)
    assert ilu.sweep_mode() == AUTO
    assert [ilu.last_schedule(f, b) for f in (False, True) for b in (False, True)] == [-1] * 4
    for fp64, want in ((False, want32), (True, want64)):
        assert _rule(gpu, port, ilu, fp64) == [want, want]
        assert _sweep_both(ilu, fp64, n3) == [want, want], (nc, fp64)


def test_auto_takes_the_chains_on_cloth(gpu, port):
    from delfem2_gb300 import cloth as DC
    _, _, _, quad = DC.SetClothShape_Square(52, 1.0)
    ind, psup = port.psup(quad, 4, 53 * 53)
    ilu, n3 = _pattern_ilu(np.asarray(ind, np.uint32), np.asarray(psup, np.uint32), 3)
    for fp64 in (False, True):
        assert _rule(gpu, port, ilu, fp64) == [CHAINS, CHAINS]
        assert _sweep_both(ilu, fp64, n3) == [CHAINS, CHAINS]
    ilu.set_sweep_mode(TILES)  # explicit: the tiles run although the rule would not take them
    assert _sweep_both(ilu, False, n3) == [TILES, TILES]


def test_auto_takes_the_chains_on_iluk(gpu, port):
    ilu, n3 = _voxel_ilu(48, k=1)
    for fp64 in (False, True):
        assert _rule(gpu, port, ilu, fp64) == [CHAINS, CHAINS]
        assert _sweep_both(ilu, fp64, n3) == [CHAINS, CHAINS], fp64


def test_auto_on_scalar_blocks(gpu):
    n = 5000
    nbr = [[j for j in (i - 1, i + 1) if 0 <= j < n] for i in range(n)]
    ind = np.zeros(n + 1, np.uint32)
    ind[1:] = np.cumsum([len(a) for a in nbr])
    psup = np.array([j for a in nbr for j in a], np.uint32)
    ilu, n1 = _pattern_ilu(ind, psup, 1)
    for fp64 in (False, True):
        assert _sweep_both(ilu, fp64, n1) == [CHAINS, CHAINS]


def test_cluster_falls_back_to_the_automatic_choice(gpu, port):
    ilu, n3 = _voxel_ilu(48)  # 352,947 FP32 values: more than one CTA's shared memory
    ilu.set_sweep_mode(CLUSTER)
    assert _sweep_both(ilu, False, n3) == [TILES, TILES]


def test_last_schedule_rejects_bad_arguments(gpu):
    from delfem2_gb300 import _native as N
    ilu, _ = _voxel_ilu(4)
    m = C.c_int(0)
    assert gpu.dfm2g_ilu_last_schedule(ilu._h, 5, 0, C.byref(m)) != 0
    assert gpu.dfm2g_ilu_last_schedule(ilu._h, N.F32, 0, None) != 0
    assert gpu.dfm2g_ilu_last_schedule(None, N.F32, 0, C.byref(m)) != 0
