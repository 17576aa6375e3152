"""ILU(k) on the GPU (Initialize_ILUk, fill level k > 0) against the reference
fixture tests/golden/iluk.npz and the oracle.

Bars: patterns bit-exact; factor samples 1e-10 relative; sweeps 1e-10 (FP64)
in every schedule; Solve_PCG iterations equal (+-1) and x within 1e-8 of the
reference's; the mixed solver reaches 1e-10 with the ILU(k) factors."""
import numpy as np
import pytest

from conftest import golden, rel_err

pytestmark = pytest.mark.gpu

TAGS = [(1, "1"), (2, "2"), (3, "3"), (-1, "full")]


@pytest.fixture(scope="module")
def prob(gpu):
    import delfem2_gb300 as D
    a = D.voxel_problem_arrays(8, 8, 8, 1.0 / 8, seed=9, e_range=(0.1, 10.0))
    P = D.StaticElasticProblem(a)
    b = P.assemble()
    return a, P, b


@pytest.mark.parametrize("k,tag", TAGS)
def test_iluk_matches_reference_fixture(prob, k, tag):
    import delfem2_gb300 as D
    G = golden("iluk")
    a, P, b = prob
    ilu = D.CPreconditionerILU()
    ilu.Initialize_ILUk(P.K, k)
    col, dia = ilu.pattern()
    assert np.array_equal(ilu.row_start(), G[f"k{tag}_rs"])
    assert np.array_equal(col, G[f"k{tag}_col"]) and np.array_equal(dia, G[f"k{tag}_dia"])
    ilu.CopyValue(P.K)
    assert ilu.Decompose()
    vc, vd = ilu.values()
    assert rel_err(vc[G[f"k{tag}_ivc_idx"]], G[f"k{tag}_ivc_sample"]) < 1e-10
    assert abs(np.abs(vd).sum() - float(G[f"k{tag}_ivd_abs_sum"])) < 1e-10 * float(G[f"k{tag}_ivd_abs_sum"])
    r, x = b.copy(), np.zeros_like(b)
    hist = D.Solve_PCG(r, x, 1e-10, 1000, P.K, ilu)
    assert abs(len(hist) - len(G[f"k{tag}_hist"])) <= 1
    assert rel_err(x, G[f"k{tag}_x"]) < 1e-8
    xm = np.zeros_like(b)
    st = D.Solve_PCG_Mixed(b, xm, 1e-10, P.K, ilu, method="reliable")
    assert st.rel_residual < 1e-10 and rel_err(xm, G[f"k{tag}_x"]) < 1e-8


@pytest.mark.parametrize("mode", [0, 1, 3, 4, 5, 6, 7, 8])
def test_iluk_sweeps_match_oracle_in_every_schedule(prob, port, mode):
    import delfem2_gb300 as D
    a, P, b = prob
    ilu = D.CPreconditionerILU()
    ilu.Initialize_ILUk(P.K, 2)
    ilu.CopyValue(P.K)
    assert ilu.Decompose()
    ilu.set_sweep_mode(mode)
    rs = ilu.row_start()
    col, dia = ilu.pattern()
    vc, vd = ilu.values()
    v = np.random.default_rng(6).standard_normal(b.size)
    f = v.copy()
    ilu.ForwardSubstitution(f)
    fo = port.ilu_forward(rs, col, dia, vc, vd, v)
    assert rel_err(f, fo) < 1e-10
    g = fo.copy()
    ilu.BackwardSubstitution(g)
    assert rel_err(g, port.ilu_backward(rs, col, dia, vc, fo)) < 1e-10


def _outside_rows_per_step(lib, port, rs, col, dia, backward):
    """Most rows of other tiles that one step of the tile schedule depends on
    (dfm2g_tile_partition with the FP64 sweep's sizes; on a 28^3 block the
    FP32 tiles are the same, its 29-row z lines being one segment either way)."""
    import ctypes as C
    n = rs.size - 1
    _, order, _ = port.ilu_levels(rs, col, dia, backward)
    u32 = lambda x: np.ascontiguousarray(x, np.uint32)
    rs_, col_, dia_, order = u32(rs), u32(col), u32(dia), u32(order)
    tile_of, level = np.zeros(n, np.uint32), np.zeros(n, np.uint32)
    nt, m = C.c_uint(0), C.c_uint(0)
    assert lib.dfm2g_tile_partition(n, rs_.ctypes.data, col_.ctypes.data, dia_.ctypes.data, order.ctypes.data,
                                    int(backward), 1617, 49, tile_of.ctypes.data, level.ctypes.data, C.byref(nt),
                                    C.byref(m)) == 0
    lo, hi = (dia_, rs_[1:]) if backward else (rs_[:-1], dia_)
    rows = np.repeat(np.arange(n), (hi - lo).astype(np.int64))
    deps = np.concatenate([col_[a:b] for a, b in zip(lo, hi)])
    out = tile_of[deps] != tile_of[rows]
    step = tile_of[rows[out]].astype(np.int64) * (1 << 20) + level[rows[out]]
    pairs = np.unique(np.stack([step, deps[out].astype(np.int64)], 1), axis=0)
    return int(np.unique(pairs[:, 0], return_counts=True)[1].max()), int(m.value)


def test_iluk_tiles_with_rows_read_in_global_memory(gpu, port):
    """ILU(1) of a 28^3 voxel block, swept by the tile schedule (13 blocks per
    triangle row fit its records), where some backward steps depend on more
    than 128 rows of other tiles: the first 128 are copied ahead, the rest
    read in global memory. FP64 and FP32 sweeps match the oracle's sweeps of
    the same factors (1e-10, 1e-4), and the mixed solver reaches 1e-10."""
    import ctypes as C
    import torch
    import delfem2_gb300 as D
    from delfem2_gb300 import _native as N
    a = D.voxel_problem_arrays(28, 28, 28, 1.0 / 28, seed=4, e_range=(0.1, 10.0))
    P = D.StaticElasticProblem(a)
    b = P.assemble()
    ilu = D.CPreconditionerILU()
    ilu.Initialize_ILUk(P.K, 1)
    ilu.CopyValue(P.K)
    assert ilu.Decompose()
    ilu.set_sweep_mode(6)  # the default takes the chains backward here (19.6 rows per step)
    rs = ilu.row_start()
    col, dia = ilu.pattern()
    vc, vd = ilu.values()
    most, m = _outside_rows_per_step(gpu, port, rs, col, dia, True)
    assert m == 13 and most > 128, (m, most)
    v = np.random.default_rng(8).standard_normal(b.size)
    fo = port.ilu_forward(rs, col, dia, vc, vd, v)
    zo = port.ilu_backward(rs, col, dia, vc, fo)
    f = v.copy()
    ilu.ForwardSubstitution(f)
    assert rel_err(f, fo) < 1e-10
    g = fo.copy()
    ilu.BackwardSubstitution(g)
    assert rel_err(g, zo) < 1e-10
    z32 = torch.tensor(v, dtype=torch.float32, device="cuda")
    N.call("dfm2g_ilu_solve_precond", ilu._h, N.F32, C.c_void_p(z32.data_ptr()), N.MEM_DEVICE)
    assert rel_err(z32.double().cpu().numpy(), zo) < 1e-4
    xm = np.zeros_like(b)
    st = D.Solve_PCG_Mixed(b, xm, 1e-10, P.K, ilu, method="reliable")
    assert st.rel_residual < 1e-10


def test_iluk_on_the_cloth_pattern(gpu, port):
    """ILU(1) of the cloth sheet's quad-adjacency pattern: the same pattern as
    the oracle (bit-exact) and a converged step-sized solve."""
    import delfem2_gb300 as D
    from delfem2_gb300 import cloth as DC
    xyz0, _, tri, quad = DC.SetClothShape_Square(12, 1.0)
    c = DC.Cloth(xyz0, tri, quad)
    ind, psup = port.psup(quad, 4, c.np)
    ilu = D.CPreconditionerILU()
    ilu.Initialize_ILUk(c.mat, 1)
    rs, col, dia = port.ilu_pattern_k(ind, psup, 1)
    gc, gd = ilu.pattern()
    assert np.array_equal(ilu.row_start(), rs) and np.array_equal(gc, col) and np.array_equal(gd, dia)


def test_iluk_rejects_bad_handles(gpu):
    import delfem2_gb300 as D
    from delfem2_gb300 import _native as N
    K = D.CMatrixSparse()
    K.Initialize(4, 3, True)
    ilu = D.CPreconditionerILU()
    with pytest.raises(N.Dfm2gError):
        ilu.Initialize_ILUk(K, 1)  # the matrix has no pattern yet
