"""Scalar and 2x2 block matrices on patterns that stress edge paths, against
the oracle, and empty systems.

The arrow pattern (block row 0 coupled to every row) gives row 0 a triangle of
n-1 blocks in the backward sweep, far past the 32 blocks a warp holds in
registers (the streamed tail of the sync-free sweep), and a product row that
eight lanes walk n/8 times. The chain pattern (tridiagonal) has one row per
level. Tolerances: 1e-12 relative in FP64 (summation order only)."""
import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu


def _system(kind, n, nd, seed=3):
    rng = np.random.default_rng(seed)
    if kind == "arrow":
        nbr = [list(range(1, n))] + [[0] for _ in range(1, n)]
    else:
        nbr = [[j for j in (i - 1, i + 1) if 0 <= j < n] for i in range(n)]
    ind = np.zeros(n + 1, np.uint32)
    ind[1:] = np.cumsum([len(a) for a in nbr])
    psup = np.array([j for a in nbr for j in a], np.uint32)
    bb = nd * nd
    vc = 0.1 * rng.standard_normal(psup.size * bb) / (np.sqrt(n) if kind == "arrow" else 1.0)
    vd = np.tile(np.eye(nd).ravel(), n) * 4.0 + 0.1 * rng.standard_normal(n * bb)
    return ind, psup, vc, vd


@pytest.mark.parametrize("kind,n", [("arrow", 5000), ("chain", 2000)])
@pytest.mark.parametrize("nd", [1, 2])
@pytest.mark.parametrize("mode", [0, 1, 5, 7])
def test_edge_patterns(gpu, port, kind, n, nd, mode):
    import delfem2_gb300 as D
    ind, psup, vc, vd = _system(kind, n, nd)
    K = D.CMatrixSparse()
    K.Initialize(n, nd, True)
    K.SetPattern(ind, psup)
    K.set_values(vc, vd)
    ilu = D.CPreconditionerILU()
    ilu.SetPattern0(K)
    ilu.CopyValue(K)
    assert ilu.Decompose()
    ilu.set_sweep_mode(mode)
    rs, col, dia = port.ilu_pattern_k(ind, psup, 0)
    ivc, ivd = port.nd_ilu_copy_value(nd, ind, psup, vc, vd, 0, rs, col)
    st, ivc, ivd = port.nd_ilu_decompose(nd, rs, col, dia, ivc, ivd)
    assert st == 0
    gvc, gvd = ilu.values()
    assert np.array_equal(gvc, ivc) and np.array_equal(gvd, ivd)  # the reference's rounding, bit for bit
    v = np.random.default_rng(5).standard_normal(n * nd)
    f = v.copy()
    ilu.ForwardSubstitution(f)
    assert rel_err(f, port.nd_ilu_forward(nd, rs, col, dia, ivc, ivd, v)) < 1e-12
    g = v.copy()
    ilu.BackwardSubstitution(g)
    assert rel_err(g, port.nd_ilu_backward(nd, rs, col, dia, ivc, v)) < 1e-12
    y = np.random.default_rng(6).standard_normal(n * nd)
    ym = y.copy()
    K.MatVec(ym, 0.75, v, -1.25)
    assert rel_err(ym, port.nd_matvec(nd, ind, psup, vc, vd, y, 0.75, v, -1.25)) < 1e-12
    r, x = v.copy(), np.zeros_like(v)
    hist = D.Solve_PCG(r, x, 1e-10, 1000, K, ilu)
    xo, _, ho = port.nd_solve_pcg(nd, ind, psup, vc, vd, rs, col, dia, ivc, ivd, v, 1e-10, 1000)
    assert abs(len(hist) - len(ho)) <= 1 and rel_err(x, xo) < 1e-8


@pytest.mark.parametrize("nd", [1, 2, 3])
def test_empty_system(gpu, nd):
    """No block rows: every call succeeds; the solvers return the early-return
    histories of |r0| = 0 ([0] for PCG and BiCGStab, [] for CG)."""
    import delfem2_gb300 as D
    K = D.CMatrixSparse()
    K.Initialize(0, nd, True)
    K.SetPattern(np.zeros(1, np.uint32), np.zeros(0, np.uint32))
    K.setZero()
    K.SetFixedBC(np.zeros(0, np.int32))
    ilu = D.CPreconditionerILU()
    ilu.SetPattern0(K)
    ilu.CopyValue(K)
    assert ilu.Decompose()
    e = np.zeros(0)
    y = np.zeros(0)
    K.MatVec(y, 1.0, e, 0.0)
    ilu.SolvePrecond(np.zeros(0))
    assert D.Solve_PCG(np.zeros(0), np.zeros(0), 1e-10, 100, K, ilu) == [0.0]
    assert D.Solve_PBiCGStab(np.zeros(0), np.zeros(0), 1e-10, 100, K, ilu) == [0.0]
    assert D.Solve_CG(np.zeros(0), np.zeros(0), 1e-10, 100, K) == []
    st = D.Solve_PCG_Mixed(np.zeros(0), np.zeros(0), 1e-10, K, ilu)
    assert st.rel_residual == 0.0
