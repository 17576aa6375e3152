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


@pytest.mark.parametrize("mode", [0, 1, 3, 4, 5, 6])
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
