"""ILU(k) (Initialize_ILUk with fill level k > 0) in the CPU oracle, pinned
against the reference: patterns bit-exact (fixture tests/golden/iluk.npz
recorded from the reference, and directly where the reference is built),
factors to 1e-12 relative, Solve_PCG iterations equal and x to 1e-10."""
import numpy as np
import pytest

from conftest import golden, rel_err
from oracle import HAVE_REFERENCE_BUILD
from test_oracle import build_system

TAGS = [(1, "1"), (2, "2"), (3, "3"), (-1, "full")]


def _system(O):
    rng = np.random.default_rng(9)
    young = np.exp(rng.uniform(np.log(0.1), np.log(10.0), 8 ** 3 * 6))
    return build_system(O, 8, 8, 8, 1.0 / 8, young)


@pytest.mark.parametrize("k,tag", TAGS)
def test_pattern_factors_and_solve_match_golden(port, k, tag):
    G = golden("iluk")
    s = _system(port)
    rs, col, dia = port.ilu_pattern_k(s["ind"], s["psup"], k)
    assert np.array_equal(rs, G[f"k{tag}_rs"]) and np.array_equal(col, G[f"k{tag}_col"])
    assert np.array_equal(dia, G[f"k{tag}_dia"])
    ivc, ivd = port.ilu_copy_value_k(s["ind"], s["psup"], s["vc"], s["vd"], k, rs, col)
    assert port.ilu_decompose(rs, col, dia, ivc, ivd)[0] == 0
    assert rel_err(ivc[G[f"k{tag}_ivc_idx"]], G[f"k{tag}_ivc_sample"]) < 1e-12
    assert abs(np.abs(ivc).sum() - float(G[f"k{tag}_ivc_abs_sum"])) < 1e-12 * float(G[f"k{tag}_ivc_abs_sum"])
    assert abs(np.abs(ivd).sum() - float(G[f"k{tag}_ivd_abs_sum"])) < 1e-12 * float(G[f"k{tag}_ivd_abs_sum"])
    x, _, hist = port.solve_pcg_k(s["ind"], s["psup"], s["vc"], s["vd"], rs, col, dia, ivc, ivd, s["b"], 1e-10, 1000)
    assert len(hist) == len(G[f"k{tag}_hist"])
    assert rel_err(x, G[f"k{tag}_x"]) < 1e-10


def test_fill_grows_with_k_and_level0_is_pattern0(port):
    s = _system(port)
    rs0, col0, dia0 = port.ilu_pattern_k(s["ind"], s["psup"], 0)
    c, d = port.ilu_pattern0(s["ind"], s["psup"])
    assert np.array_equal(rs0, s["ind"]) and np.array_equal(col0, c) and np.array_equal(dia0, d)
    sizes = [port.ilu_pattern_k(s["ind"], s["psup"], k)[1].size for k in (0, 1, 2)]
    assert sizes[0] < sizes[1] < sizes[2]
    # each ILU(k) row is sorted, has no diagonal, and contains the matrix row
    rs, col, dia = port.ilu_pattern_k(s["ind"], s["psup"], 2)
    for i in range(0, rs.size - 1, 37):
        row = col[rs[i]:rs[i + 1]]
        assert np.all(np.diff(row.astype(np.int64)) > 0) and i not in row
        assert set(s["psup"][s["ind"][i]:s["ind"][i + 1]]) <= set(row)
        assert dia[i] == rs[i] + np.searchsorted(row, i)


@pytest.mark.skipif(not HAVE_REFERENCE_BUILD(), reason="reference source tree not available")
@pytest.mark.parametrize("k", [1, 2, 4, -1])
def test_port_equals_reference_directly(port, k):
    from oracle import cloth as CL
    from oracle import reference
    R = reference()
    # a tet block and a cloth sheet (quad-adjacency pattern)
    s = build_system(port, 4, 3, 5, 0.25, np.ones(4 * 3 * 5 * 6))
    x0, tri, quad = CL.cloth_square(port, 7)
    cind, cpsup = port.psup(quad, 4, x0.size // 3)
    for ind, psup in ((s["ind"], s["psup"]), (cind, cpsup)):
        a = port.ilu_pattern_k(ind, psup, k)
        b = R.ilu_pattern_k(ind, psup, k)
        for u, v in zip(a, b):
            assert np.array_equal(u, v)
    rs, col, dia = port.ilu_pattern_k(s["ind"], s["psup"], k)
    a = port.ilu_copy_value_k(s["ind"], s["psup"], s["vc"], s["vd"], k, rs, col)
    b = R.ilu_copy_value_k(s["ind"], s["psup"], s["vc"], s["vd"], k, rs, col)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
