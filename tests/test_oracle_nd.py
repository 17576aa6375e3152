"""Scalar (ndim 1) and 2x2 (ndim 2) blocks in the CPU oracle, pinned against
the reference: the fixture tests/golden/nd.npz (written by the reference, see
tests/golden/make_golden.py) and directly where the reference is built.

The restatement follows the reference's loops and expression order, so every
comparison is exact: assembly (Poisson on tets and triangles, 2-D linear
solid), SetFixedBC, MatVec, the ILU(0) / ILU(1) factors and sweeps, and the
Solve_PCG / Solve_PBiCGStab histories and solutions. The Merge case repeats a
node inside one element, where the reference adds the (irow, irow) block."""
import numpy as np
import pytest

import nd_systems as S
from conftest import golden
from oracle import HAVE_REFERENCE_BUILD


@pytest.mark.parametrize("name", list(S.SYSTEMS))
def test_assembly_and_matvec_match_golden(port, name):
    G = golden("nd")
    s = S.SYSTEMS[name](port)
    for k in ("ind", "psup", "bc", "elem"):
        assert np.array_equal(s[k], G[f"{name}_{k}"])
    for k in ("vc", "vd", "b"):
        assert np.array_equal(s[k], G[f"{name}_{k}"]), k
    y = port.nd_matvec(s["ndim"], s["ind"], s["psup"], s["vc"], s["vd"], G[f"{name}_mv_y"], 1.5, G[f"{name}_mv_x"],
                       0.5)
    assert np.array_equal(y, G[f"{name}_mv"])


@pytest.mark.parametrize("name", list(S.SYSTEMS))
@pytest.mark.parametrize("k", [0, 1])
def test_factors_sweeps_and_solvers_match_golden(port, name, k):
    G = golden("nd")
    s = S.SYSTEMS[name](port)
    nd = s["ndim"]
    rs, col, dia, ivc, ivd = S.factor(port, s, k)
    t = f"{name}_k{k}"
    for a, key in ((rs, "rs"), (col, "col"), (dia, "dia"), (ivc, "vc"), (ivd, "vd")):
        assert np.array_equal(a, G[f"{t}_{key}"]), key
    x = G[f"{name}_mv_x"]
    assert np.array_equal(port.nd_ilu_forward(nd, rs, col, dia, ivc, ivd, x), G[f"{t}_fwd"])
    assert np.array_equal(port.nd_ilu_backward(nd, rs, col, dia, ivc, x), G[f"{t}_bwd"])
    for solver, f in (("pcg", port.nd_solve_pcg), ("pbicgstab", port.nd_solve_pbicgstab)):
        xs, _, hist = f(nd, s["ind"], s["psup"], s["vc"], s["vd"], rs, col, dia, ivc, ivd, s["b"], 1e-10, 1000)
        assert np.array_equal(hist, G[f"{t}_{solver}_hist"]), solver
        assert np.array_equal(xs, G[f"{t}_{solver}_x"]), solver


@pytest.mark.parametrize("nd", [1, 2, 3])
def test_merge_repeated_node_matches_golden(port, nd):
    G = golden("nd")
    ind = np.array([0, 2, 4, 6], np.uint32)
    psup = np.array([1, 2, 0, 2, 0, 1], np.uint32)
    vc, vd = G[f"merge{nd}_vc0"].copy(), G[f"merge{nd}_vd0"].copy()
    nodes = np.array([0, 1, 0, 2], np.uint32)
    emat = G[f"merge{nd}_emat"]
    st = port.nd_merge(nd, ind, psup, vc, vd, nodes, emat) if nd < 3 else port.merge(ind, psup, vc, vd, nodes, emat)
    assert st == 0
    assert np.array_equal(vc, G[f"merge{nd}_vc"]) and np.array_equal(vd, G[f"merge{nd}_vd"])


def test_singular_pivots(port):
    """A zero pivot is counted and left; the eleventh stops the factorisation
    with failure (ls_ilu_block_sparse.cpp:154, 192-201, 255-264)."""
    n = 12
    ind = np.zeros(n + 1, np.uint32)
    psup = np.zeros(0, np.uint32)
    dia = np.zeros(n, np.uint32)
    for nd, vd in ((1, np.zeros(n)), (2, np.zeros(4 * n))):
        st, _, out = port.nd_ilu_decompose(nd, ind, psup, dia, np.zeros(0), vd.copy())
        assert st == 1
    vd = np.zeros(10)
    st, _, out = port.nd_ilu_decompose(1, ind[:11], psup, dia[:10], np.zeros(0), vd)
    assert st == 0 and not out.any()  # ten singular pivots are tolerated


@pytest.mark.skipif(not HAVE_REFERENCE_BUILD(), reason="reference driver not built")
@pytest.mark.parametrize("name", list(S.SYSTEMS))
def test_port_equals_reference_directly(port, name):
    from oracle import reference
    R = reference()
    sp, sr = S.SYSTEMS[name](port), S.SYSTEMS[name](R)
    for k in ("vc", "vd", "b"):
        assert np.array_equal(sp[k], sr[k])
    nd = sp["ndim"]
    for k in (0, 2):
        fp, fr = S.factor(port, sp, k), S.factor(R, sp, k)
        for a, b in zip(fp, fr):
            assert np.array_equal(a, b)
        xp, _, hp = port.nd_solve_pcg(nd, sp["ind"], sp["psup"], sp["vc"], sp["vd"], *fp, sp["b"], 1e-12, 1000)
        xr, _, hr = R.nd_solve_pcg(nd, sp["ind"], sp["psup"], sp["vc"], sp["vd"], *fp, sp["b"], 1e-12, 1000)
        assert np.array_equal(hp, hr) and np.array_equal(xp, xr)
