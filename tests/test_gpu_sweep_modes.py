"""Sweep schedules on patterns that stress their edge paths, against the oracle.

The arrow pattern (row 0 coupled to every row) has two levels per direction:
the forward sweep's second level reads row 0 from more than a shared-memory
ring's length back (the single-CTA schedule's global-memory path), and the
backward sweep's row 0 has n-1 blocks (the long-row paths). The chain pattern
(tridiagonal blocks) has one row per level (n levels) and is one chain of the
chain schedule. The random pattern (runs of (i-1, i) couplings plus random
long-range ones) makes the chain schedule cut chains where a row's other
dependencies lie in later chains. Tolerance 1e-12
relative (FP64), 1e-5 (FP32).
"""
import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu


def _system(kind, n, seed):
    rng = np.random.default_rng(seed)
    if kind == "arrow":
        nbr = [list(range(1, n))] + [[0] for _ in range(1, n)]
    elif kind == "chain":
        nbr = [[j for j in (i - 1, i + 1) if 0 <= j < n] for i in range(n)]
    else:  # runs of i-1 couplings cut at random, plus two random couplings per row
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
        nbr = [sorted(a) for a in nbr]
    ind = np.zeros(n + 1, np.uint32)
    ind[1:] = np.cumsum([len(a) for a in nbr])
    psup = np.array([j for a in nbr for j in a], np.uint32)
    vc = 0.1 * rng.standard_normal(psup.size * 9) / max(1.0, np.sqrt(n) if kind == "arrow" else 1.0)
    vd = np.tile(np.eye(3).ravel(), n) * 4.0 + 0.1 * rng.standard_normal(n * 9)
    return ind, psup, vc, vd


@pytest.mark.parametrize("kind,n", [("arrow", 20000), ("chain", 3000), ("random", 6000)])
@pytest.mark.parametrize("mode", [0, 1, 3, 4, 5, 6, 7, 8])
def test_sweep_modes_on_edge_patterns(gpu, port, kind, n, mode):
    import delfem2_gb300 as D
    ind, psup, vc, vd = _system(kind, n, 3)
    K = D.CMatrixSparse()
    K.Initialize(n, 3, True)
    K.SetPattern(ind, psup)
    K.set_values(vc, vd)
    ilu = D.CPreconditionerILU()
    ilu.SetPattern0(K)
    ilu.CopyValue(K)
    assert ilu.Decompose()
    ilu.set_sweep_mode(mode)
    col, dia = port.ilu_pattern0(ind, psup)
    ivc, ivd = port.ilu_copy_value(ind, col, psup, vc, vd)
    st, _ = port.ilu_decompose(ind, col, dia, ivc, ivd)
    assert st == 0
    v = np.random.default_rng(5).standard_normal(n * 3)
    f = v.copy()
    ilu.ForwardSubstitution(f)
    fo = port.ilu_forward(ind, col, dia, ivc, ivd, v)
    assert rel_err(f, fo) < 1e-12
    g = fo.copy()
    ilu.BackwardSubstitution(g)
    go = port.ilu_backward(ind, col, dia, ivc, fo)
    assert rel_err(g, go) < 1e-12
    z32 = v.astype(np.float32)
    ilu.SolvePrecond(z32)
    assert rel_err(z32, go) < 1e-5


def test_chain_kernels_shared_by_patterns_with_different_records(gpu, port):
    """Two preconditioners whose chain sweeps run the same kernel with different
    record sizes (a voxel mesh: six cross blocks per row; a block-tridiagonal
    matrix: none), swept in turn: the second must not break the first's
    launches (the kernel's shared-memory limit is shared by both)."""
    import delfem2_gb300 as D

    def prepare(ind, psup, vc, vd, n):
        K = D.CMatrixSparse()
        K.Initialize(n, 3, True)
        K.SetPattern(ind, psup)
        K.set_values(vc, vd)
        ilu = D.CPreconditionerILU()
        ilu.SetPattern0(K)
        ilu.CopyValue(K)
        assert ilu.Decompose()
        assert ilu.sweep_mode() == 7  # the default: tiles or chains, picked per pattern
        ilu.set_sweep_mode(5)
        col, dia = port.ilu_pattern0(ind, psup)
        ivc, ivd = port.ilu_copy_value(ind, col, psup, vc, vd)
        assert port.ilu_decompose(ind, col, dia, ivc, ivd)[0] == 0
        return ilu, (ind, col, dia, ivc, ivd)

    a = D.voxel_problem_arrays(4, 4, 4, 0.25, young=1.0)
    n1 = a["np"]
    rng = np.random.default_rng(11)
    vc1 = 0.05 * rng.standard_normal(a["psup"].size * 9)
    vd1 = np.tile(np.eye(3).ravel(), n1) * 4.0 + 0.1 * rng.standard_normal(n1 * 9)
    ilu1, o1 = prepare(a["psup_ind"], a["psup"], vc1, vd1, n1)
    ind2, psup2, vc2, vd2 = _system("chain", 500, 4)
    ilu2, o2 = prepare(ind2, psup2, vc2, vd2, 500)
    for ilu, o, n in ((ilu1, o1, n1), (ilu2, o2, 500), (ilu1, o1, n1)):
        v = np.random.default_rng(n).standard_normal(n * 3).astype(np.float32)
        f = v.copy()
        ilu.ForwardSubstitution(f)
        fo = port.ilu_forward(o[0], o[1], o[2], o[3], o[4], v.astype(np.float64))
        assert rel_err(f, fo) < 1e-5
