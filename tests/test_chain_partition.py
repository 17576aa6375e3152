"""Chain partition of the chain-scheduled sweeps (dfm2g_chain_partition, host
only; csrc/chain.cu), on ILU patterns and level orders from the oracle.

Checked for both sweep directions: every chain is a run of consecutive rows in
which each row depends on the one before (ascending forward, descending
backward); every dependency of a row lies in a lower-numbered chain or earlier
in the row's own chain, the rule the sweep's freedom from deadlock rests on;
chains are numbered in the level order of their first rows. On the natural
ordering of a voxel mesh (nodes numbered z fastest) the chains are the z
pencils, with six dependencies outside the chain per row."""
import ctypes as C

import numpy as np
import pytest


def _partition(lib, ind, col, dia, order, backward):
    n = ind.size - 1
    chain_of = np.zeros(max(n, 1), np.uint32)
    nchain, m = C.c_uint(0), C.c_uint(0)
    u32 = lambda a: np.ascontiguousarray(a, np.uint32)
    ind, col, dia, order = u32(ind), u32(col), u32(dia), u32(order)
    st = lib.dfm2g_chain_partition(n, ind.ctypes.data, col.ctypes.data, dia.ctypes.data, order.ctypes.data,
                                   int(backward), chain_of.ctypes.data, C.byref(nchain), C.byref(m))
    assert st == 0
    return chain_of[:n], nchain.value, m.value


def _check(ind, col, dia, level, chain_of, nchain, m, backward):
    n = ind.size - 1
    assert chain_of.max() + 1 == nchain
    rows_of = [[] for _ in range(nchain)]
    for i in (range(n - 1, -1, -1) if backward else range(n)):
        rows_of[chain_of[i]].append(i)
    step = -1 if backward else 1
    heads = []
    max_cross = 0
    for c, rows in enumerate(rows_of):
        assert rows, c
        heads.append(rows[0])
        for a, b in zip(rows, rows[1:]):
            assert b == a + step, (c, a, b)  # consecutive rows
            deps = col[dia[b]:ind[b + 1]] if backward else col[ind[b]:dia[b]]
            assert a in deps, (c, a, b)      # each row depends on the one before
    for i in range(n):
        deps = col[dia[i]:ind[i + 1]] if backward else col[ind[i]:dia[i]]
        prev = i + 1 if backward else i - 1
        linked = chain_of[i] == chain_of[prev] if 0 <= prev < n and prev in deps else False
        max_cross = max(max_cross, len(deps) - (1 if linked else 0))
        for j in deps:
            assert chain_of[j] <= chain_of[i], (i, j)
            if chain_of[j] == chain_of[i]:  # earlier in the same chain
                assert (j > i) if backward else (j < i), (i, j)
    assert max_cross == m
    hl = level[np.array(heads)]
    assert np.all(np.diff(hl.astype(np.int64)) >= 0)  # numbered in the level order of the first rows


def test_voxel_mesh_chains_are_z_pencils(built_lib, port):
    import delfem2_gb300 as D
    a = D.voxel_problem_arrays(8, 6, 5, 1.0 / 8, young=1.0)
    ind, psup = a["psup_ind"], a["psup"]
    col, dia = port.ilu_pattern0(ind, psup)
    for backward in (False, True):
        level, order, _ = port.ilu_levels(ind, col, dia, backward)
        chain_of, nchain, m = _partition(built_lib, ind, col, dia, order, backward)
        _check(ind, col, dia, level, chain_of, nchain, m, backward)
        assert nchain == 9 * 7 and m == 6  # (nx+1)(ny+1) pencils of nz+1 rows
        assert np.array_equal(np.bincount(chain_of), np.full(nchain, 6))


@pytest.mark.parametrize("seed", [0, 1])
def test_random_pattern_cuts_chains_by_the_rule(built_lib, port, seed):
    rng = np.random.default_rng(seed)
    n = 400
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
    ind[1:] = np.cumsum([len(x) for x in nbr])
    psup = np.array([j for x in nbr for j in sorted(x)], np.uint32)
    col, dia = port.ilu_pattern0(ind, psup)
    for backward in (False, True):
        level, order, _ = port.ilu_levels(ind, col, dia, backward)
        chain_of, nchain, m = _partition(built_lib, ind, col, dia, order, backward)
        _check(ind, col, dia, level, chain_of, nchain, m, backward)
        assert 1 < nchain < n  # some rows chained, some chains cut


def test_empty_pattern(built_lib):
    z = np.zeros(1, np.uint32)
    nchain, m = C.c_uint(7), C.c_uint(7)
    assert built_lib.dfm2g_chain_partition(0, z.ctypes.data, z.ctypes.data, z.ctypes.data, z.ctypes.data, 0,
                                           z.ctypes.data, C.byref(nchain), C.byref(m)) == 0
    assert nchain.value == 0 and m.value == 0


@pytest.mark.parametrize("k", [1, 2, -1])
def test_fill_in_patterns(built_lib, port, k):
    """ILU(k) patterns (Initialize_ILUk's fill, -1 = full) of a small voxel
    mesh: longer rows, more dependencies outside a row's chain."""
    import delfem2_gb300 as D
    a = D.voxel_problem_arrays(5, 4, 3, 0.2, young=1.0)
    rs, col, dia = port.ilu_pattern_k(a["psup_ind"], a["psup"], k)
    m_prev = None
    for backward in (False, True):
        level, order, _ = port.ilu_levels(rs, col, dia, backward)
        chain_of, nchain, m = _partition(built_lib, rs, col, dia, order, backward)
        _check(rs, col, dia, level, chain_of, nchain, m, backward)
        assert m > 6  # fill adds dependencies beyond the ILU(0) neighbours
        if m_prev is not None:
            assert m == m_prev  # the pattern is symmetric: both triangles alike
        m_prev = m
