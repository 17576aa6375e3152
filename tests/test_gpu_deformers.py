"""The two deformers of the reference that solve through the block ILU-PCG
path, driven through the drop-in: the ARAP deformer (Deformer_Arap,
defarap.cpp:436-540: per-point elements through the runtime-size Merge,
AddDia(1e-8), SetFixedBC, setRHS_Zero, ILU(0), Solve_PCG to 1e-7 with at most
300 iterations) and the linear Laplacian deformer (CDef_LaplacianLinear,
deflap.cpp:228-360: dual-Laplacian elements, Initialize_ILUk(Mat, 20) of the
matrix with its boundary penalties, Solve_PCG to 1e-5 over the penalised
operator). The deformers' element code stays on the host, as in the
reference; the element matrices are the ones the reference handed to Merge
(tests/golden/deform.npz, recorded by tests/golden/make_golden.py).

Checked: the matrix pattern (the 1-ring extended to the 2-ring) and the
ILU(20) fill pattern bit-exact; the assembled matrix against the same
elements merged by the oracle (1e-12); the PCG history length within one of
the reference's and the deformed positions within 1e-6 of the displacement
(both solves stop at a relative residual of 1e-7 / 1e-5)."""
import os
import sys

import numpy as np
import pytest

from conftest import golden, rel_err

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from deform_systems import extend_pattern  # noqa: E402


def _pattern(tri, np_):
    import delfem2_gb300 as D
    ind, psup = D.JArray_PSuP_MeshElem(tri, 3, np_)
    return extend_pattern(ind, psup, np_)


def test_deformer_pattern_is_the_reference_2ring(built_lib):
    """CPU: the 2-ring pattern built here from the C ABI's 1-ring is the one
    the reference's deformers build (JArray_Extend + JArray_Sort)."""
    G = golden("deform")
    np_ = G["xyz0"].size // 3
    ind, col = _pattern(G["tri"], np_)
    assert np.array_equal(ind, G["lap_pat_start"]) and np.array_equal(col, G["lap_pat_col"])


def _merge_elements(K, ptr, idx, eM):
    """Merge every point's element (variable size: its 1-ring and itself),
    one batch per element size, as the deformers' Mearge loop does."""
    import delfem2_gb300 as D
    np_ = ptr.size - 1
    sizes = np.diff(ptr)
    mstart = np.concatenate([[0], np.cumsum(9 * sizes.astype(np.int64) ** 2)])
    for n in np.unique(sizes):
        pts = np.nonzero(sizes == n)[0]
        elem = np.stack([idx[ptr[p]:ptr[p + 1]] for p in pts])
        em = np.stack([eM[mstart[p]:mstart[p + 1]] for p in pts])
        D.Merge(K, elem, em.reshape(len(pts), n, n, 3, 3))




@pytest.mark.gpu
def test_arap_deformer_through_the_dropin(gpu, port):
    import delfem2_gb300 as D
    G = golden("deform")
    xyz0, tri, bc, xdef = G["xyz0"], G["tri"], G["bc"], G["xdef"]
    np_ = xyz0.size // 3
    ind, col = _pattern(tri, np_)
    K = D.CMatrixSparse()
    K.Initialize(np_, 3, True)
    K.SetPattern(ind, col)
    K.setZero()
    ptr, idx, eM, eR = G["arap_ptr"], G["arap_idx"], G["arap_eM"], G["arap_eR"]
    _merge_elements(K, ptr, idx, eM)
    # the residual the deformer accumulates on the host
    res = np.zeros(np_ * 3)
    np.add.at(res, (3 * idx[:, None] + np.arange(3)).ravel(), eR)
    # the same elements merged by the oracle, in the reference's element order
    vc_o, vd_o = np.zeros(col.size * 9), np.zeros(np_ * 9)
    sizes = np.diff(ptr)
    mstart = np.concatenate([[0], np.cumsum(9 * sizes.astype(np.int64) ** 2)])
    for p in range(np_):
        e = idx[ptr[p]:ptr[p + 1]]
        assert port.merge(ind, col, vc_o, vd_o, e, eM[mstart[p]:mstart[p + 1]]) == 0
    vc, vd = K.get_values()
    assert rel_err(vc, vc_o) < 1e-12 and rel_err(vd, vd_o) < 1e-12
    K.AddDia(1e-8)
    K.SetFixedBC(bc)
    D.setRHS_Zero(res, bc)
    ilu = D.CPreconditionerILU()
    ilu.SetPattern0(K)
    ilu.CopyValue(K)
    assert ilu.Decompose()
    upd = np.zeros_like(res)
    hist = D.Solve_PCG(res.copy(), upd, 1e-7, 300, K, ilu)
    href = G["arap_hist"]
    assert abs(len(hist) - len(href)) <= 1
    x = xdef - upd
    assert np.abs(x - G["arap_x"]).max() <= 1e-6 * np.abs(upd).max()


@pytest.mark.gpu
def test_laplacian_deformer_ilu20_through_the_dropin(gpu):
    import delfem2_gb300 as D
    G = golden("deform")
    xyz0, tri, bc, xdef = G["xyz0"], G["tri"], G["bc"], G["xdef"]
    np_ = xyz0.size // 3
    ind, col = _pattern(tri, np_)
    K = D.CMatrixSparse()
    K.Initialize(np_, 3, True)
    K.SetPattern(ind, col)
    K.setZero()
    _merge_elements(K, G["lap_ptr"], G["lap_idx"], G["lap_eM"])
    # right-hand side of Deform: aRes0 - Mat x_def with aRes0 = -Mat x0, i.e. Mat (x0 - x_def)
    rhs = np.zeros(np_ * 3)
    K.MatVec(rhs, 1.0, xyz0 - xdef, 0.0)
    # the boundary penalty (weight_bc = 100 on the fixed DOFs' diagonal) makes
    # the deformer's operator; the preconditioner is ILU(20) of it
    vc, vd = K.get_values()
    vd = vd.reshape(np_, 3, 3)
    fixed = bc.reshape(np_, 3)
    for d in range(3):
        vd[:, d, d] += 100.0 * (fixed[:, d] != 0)
    K.set_values(vc, vd.ravel())
    ilu = D.CPreconditionerILU()
    ilu.Initialize_ILUk(K, 20)
    icol, _ = ilu.pattern()
    assert np.array_equal(ilu.row_start(), G["lap_ilu_start"]) and np.array_equal(icol, G["lap_ilu_col"])
    ilu.CopyValue(K)
    assert ilu.Decompose()
    upd = np.zeros_like(rhs)
    hist = D.Solve_PCG(rhs.copy(), upd, 1e-5, 300, K, ilu)
    href = G["lap_hist"]
    assert abs(len(hist) - len(href)) <= 1
    x = xdef + upd
    assert np.abs(x - G["lap_xyz_def"]).max() <= 1e-6 * np.abs(upd).max()
