"""Scalar (1x1) and 2x2 block matrices on the GPU against the reference's
outputs in tests/golden/nd.npz (tests/nd_systems.py describes the systems:
Poisson on tets, Poisson on 2-D triangles, the 2-D linear solid).

Bars: the ILU(0) / ILU(1) factors are bit-identical to the reference's (the
device factorisation keeps the reference's rounding for 1x1 and 2x2 blocks);
assembly, MatVec and sweeps within 1e-12 (summation order); Solve_PCG with
the same history length (+-1) and x within 1e-8; Solve_PBiCGStab and the
mixed-precision solver converged with x within 1e-6 of the reference's."""
import numpy as np
import pytest

import nd_systems as S
from conftest import golden, rel_err

pytestmark = pytest.mark.gpu
NAMES = list(S.SYSTEMS)


def _device_system(name, G):
    """Pattern from the fixture, assembly on the device, clamp, rhs zero."""
    import delfem2_gb300 as D
    from oracle import port
    s = S.SYSTEMS[name](port())  # mesh and boundary values (the restatement's, equal to the reference's)
    nd = s["ndim"]
    ind, psup = G[f"{name}_ind"], G[f"{name}_psup"]
    K = D.CMatrixSparse()
    K.Initialize(ind.size - 1, nd, True)
    K.SetPattern(ind, psup)
    b = np.zeros((ind.size - 1) * nd)
    if name == "poisson_tet":
        mesh = D.TetMesh(K, s["xyz"], s["elem"])
        mesh.assemble_poisson(S.POISSON["alpha"], S.POISSON["source"], b, s["val"])
    else:
        mesh = D.TriMesh2(K, s["xy"], s["elem"])
        if nd == 1:
            mesh.assemble_poisson(S.POISSON["alpha"], S.POISSON["source"], b, s["val"])
        else:
            p = S.SOLID2
            mesh.assemble_solid_linear(p["myu"], p["lam"], p["rho"], (p["gx"], p["gy"]), b)
    K.SetFixedBC(G[f"{name}_bc"])
    D.setRHS_Zero(b, G[f"{name}_bc"])
    return K, b, mesh


def _matrix_from_fixture(name, G):
    import delfem2_gb300 as D
    ind, psup = G[f"{name}_ind"], G[f"{name}_psup"]
    nd = int(round(np.sqrt(G[f"{name}_vd"].size / (ind.size - 1))))
    K = D.CMatrixSparse()
    K.Initialize(ind.size - 1, nd, True)
    K.SetPattern(ind, psup)
    K.set_values(G[f"{name}_vc"], G[f"{name}_vd"])
    return K


@pytest.mark.parametrize("name", NAMES)
def test_device_assembly(gpu, name):
    G = golden("nd")
    K, b, _ = _device_system(name, G)
    vc, vd = K.get_values()
    assert rel_err(vc, G[f"{name}_vc"]) < 1e-12
    assert rel_err(vd, G[f"{name}_vd"]) < 1e-12
    assert rel_err(b, G[f"{name}_b"]) < 1e-12


@pytest.mark.parametrize("name", NAMES)
def test_matvec(gpu, name):
    import torch
    G = golden("nd")
    K = _matrix_from_fixture(name, G)
    y = G[f"{name}_mv_y"].copy()
    K.MatVec(y, 1.5, G[f"{name}_mv_x"], 0.5)
    assert rel_err(y, G[f"{name}_mv"]) < 1e-12
    yd = torch.tensor(G[f"{name}_mv_y"], device="cuda")
    K.MatVec(yd, 1.5, torch.tensor(G[f"{name}_mv_x"], device="cuda"), 0.5)
    assert np.array_equal(yd.cpu().numpy(), y)
    # beta = 0 keeps a NaN of y (y is scaled by beta first)
    y = G[f"{name}_mv_y"].copy()
    y[3] = np.nan
    K.MatVec(y, 1.0, G[f"{name}_mv_x"], 0.0)
    assert np.isnan(y[3]) and np.isfinite(np.delete(y, 3)).all()


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("k", [0, 1])
def test_factors_are_the_reference_bits(gpu, name, k):
    import delfem2_gb300 as D
    G = golden("nd")
    K = _matrix_from_fixture(name, G)
    ilu = D.CPreconditionerILU()
    ilu.Initialize_ILUk(K, k)
    ilu.CopyValue(K)
    assert ilu.Decompose()
    t = f"{name}_k{k}"
    col, dia = ilu.pattern()
    assert np.array_equal(ilu.row_start(), G[f"{t}_rs"])
    assert np.array_equal(col, G[f"{t}_col"]) and np.array_equal(dia, G[f"{t}_dia"])
    vc, vd = ilu.values()
    assert np.array_equal(vc, G[f"{t}_vc"]) and np.array_equal(vd, G[f"{t}_vd"])


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("k", [0, 1])
@pytest.mark.parametrize("mode", [0, 1, 5, 7])
def test_sweeps(gpu, name, k, mode):
    import delfem2_gb300 as D
    G = golden("nd")
    K = _matrix_from_fixture(name, G)
    ilu = D.CPreconditionerILU()
    ilu.Initialize_ILUk(K, k)
    ilu.CopyValue(K)
    assert ilu.Decompose()
    ilu.set_sweep_mode(mode)
    t = f"{name}_k{k}"
    v = G[f"{name}_mv_x"].copy()
    ilu.ForwardSubstitution(v)
    assert rel_err(v, G[f"{t}_fwd"]) < 1e-12
    v = G[f"{name}_mv_x"].copy()
    ilu.BackwardSubstitution(v)
    assert rel_err(v, G[f"{t}_bwd"]) < 1e-12
    for m in (2, 3, 4):  # the blob, block and row-range schedules are written for 3x3 blocks
        with pytest.raises(D.Dfm2gError):
            ilu.set_sweep_mode(m)


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("k", [0, 1])
def test_solvers(gpu, name, k):
    import delfem2_gb300 as D
    G = golden("nd")
    K = _matrix_from_fixture(name, G)
    ilu = D.CPreconditionerILU()
    ilu.Initialize_ILUk(K, k)
    ilu.CopyValue(K)
    assert ilu.Decompose()
    b = G[f"{name}_b"]
    t = f"{name}_k{k}"
    r, x = b.copy(), np.zeros_like(b)
    hist = D.Solve_PCG(r, x, 1e-10, 1000, K, ilu)
    gh = G[f"{t}_pcg_hist"]
    assert abs(len(hist) - len(gh)) <= 1
    assert rel_err(x, G[f"{t}_pcg_x"]) < 1e-8
    r, x = b.copy(), np.zeros_like(b)
    st = D.SolveStats()
    hb = D.Solve_PBiCGStab(r, x, 1e-10, 1000, K, ilu, st)
    assert hb[-1] < 1e-10 and st.rel_residual < 1e-9
    assert rel_err(x, G[f"{t}_pbicgstab_x"]) < 1e-6
    x = np.zeros_like(b)
    st = D.Solve_PCG_Mixed(b, x, 1e-10, K, ilu)
    assert st.rel_residual < 1e-10
    assert rel_err(x, G[f"{t}_pcg_x"]) < 1e-6


@pytest.mark.parametrize("name", NAMES)
def test_solve_on_device_tensors_is_deterministic(gpu, name):
    import torch
    import delfem2_gb300 as D
    G = golden("nd")
    K = _matrix_from_fixture(name, G)
    ilu = D.CPreconditionerILU()
    ilu.SetPattern0(K)
    ilu.CopyValue(K)
    assert ilu.Decompose()
    b = G[f"{name}_b"]
    rh, xh = b.copy(), np.zeros_like(b)
    hh = D.Solve_PCG(rh, xh, 1e-10, 1000, K, ilu)
    rd = torch.tensor(b, device="cuda")
    xd = torch.zeros_like(rd)
    hd = D.Solve_PCG(rd, xd, 1e-10, 1000, K, ilu)
    assert hd == hh and np.array_equal(xd.cpu().numpy(), xh)


@pytest.mark.parametrize("nd", [1, 2, 3])
def test_merge_repeated_node(gpu, nd):
    """One element whose nodes 0 and 2 coincide: the (irow, irow) diagonal rule
    and the reference's order of additions (bit-identical)."""
    import delfem2_gb300 as D
    G = golden("nd")
    ind = np.array([0, 2, 4, 6], np.uint32)
    psup = np.array([1, 2, 0, 2, 0, 1], np.uint32)
    K = D.CMatrixSparse()
    K.Initialize(3, nd, True)
    K.SetPattern(ind, psup)
    K.set_values(G[f"merge{nd}_vc0"], G[f"merge{nd}_vd0"])
    D.Merge(K, np.array([0, 1, 0, 2], np.uint32), G[f"merge{nd}_emat"])
    vc, vd = K.get_values()
    assert np.array_equal(vc, G[f"merge{nd}_vc"]) and np.array_equal(vd, G[f"merge{nd}_vd"])


def test_block_size_guards(gpu):
    """Assemblers written for one block size refuse the others."""
    import delfem2_gb300 as D
    from oracle import port
    s = S.poisson_tet(port(), 4)
    K = D.CMatrixSparse()
    K.Initialize(s["ind"].size - 1, 1, True)
    K.SetPattern(s["ind"], s["psup"])
    mesh = D.TetMesh(K, s["xyz"], s["elem"])
    with pytest.raises(D.Dfm2gError):
        mesh.assemble_linear(np.ones(s["elem"].size // 4), 0.3, 1.0, (0, 0, -1), np.zeros(s["ind"].size * 3))
    K2 = D.CMatrixSparse()
    K2.Initialize(s["ind"].size - 1, 2, True)
    K2.SetPattern(s["ind"], s["psup"])
    with pytest.raises(D.Dfm2gError):
        D.TetMesh(K2, s["xyz"], s["elem"])
    K4 = D.CMatrixSparse()
    with pytest.raises(D.Dfm2gError):
        K4.Initialize(8, 4, True)
