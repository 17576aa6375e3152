"""Dynamic linear-tet assembly on the GPU against the reference's outputs
(tests/golden/dynamic.npz): backward Euler, stiffness-warped backward Euler
and Newmark-beta (fem_solidlinear.h:331-530). K and b within 1e-12. The
warped matrix is not symmetric (R_i K_ij R_i^T); it is solved with
Solve_PBiCGStab and ILU(0) as 603_Fem3DStiffwarp/main.cpp:201-220 does, and
checked against the oracle's BiCGStab solution."""
import numpy as np
import pytest

import dyn_systems as DS
from conftest import golden, rel_err

pytestmark = pytest.mark.gpu


def _assemble(kind, s, device=False):
    import torch
    import delfem2_gb300 as D
    nb = s["xyz"].size // 3
    K = D.CMatrixSparse()
    K.Initialize(nb, 3, True)
    K.SetPattern(s["ind"], s["psup"])
    mesh = D.TetMesh(K, s["xyz"], s["tet"])
    m = DS.MAT
    conv = (lambda a: torch.tensor(a, device="cuda")) if device else (lambda a: a)
    b = conv(np.zeros(nb * 3))
    if kind == "newmark":
        mesh.assemble_newmark(m["myu"], m["lam"], m["rho"], m["g"], m["dt"], m["gamma"], m["beta"], conv(s["u"]),
                              conv(s["v"]), conv(s["acc"]), b)
    else:
        mesh.assemble_beuler(m["myu"], m["lam"], m["rho"], m["g"], m["dt"], conv(s["u"]), conv(s["v"]), b,
                             rot=conv(s["rot"]) if kind == "warp" else None)
    return K, (b.cpu().numpy() if device else b), mesh


@pytest.mark.parametrize("kind", DS.KINDS)
@pytest.mark.parametrize("device", [False, True])
def test_assembly_matches_reference(gpu, kind, device):
    from oracle import port
    G = golden("dynamic")
    s = DS.inputs(port())
    K, b, _ = _assemble(kind, s, device)
    vc, vd = K.get_values()
    assert rel_err(vc, G[f"{kind}_vc"]) < 1e-12
    assert rel_err(vd, G[f"{kind}_vd"]) < 1e-12
    assert rel_err(b, G[f"{kind}_b"]) < 1e-12


def test_warped_system_solved_with_bicgstab(gpu):
    import delfem2_gb300 as D
    from oracle import port
    O = port()
    s = DS.inputs(O)
    K, b, _ = _assemble("warp", s)
    z = s["xyz"].reshape(-1, 3)[:, 2]  # the z = 0 face is clamped
    bc = np.repeat((z < 1e-12).astype(np.int32), 3)
    K.SetFixedBC(bc)
    D.setRHS_Zero(b, bc)
    ilu = D.CPreconditionerILU()
    ilu.SetPattern0(K)
    ilu.CopyValue(K)
    assert ilu.Decompose()
    r, x = b.copy(), np.zeros_like(b)
    st = D.SolveStats()
    hist = D.Solve_PBiCGStab(r, x, 1e-10, 1000, K, ilu, st)
    assert hist[-1] < 1e-10 and st.rel_residual < 1e-9
    vc, vd = K.get_values()
    col, dia = ilu.pattern()
    ivc, ivd = ilu.values()
    xo, _, _ = O.solve_pbicgstab(s["ind"], s["psup"], vc, vd, s["ind"], col, dia, ivc, ivd, b, 1e-12, 2000)
    assert rel_err(x, xo) < 1e-7


@pytest.mark.parametrize("device", [False, True])
def test_hex_q1_assembly_matches_reference(gpu, device):
    import torch
    import delfem2_gb300 as D
    from oracle import port
    G = golden("dynamic")
    s = DS.hex_inputs(port())
    nb = s["xyz"].size // 3
    K = D.CMatrixSparse()
    K.Initialize(nb, 3, True)
    K.SetPattern(s["ind"], s["psup"])
    mesh = D.HexMesh(K, s["xyz"], s["hex"])
    m = DS.MAT
    if device:
        b = torch.zeros(nb * 3, dtype=torch.float64, device="cuda")
        mesh.assemble_linear(m["myu"], m["lam"], m["rho"], m["g"], b, torch.tensor(s["u"], device="cuda"))
        b = b.cpu().numpy()
    else:
        b = np.zeros(nb * 3)
        mesh.assemble_linear(m["myu"], m["lam"], m["rho"], m["g"], b, s["u"])
    vc, vd = K.get_values()
    assert rel_err(vc, G["hexq1_vc"]) < 1e-12
    assert rel_err(vd, G["hexq1_vd"]) < 1e-12
    assert rel_err(b, G["hexq1_b"]) < 1e-12


def test_hex_with_repeated_node_is_refused(gpu):
    import delfem2_gb300 as D
    from oracle import port
    s = DS.hex_inputs(port(), 1, 1, 1)
    K = D.CMatrixSparse()
    K.Initialize(8, 3, True)
    K.SetPattern(s["ind"], s["psup"])
    bad = s["hex"].copy()
    bad[3] = bad[0]
    with pytest.raises(D.Dfm2gError):
        D.HexMesh(K, s["xyz"], bad)
