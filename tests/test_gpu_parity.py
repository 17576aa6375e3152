"""GPU path vs the CPU oracle and the reference-recorded fixtures.

Tolerances: integer data (patterns, dia_ind, level sets, orders) bit-exact;
FP64 values within 1e-12 relative (summation order differs); FP32 kernels
within 1e-5 relative of the FP64 oracle; solutions of Solve_PCG within 1e-8.
"""
import numpy as np
import pytest

from conftest import golden, rel_err

pytestmark = pytest.mark.gpu

NU, RHO, G = 0.3, 1.0, (0.0, 0.0, -1e-3)


def oracle_system(port, nx, ny, nz, h, young):
    xyz, tet = port.voxel_tet_mesh(nx, ny, nz, h)
    np_ = xyz.size // 3
    ind, psup = port.psup(tet, 4, np_)
    vc, vd, b = np.zeros(psup.size * 9), np.zeros(np_ * 9), np.zeros(np_ * 3)
    assert port.assemble_tet_linear(ind, psup, vc, vd, b, xyz, tet, young, NU, RHO, G) == 0
    K0 = (vc.copy(), vd.copy(), b.copy())
    bc = np.zeros(np_ * 3, np.int32)
    bc[np.repeat(xyz[2::3] == 0.0, 3)] = 1
    port.set_fixed_bc(ind, psup, vc, vd, bc)
    port.rhs_zero(b, bc)
    col, dia = port.ilu_pattern0(ind, psup)
    ivc, ivd = port.ilu_copy_value(ind, col, psup, vc, vd)
    st, _ = port.ilu_decompose(ind, col, dia, ivc, ivd)
    assert st == 0
    return dict(xyz=xyz, tet=tet, ind=ind, psup=psup, vc=vc, vd=vd, b=b, bc=bc, col=col, dia=dia, ivc=ivc,
                ivd=ivd, K0=K0, young=young)


def gpu_problem(s):
    import delfem2_gb300 as D
    arrays = dict(xyz=s["xyz"], tet=s["tet"], psup_ind=s["ind"], psup=s["psup"], bc=s["bc"], young=s["young"],
                  np=s["xyz"].size // 3, ntet=s["tet"].size // 4)
    P = D.StaticElasticProblem(arrays, nu=NU, rho=RHO, g=G)
    return P


CASES = {
    "tiny": (3, 2, 2, 1 / 3, lambda n: np.exp(np.random.default_rng(7).uniform(np.log(0.1), np.log(10), n))),
    "cfg1": (16, 16, 16, 1 / 16, lambda n: np.ones(n)),
    "cfg1e": (16, 16, 16, 1 / 16, lambda n: np.exp(np.random.default_rng(0).uniform(np.log(0.1), np.log(10), n))),
}


@pytest.fixture(scope="module", params=list(CASES))
def case(request, gpu, port):
    nx, ny, nz, h, ef = CASES[request.param]
    s = oracle_system(port, nx, ny, nz, h, ef(nx * ny * nz * 6))
    P = gpu_problem(s)
    b = P.assemble()
    ok = P.factor()
    assert ok
    return request.param, s, P, b


def test_assembly_matches_oracle(case):
    name, s, P, b = case
    vc, vd = P.K.get_values()
    assert rel_err(vc, s["vc"]) < 1e-12
    assert rel_err(vd, s["vd"]) < 1e-12
    assert rel_err(b, s["b"]) < 1e-12
    assert P.mesh.ncolor >= 24  # interior voxel nodes touch 24 tets


def test_assembly_without_bc_matches_oracle(case, port):
    name, s, P, _ = case
    import delfem2_gb300 as D
    K = D.CMatrixSparse()
    K.Initialize(s["xyz"].size // 3, 3)
    K.SetPattern(s["ind"], s["psup"])
    m = D.TetMesh(K, s["xyz"], s["tet"])
    b = np.zeros(s["b"].size)
    disp = np.random.default_rng(2).standard_normal(b.size) * 1e-3
    m.assemble_linear(s["young"], NU, RHO, G, b, disp=disp)
    vc0, vd0, _ = s["K0"]
    vc, vd = K.get_values()
    assert rel_err(vc, vc0) < 1e-12 and rel_err(vd, vd0) < 1e-12
    vco, vdo, bo = np.zeros_like(vc0), np.zeros_like(vd0), np.zeros(b.size)
    port.assemble_tet_linear(s["ind"], s["psup"], vco, vdo, bo, s["xyz"], s["tet"], s["young"], NU, RHO, G, disp)
    assert rel_err(b, bo) < 1e-11


def test_ilu_pattern_and_levels_bit_exact(case, port):
    name, s, P, b = case
    col, dia = P.ilu.pattern()
    assert np.array_equal(col, s["col"]) and np.array_equal(dia, s["dia"])
    for backward in (False, True):
        lv, order, ls = P.ilu.levels(backward)
        lo, oo, lso = port.ilu_levels(s["ind"], s["col"], s["dia"], backward)
        assert np.array_equal(lv, lo) and np.array_equal(order, oo) and np.array_equal(ls, lso), backward


def test_ilu_factors_match_oracle(case):
    name, s, P, b = case
    vc, vd = P.ilu.values()
    assert rel_err(vc, s["ivc"]) < 1e-10
    assert rel_err(vd, s["ivd"]) < 1e-10


@pytest.mark.parametrize("mode", [0, 1, 2, 3, 4, 5, 6, 7, 8])
def test_sweeps_match_oracle(case, port, mode):
    name, s, P, b = case
    default = P.ilu.sweep_mode()
    P.ilu.set_sweep_mode(mode)
    try:
        v = np.random.default_rng(4).standard_normal(s["b"].size)
        f = v.copy()
        P.ilu.ForwardSubstitution(f)
        fo = port.ilu_forward(s["ind"], s["col"], s["dia"], s["ivc"], s["ivd"], v)
        assert rel_err(f, fo) < 1e-10
        g = fo.copy()
        P.ilu.BackwardSubstitution(g)
        go = port.ilu_backward(s["ind"], s["col"], s["dia"], s["ivc"], fo)
        assert rel_err(g, go) < 1e-10
        z = v.copy()
        P.ilu.SolvePrecond(z)
        assert rel_err(z, go) < 1e-10
        z32 = v.astype(np.float32)
        P.ilu.SolvePrecond(z32)
        assert rel_err(z32, go) < 1e-4
    finally:
        P.ilu.set_sweep_mode(default)


def test_matvec_matches_oracle(case, port):
    name, s, P, b = case
    rng = np.random.default_rng(9)
    x = rng.standard_normal(s["b"].size)
    y0 = rng.standard_normal(s["b"].size)
    for alpha, beta in [(1.0, 0.0), (0.7, -1.3), (-1.0, 1.0)]:
        y = y0.copy()
        P.K.MatVec(y, alpha, x, beta)
        yo = port.matvec(s["ind"], s["psup"], s["vc"], s["vd"], y0, alpha, x, beta)
        assert rel_err(y, yo) < 1e-12
    y32 = y0.astype(np.float32)
    P.K.MatVec(y32, 1.0, x.astype(np.float32), 0.0)
    yo = port.matvec(s["ind"], s["psup"], s["vc"], s["vd"], y0, 1.0, x, 0.0)
    assert rel_err(y32, yo) < 1e-5
    # beta == 0 keeps a NaN already in y (ls_block_sparse.cpp:222)
    y = y0.copy()
    y[5] = np.nan
    P.K.MatVec(y, 1.0, x, 0.0)
    assert np.isnan(y[5]) and np.isfinite(np.delete(y, 5)).all()


@pytest.mark.parametrize("mode", [0, 1, 2, 3, 4, 5, 6, 7, 8])
def test_solve_pcg_matches_oracle(case, port, mode):
    import delfem2_gb300 as D
    name, s, P, b = case
    default = P.ilu.sweep_mode()
    P.ilu.set_sweep_mode(mode)
    try:
        r = s["b"].copy()
        x = np.zeros_like(r)
        st = D.SolveStats()
        hist = D.Solve_PCG(r, x, 1e-10, 1000, P.K, P.ilu, st)
        xo, ro, ho = port.solve_pcg(s["ind"], s["psup"], s["vc"], s["vd"], s["col"], s["dia"], s["ivc"], s["ivd"],
                                    s["b"], 1e-10, 1000)
        assert abs(len(hist) - len(ho)) <= 1
        # CG histories drift apart chaotically from ulp-level differences in
        # summation order (the port and the reference already differ by ~1e-6)
        k = min(len(hist), len(ho)) // 2
        assert rel_err(hist[:k], ho[:k]) < 1e-4
        assert rel_err(x, xo) < 1e-8
        assert st.rel_residual < 1e-9
        if name.startswith("cfg1"):
            g = golden(name)
            assert abs(len(hist) - 1 - int(g["n_iter"])) <= 1
            assert rel_err(x, g["x"]) < 1e-8
    finally:
        P.ilu.set_sweep_mode(default)


def test_solve_pcg_semantics_exhaustion_and_tiny_rhs(case):
    import delfem2_gb300 as D
    name, s, P, b = case
    r = s["b"].copy()
    x = np.zeros_like(r)
    hist = D.Solve_PCG(r, x, 1e-30, 3, P.K, P.ilu)
    assert len(hist) == 5 and hist[-1] == hist[-2]  # final |r| appended (lsitrsol.h:142-147)
    r = np.full_like(s["b"], 1e-18)
    hist = D.Solve_PCG(r, x, 1e-10, 100, P.K, P.ilu)
    assert len(hist) == 1 and not x.any()  # |r0|^2 < 1e-30: early return with x = 0


def test_solve_cg_matches_oracle(case, port):
    import delfem2_gb300 as D
    name, s, P, b = case
    r = s["b"].copy()
    x = np.zeros_like(r)
    hist = D.Solve_CG(r, x, 1e-8, 3000, P.K)
    xo, ro, ho = port.solve_cg(s["ind"], s["psup"], s["vc"], s["vd"], s["b"], 1e-8, 3000)
    assert abs(len(hist) - len(ho)) <= 10
    assert rel_err(x, xo) < 1e-6


@pytest.mark.parametrize("method", ["reliable", "restart"])
def test_mixed_precision_reaches_fp64_accuracy(case, port, method):
    name, s, P, b = case
    x, st = P.solve_mixed(b, tol=1e-10, inner_tol=1e-4, method=method)
    xo, _, _ = port.solve_pcg(s["ind"], s["psup"], s["vc"], s["vd"], s["col"], s["dia"], s["ivc"], s["ivd"],
                              s["b"], 1e-13, 5000)
    assert st.rel_residual < 1e-10
    assert rel_err(x, xo) < 1e-8
    assert st.outer >= 2


def test_merge_batch_matches_oracle(gpu, port):
    import delfem2_gb300 as D
    xyz, tet = port.voxel_tet_mesh(3, 3, 2, 1.0)
    np_ = xyz.size // 3
    ind, psup = port.psup(tet, 4, np_)
    rng = np.random.default_rng(3)
    elem = tet.reshape(-1, 4)
    emat = rng.standard_normal((elem.shape[0], 4, 4, 3, 3))
    K = D.CMatrixSparse()
    K.Initialize(np_, 3)
    K.SetPattern(ind, psup)
    D.Merge(K, elem, emat)
    vc, vd = np.zeros(psup.size * 9), np.zeros(np_ * 9)
    for e in range(elem.shape[0]):
        assert port.merge(ind, psup, vc, vd, elem[e], emat[e]) == 0
    gvc, gvd = K.get_values()
    assert rel_err(gvc, vc) < 1e-13 and rel_err(gvd, vd) < 1e-13
    with pytest.raises(D.Dfm2gError) as ei:
        D.Merge(K, np.array([[0, np_ - 1, 1, 2]], np.uint32), emat[:1])
    assert ei.value.status == D._native.ERR_MISSING_SLOT
    gvc2, _ = K.get_values()
    assert np.array_equal(gvc2, gvc)  # nothing added on failure


def test_set_fixed_bc_and_add_dia(gpu, port):
    import delfem2_gb300 as D
    xyz, tet = port.voxel_tet_mesh(2, 3, 2, 1.0)
    np_ = xyz.size // 3
    ind, psup = port.psup(tet, 4, np_)
    rng = np.random.default_rng(8)
    vc, vd = rng.standard_normal(psup.size * 9), rng.standard_normal(np_ * 9)
    bc = (rng.random(np_ * 3) < 0.3).astype(np.int32)
    K = D.CMatrixSparse()
    K.Initialize(np_, 3)
    K.SetPattern(ind, psup)
    K.set_values(vc, vd)
    K.SetFixedBC(bc)
    K.AddDia(0.25)
    port.set_fixed_bc(ind, psup, vc, vd, bc)
    vd.reshape(-1, 9)[:, [0, 4, 8]] += 0.25
    gvc, gvd = K.get_values()
    assert np.array_equal(gvc, vc) and rel_err(gvd, vd) < 1e-15


def test_singular_pivots_reported(gpu):
    import delfem2_gb300 as D
    n = 14  # 14 rows, no off-diagonal blocks, all-zero diagonals -> 14 singular pivots
    K = D.CMatrixSparse()
    K.Initialize(n, 3)
    K.SetPattern(np.zeros(n + 1, np.uint32), np.zeros(0, np.uint32))
    ilu = D.CPreconditionerILU()
    ilu.SetPattern0(K)
    ilu.CopyValue(K)
    assert ilu.Decompose() is False and ilu.n_singular == 14
    vd = np.tile(np.eye(3).ravel(), n)
    vd[:9 * 10] = 0.0  # 10 singular pivots: tolerated, like the reference
    K.set_values(None, vd)
    ilu.CopyValue(K)
    assert ilu.Decompose() is True and ilu.n_singular == 10


def test_nonfinite_rhs_is_reported(case):
    import delfem2_gb300 as D
    name, s, P, b = case
    r = s["b"].copy()
    r[0] = np.nan
    x = np.zeros_like(r)
    with pytest.raises(D.Dfm2gError) as ei:
        D.Solve_PCG(r, x, 1e-10, 100, P.K, P.ilu)
    assert ei.value.status == D._native.ERR_NONFINITE


def test_grid_barrier_meets_and_times_out(gpu):
    """The bounded grid barrier of the fused solver kernels: two rounds pass when
    every CTA arrives; when one CTA never arrives the others give up, the call
    reports the timeout and the context stays usable (a solve runs after it)."""
    import delfem2_gb300 as D
    from delfem2_gb300 import _native as N
    lib = N.load()
    assert lib.dfm2g_debug_grid_barrier(50, 0) == N.OK
    assert lib.dfm2g_debug_grid_barrier(50, 1) == N.ERR_WAIT_TIMEOUT
    assert "grid barrier timed out" in N.last_error()
    a = D.voxel_problem_arrays(4, 4, 4, 0.25, young=1.0)
    P = D.StaticElasticProblem(a)
    b = P.assemble()
    assert P.factor()
    x = np.zeros_like(b)
    hist = D.Solve_PCG(b.copy(), x, 1e-10, 1000, P.K, P.ilu)
    assert hist[-1] < 1e-10 * hist[0]


def test_bounded_wait_times_out_and_context_survives(gpu):
    from delfem2_gb300 import _native as N
    st = N.load().dfm2g_debug_wait_timeout(50)
    assert st == N.ERR_WAIT_TIMEOUT
    # the context is still usable
    import delfem2_gb300 as D
    xyz, tet = D.MeshTet3D_VoxelGrid(1, 1, 1, 1.0)
    ind, psup = D.JArray_PSuP_MeshElem(tet, 4, 8)
    K = D.CMatrixSparse()
    K.Initialize(8, 3)
    K.SetPattern(ind, psup)
    K.set_values(None, np.tile(np.eye(3).ravel(), 8))
    y = np.zeros(24)
    K.MatVec(y, 1.0, np.arange(24.0), 0.0)
    assert np.array_equal(y, np.arange(24.0))


def test_torch_device_tensors(case):
    import torch
    import delfem2_gb300 as D
    name, s, P, b = case
    bt = torch.from_numpy(s["b"]).cuda()
    r = bt.clone()
    x = torch.zeros_like(r)
    hist = D.Solve_PCG(r, x, 1e-10, 1000, P.K, P.ilu)
    xh = np.zeros_like(s["b"])
    hist_h = D.Solve_PCG(s["b"].copy(), xh, 1e-10, 1000, P.K, P.ilu)
    assert len(hist) == len(hist_h)
    assert rel_err(x.cpu().numpy(), xh) < 1e-14
