"""dfm2g_ilu_solve_precond_noalloc: the SolvePrecond entry point for callers
that cannot allocate device memory while they solve (an application that
reserves all GPU memory up front, or a frame loop that cannot afford the
device-wide synchronisation of cudaMalloc/cudaFree).

Called through the C ABI, in every sweep schedule and in FP64 and FP32, and
checked three ways on two calls in a row:
- against the oracle's ForwardSubstitution + BackwardSubstitution (the
  reference's ILU(0) sweeps) on the same vector, within the sweep tolerance
  of the other GPU tests (1e-10 FP64, 1e-4 FP32 against the FP64 oracle);
- against the ordinary dfm2g_ilu_solve_precond on the same vector;
- through the library's allocation counter (dfm2g_alloc_count), which must
  not move across a no-alloc call, and through the device's free memory.
A fresh handle is also swept before any ordinary sweep has built a
schedule's data: the schedules that build on first use (tiles, chains,
block) then sweep sync-free, still without allocating.
This file is named so that pytest collects it last."""
import ctypes as C

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

SWEEP_TOL_F64 = 1e-10  # as tests/test_gpu_parity.py::test_sweeps_match_oracle
SWEEP_TOL_F32 = 1e-4   # FP32 sweeps against the FP64 oracle, as there
MODES = [0, 1, 2, 3, 4, 5, 6, 7, 8]  # sync-free, levels, groups, block, parts, chains, tiles, auto, cluster
NU, RHO, G = 0.3, 1.0, (0.0, 0.0, -1e-3)


def _system(port, n, seed):
    """The oracle's factored ILU(0) of an n^3-voxel elastic system and the
    same system on the GPU (assembled and factored there)."""
    import delfem2_gb300 as D
    xyz, tet = port.voxel_tet_mesh(n, n, n, 1.0 / n)
    np_ = xyz.size // 3
    young = np.exp(np.random.default_rng(seed).uniform(np.log(0.1), np.log(10), tet.size // 4))
    ind, psup = port.psup(tet, 4, np_)
    vc, vd, b = np.zeros(psup.size * 9), np.zeros(np_ * 9), np.zeros(np_ * 3)
    assert port.assemble_tet_linear(ind, psup, vc, vd, b, xyz, tet, young, NU, RHO, G) == 0
    bc = np.zeros(np_ * 3, np.int32)
    bc[np.repeat(xyz[2::3] == 0.0, 3)] = 1
    port.set_fixed_bc(ind, psup, vc, vd, bc)
    col, dia = port.ilu_pattern0(ind, psup)
    ivc, ivd = port.ilu_copy_value(ind, col, psup, vc, vd)
    assert port.ilu_decompose(ind, col, dia, ivc, ivd)[0] == 0
    arrays = dict(xyz=xyz, tet=tet, psup_ind=ind, psup=psup, bc=bc, young=young, np=np_, ntet=tet.size // 4)
    P = D.StaticElasticProblem(arrays, nu=NU, rho=RHO, g=G)
    P.assemble()
    assert P.factor()
    oracle = dict(ind=ind, col=col, dia=dia, ivc=ivc, ivd=ivd)
    return P, oracle


def _oracle_precond(port, o, v):
    f = port.ilu_forward(o["ind"], o["col"], o["dia"], o["ivc"], o["ivd"], v)
    return port.ilu_backward(o["ind"], o["col"], o["dia"], o["ivc"], f)


def _allocs():
    from delfem2_gb300 import _native as N
    c = C.c_ulonglong(0)
    N.call("dfm2g_alloc_count", C.byref(c))
    return c.value


def _existing(P, prec, v):
    from delfem2_gb300 import _native as N
    N.call("dfm2g_ilu_solve_precond", P.ilu._h, prec, C.c_void_p(v.data_ptr()), N.MEM_DEVICE)


def _noalloc(P, prec, v):
    import torch
    from delfem2_gb300 import _native as N
    N.load().dfm2g_set_stream(C.c_void_p(torch.cuda.current_stream().cuda_stream))
    return N.load().dfm2g_ilu_solve_precond_noalloc(P.ilu._h, prec, C.c_void_p(v.data_ptr()))


def _set_mode(P, mode):
    """Selects a schedule; False when the pattern does not support it."""
    from delfem2_gb300 import _native as N
    return N.load().dfm2g_ilu_set_sweep_mode(P.ilu._h, mode) == N.OK


@pytest.fixture(scope="module")
def problem(gpu, port):
    return _system(port, 16, seed=0)


def test_noalloc_fresh_handle_before_any_sweep(gpu, port):
    """No ordinary sweep has run on this handle, so no schedule has built its
    data: every schedule sweeps without allocating (tiles, chains and block
    fall back to sync-free) and matches the oracle."""
    import torch
    from delfem2_gb300 import _native as N
    P, o = _system(port, 8, seed=1)
    rng = np.random.default_rng(2)
    torch.cuda.synchronize()
    for mode in MODES:
        if not _set_mode(P, mode):
            continue
        for call in range(2):
            v = rng.standard_normal(P.ndof)
            out = torch.tensor(v, device="cuda")
            a0, free0 = _allocs(), torch.cuda.mem_get_info()[0]
            assert _noalloc(P, N.F64, out) == N.OK, N.last_error()
            torch.cuda.synchronize()
            assert _allocs() == a0, f"mode {mode}: the no-alloc call allocated"
            assert torch.cuda.mem_get_info()[0] == free0
            assert rel_err(out.cpu().numpy(), _oracle_precond(port, o, v)) < SWEEP_TOL_F64, (mode, call)


@pytest.mark.parametrize("prec", ["f64", "f32"])
@pytest.mark.parametrize("mode", MODES)
def test_noalloc_matches_oracle_and_solve_precond(problem, port, mode, prec):
    """After an ordinary sweep has built the schedule's data (and, for FP32,
    the FP32 factors), two no-alloc calls in a row match the oracle and the
    ordinary entry point and leave the allocation count and free memory as
    they were."""
    import torch
    from delfem2_gb300 import _native as N
    P, o = problem
    prior = P.ilu.sweep_mode()
    if not _set_mode(P, mode):
        pytest.skip(f"schedule {mode} unavailable for this pattern")
    try:
        p = N.F64 if prec == "f64" else N.F32
        dt = torch.float64 if prec == "f64" else torch.float32
        tol = SWEEP_TOL_F64 if prec == "f64" else SWEEP_TOL_F32
        rng = np.random.default_rng(10 + mode)
        warm = torch.tensor(rng.standard_normal(P.ndof), dtype=dt, device="cuda")
        _existing(P, p, warm)  # builds what this schedule needs (this call may allocate)
        torch.cuda.synchronize()
        for call in range(2):
            v = rng.standard_normal(P.ndof)
            ref = torch.tensor(v, dtype=dt, device="cuda")
            out = ref.clone()
            _existing(P, p, ref)
            torch.cuda.synchronize()
            a0, free0 = _allocs(), torch.cuda.mem_get_info()[0]
            assert _noalloc(P, p, out) == N.OK, N.last_error()
            torch.cuda.synchronize()
            assert _allocs() == a0, f"mode {mode} {prec}: the no-alloc call allocated"
            assert torch.cuda.mem_get_info()[0] == free0
            z = out.double().cpu().numpy()
            assert rel_err(z, _oracle_precond(port, o, v)) < tol, (mode, prec, call)
            assert rel_err(z, ref.double().cpu().numpy()) < tol, (mode, prec, call)
    finally:
        P.ilu.set_sweep_mode(prior)


def test_noalloc_f32_needs_f32_factors(gpu, port):
    """Making the FP32 factors allocates, so the no-alloc entry point refuses
    FP32 until an ordinary FP32 call has made them."""
    import torch
    from delfem2_gb300 import _native as N
    P, _ = _system(port, 4, seed=3)
    v = torch.ones(P.ndof, dtype=torch.float32, device="cuda")
    a0 = _allocs()
    assert _noalloc(P, N.F32, v) == N.ERR_STATE
    assert "FP32 factors" in N.last_error()
    assert _allocs() == a0
    assert torch.equal(v, torch.ones_like(v))


def test_noalloc_rejects_systems_beyond_its_scratch(gpu):
    import torch
    import delfem2_gb300 as D
    from delfem2_gb300 import _native as N
    a = D.voxel_problem_arrays(70, 70, 70, 1 / 70, young=1.0)  # 357,911 blocks -> 1,073,733 unknowns
    P = D.StaticElasticProblem(a)
    P.assemble(b=torch.zeros(a["np"] * 3, dtype=torch.float64, device="cuda"))
    assert P.factor()
    v = torch.ones(P.ndof, dtype=torch.float64, device="cuda")
    a0 = _allocs()
    st = _noalloc(P, N.F64, v)
    assert st == N.ERR_ARG
    assert "exceed the fixed scratch" in N.last_error()
    assert _allocs() == a0
    assert torch.equal(v, torch.ones_like(v))  # untouched
