"""dfm2g_ilu_solve_precond_noalloc: the SolvePrecond entry point for callers
that cannot allocate device memory while they solve (an application that
reserves all GPU memory up front, or a frame loop that cannot afford the
device-wide synchronisation of cudaMalloc/cudaFree).

Called through the C ABI and checked against dfm2g_ilu_solve_precond on the
same vectors, on two calls in a row, within the sweep tolerance used by the
other GPU tests. This file is named so that pytest collects it last."""
import ctypes as C

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

SWEEP_TOL_F64 = 1e-10  # as tests/test_gpu_parity.py::test_sweeps_match_oracle
SWEEP_TOL_F32 = 1e-5


@pytest.fixture(scope="module")
def problem(gpu):
    import torch
    import delfem2_gb300 as D
    a = D.voxel_problem_arrays(16, 16, 16, 1 / 16, seed=0)
    P = D.StaticElasticProblem(a)
    P.assemble(b=torch.zeros(a["np"] * 3, dtype=torch.float64, device="cuda"))
    assert P.factor()
    return P


def _existing(P, prec, v):
    from delfem2_gb300 import _native as N
    N.call("dfm2g_ilu_solve_precond", P.ilu._h, prec, C.c_void_p(v.data_ptr()), N.MEM_DEVICE)


def _noalloc(P, prec, v):
    import torch
    from delfem2_gb300 import _native as N
    N.load().dfm2g_set_stream(C.c_void_p(torch.cuda.current_stream().cuda_stream))
    return N.load().dfm2g_ilu_solve_precond_noalloc(P.ilu._h, prec, C.c_void_p(v.data_ptr()))


def test_noalloc_matches_solve_precond_twice(problem):
    import torch
    from delfem2_gb300 import _native as N
    P = problem
    n = P.ndof
    gen = torch.Generator(device="cuda").manual_seed(0)
    free_after_first = None
    for call in range(2):
        v = torch.randn(n, dtype=torch.float64, device="cuda", generator=gen)
        ref, out = v.clone(), v.clone()
        _existing(P, N.F64, ref)
        assert _noalloc(P, N.F64, out) == N.OK, N.last_error()
        torch.cuda.synchronize()
        assert rel_err(out.cpu().numpy(), ref.cpu().numpy()) < SWEEP_TOL_F64
        if call == 0:
            free_after_first = torch.cuda.mem_get_info()[0]
        else:  # nothing was allocated by the second call
            assert torch.cuda.mem_get_info()[0] == free_after_first


def test_noalloc_f32_and_level_schedule(problem):
    import torch
    from delfem2_gb300 import _native as N
    P = problem
    n = P.ndof
    gen = torch.Generator(device="cuda").manual_seed(1)
    warm = torch.randn(n, dtype=torch.float32, device="cuda", generator=gen)
    _existing(P, N.F32, warm)  # creates the FP32 factors (this call may allocate)
    for call in range(2):
        v = torch.randn(n, dtype=torch.float32, device="cuda", generator=gen)
        ref, out = v.clone(), v.clone()
        _existing(P, N.F32, ref)
        assert _noalloc(P, N.F32, out) == N.OK, N.last_error()
        torch.cuda.synchronize()
        assert rel_err(out.cpu().numpy(), ref.cpu().numpy()) < SWEEP_TOL_F32
    P.ilu.set_sweep_mode(N.SWEEP_LEVELS)
    try:
        for call in range(2):
            v = torch.randn(n, dtype=torch.float64, device="cuda", generator=gen)
            ref, out = v.clone(), v.clone()
            _existing(P, N.F64, ref)
            assert _noalloc(P, N.F64, out) == N.OK, N.last_error()
            torch.cuda.synchronize()
            assert rel_err(out.cpu().numpy(), ref.cpu().numpy()) < SWEEP_TOL_F64
    finally:
        P.ilu.set_sweep_mode(N.SWEEP_SYNCFREE)


def test_noalloc_rejects_systems_beyond_its_scratch(gpu):
    import torch
    import delfem2_gb300 as D
    from delfem2_gb300 import _native as N
    a = D.voxel_problem_arrays(70, 70, 70, 1 / 70, young=1.0)  # 357,911 blocks -> 1,073,733 unknowns
    P = D.StaticElasticProblem(a)
    P.assemble(b=torch.zeros(a["np"] * 3, dtype=torch.float64, device="cuda"))
    assert P.factor()
    v = torch.ones(P.ndof, dtype=torch.float64, device="cuda")
    st = _noalloc(P, N.F64, v)
    assert st == N.ERR_ARG
    assert "exceed the fixed scratch" in N.last_error()
    assert torch.equal(v, torch.ones_like(v))  # untouched
