"""C-ABI library: loads without a GPU, exports every entry point include/dfm2g.h
declares, and its host-only helpers (mesh, pattern) are bit-exact vs the oracle."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "dfm2g.h")).read()
    return sorted(set(re.findall(r"DFM2G_API\s+[\w\s\*]+?\b(dfm2g_\w+)\s*\(", src)))


def test_header_declares_the_reference_surface():
    names = declared_symbols()
    for must in ("dfm2g_bsr_set_pattern", "dfm2g_bsr_set_zero", "dfm2g_bsr_merge", "dfm2g_bsr_matvec",
                 "dfm2g_bsr_set_fixed_bc", "dfm2g_ilu_set_pattern0", "dfm2g_ilu_copy_value",
                 "dfm2g_ilu_decompose", "dfm2g_ilu_solve_precond", "dfm2g_solve_pcg", "dfm2g_solve_pcg_mixed"):
        assert must in names


def test_library_exports_every_declared_symbol(built_lib):
    from delfem2_gb300 import _native
    for name in declared_symbols():
        assert hasattr(built_lib, name), name
        assert name in _native.SIGNATURES, f"{name} has no ctypes signature"


def test_status_strings(built_lib):
    from delfem2_gb300 import _native as N
    assert built_lib.dfm2g_version() >= 100
    for s in range(0, 12):
        assert built_lib.dfm2g_status_string(s)
    assert b"singular" in built_lib.dfm2g_status_string(N.ERR_SINGULAR_PIVOT)
    assert b"host" in built_lib.dfm2g_status_string(N.ERR_HOST)


@pytest.mark.parametrize("kind,msg", [(0, b"out of host memory"), (1, b"debug exception"), (2, b"unknown")])
def test_no_exception_crosses_the_c_abi(built_lib, kind, msg):
    """A C++ exception inside an entry point becomes DFM2G_ERR_HOST with a
    message (every entry point is a function-try-block); no device work."""
    from delfem2_gb300 import _native as N
    assert built_lib.dfm2g_debug_host_failure(kind) == N.ERR_HOST
    assert msg in built_lib.dfm2g_last_error()


@pytest.mark.parametrize("dims", [(1, 1, 1), (3, 2, 4), (16, 16, 16)])
def test_host_mesh_and_pattern_bit_exact(built_lib, port, dims):
    import delfem2_gb300 as D
    nx, ny, nz = dims
    xyz, tet = D.MeshTet3D_VoxelGrid(nx, ny, nz, 1.0 / nx)
    xo, to = port.voxel_tet_mesh(nx, ny, nz, 1.0 / nx)
    assert np.array_equal(tet, to) and np.array_equal(xyz, xo)
    ind, psup = D.JArray_PSuP_MeshElem(tet, 4, xyz.size // 3)
    io, po = port.psup(to, 4, xo.size // 3)
    assert np.array_equal(ind, io) and np.array_equal(psup, po)


def test_pattern_of_triangles_and_quads(built_lib, port):
    import delfem2_gb300 as D
    rng = np.random.default_rng(0)
    for nno in (2, 3, 4):
        elem = rng.integers(0, 50, size=(40, nno)).astype(np.uint32)
        ind, psup = D.JArray_PSuP_MeshElem(elem, nno, 50)
        io, po = port.psup(elem, nno, 50)
        assert np.array_equal(ind, io) and np.array_equal(psup, po)


def test_bad_arguments_fail_before_any_device_work(built_lib):
    import delfem2_gb300 as D
    with pytest.raises(D.Dfm2gError):
        D.JArray_PSuP_MeshElem(np.array([0, 7], np.uint32), 2, 3)  # node id out of range
    with pytest.raises(TypeError):
        from delfem2_gb300.ls import _vec
        _vec(np.zeros(3, np.float32), np.float64, True)
    from delfem2_gb300 import _native as N
    m = C.c_int(5)
    assert built_lib.dfm2g_ilu_last_schedule(None, N.F32, 0, C.byref(m)) == N.ERR_ARG and m.value == 5
    assert b"null ILU handle" in built_lib.dfm2g_last_error()
