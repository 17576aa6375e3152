"""ctypes binding of libdfm2g.so (the C ABI declared in include/dfm2g.h).

There is no fallback: if the library has not been built, every entry point
raises. Build it with ``python -m delfem2_gb300.build`` (or
``__graft_entry__.build()``).
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libdfm2g.so")

OK = 0
ERR_ARG = 1
ERR_CUDA = 2
ERR_MISSING_SLOT = 3
ERR_SINGULAR_PIVOT = 4
ERR_NOT_CONVERGED = 5
ERR_WAIT_TIMEOUT = 6
ERR_PATTERN = 7
ERR_UNSUPPORTED = 8
ERR_STATE = 9
ERR_NONFINITE = 10
ERR_HOST = 11

MEM_HOST = 0
MEM_DEVICE = 1
F64 = 0
F32 = 1
SWEEP_SYNCFREE = 0
SWEEP_LEVELS = 1
SWEEP_GROUPS = 2
SWEEP_BLOCK = 3
SWEEP_PARTS = 4
SWEEP_CHAINS = 5
SWEEP_TILES = 6
SWEEP_AUTO = 7
SWEEP_CLUSTER = 8


class SolveStats(C.Structure):
    _fields_ = [("iterations", C.c_uint), ("outer", C.c_uint), ("rel_residual", C.c_double),
                ("ms", C.c_double)]


class Dfm2gError(RuntimeError):
    def __init__(self, status: int, where: str, message: str):
        super().__init__(f"{where}: status {status}: {message}")
        self.status = status


_vp = C.c_void_p
_u = C.c_uint
_sz = C.c_size_t
_d = C.c_double
_i = C.c_int
_pu = C.POINTER(C.c_uint)
_psz = C.POINTER(C.c_size_t)
_pi = C.POINTER(C.c_int)
_pstats = C.POINTER(SolveStats)

# name -> argtypes (all return int status unless listed in _RESTYPE)
SIGNATURES = {
    "dfm2g_version": [],
    "dfm2g_status_string": [_i],
    "dfm2g_last_error": [],
    "dfm2g_set_stream": [_vp],
    "dfm2g_synchronize": [],
    "dfm2g_mesh_tet_voxel_grid": [_u, _u, _u, _d, _vp, _vp],
    "dfm2g_psup_count": [_vp, _sz, _u, _sz, _vp, _psz],
    "dfm2g_psup_fill": [_vp, _sz, _u, _sz, _vp, _vp],
    "dfm2g_bsr_create": [C.POINTER(_vp), _u, _u],
    "dfm2g_bsr_destroy": [_vp],
    "dfm2g_bsr_set_pattern": [_vp, _vp, _sz, _vp, _sz],
    "dfm2g_bsr_ndim": [_vp, _pu],
    "dfm2g_bsr_info": [_vp, _pu, _psz],
    "dfm2g_bsr_set_zero": [_vp],
    "dfm2g_bsr_set_values": [_vp, _vp, _vp, _i],
    "dfm2g_bsr_get_values": [_vp, _vp, _vp, _i],
    "dfm2g_bsr_set_fixed_bc": [_vp, _vp, _i],
    "dfm2g_bsr_add_dia": [_vp, _d],
    "dfm2g_bsr_matvec": [_vp, _i, _vp, _d, _vp, _d, _i],
    "dfm2g_bsr_update_f32": [_vp],
    "dfm2g_bsr_merge": [_vp, _u, _u, _vp, _vp, _i],
    "dfm2g_vec_zero_bc": [_vp, _vp, _sz, _i],
    "dfm2g_ilu_create": [C.POINTER(_vp)],
    "dfm2g_ilu_destroy": [_vp],
    "dfm2g_ilu_set_pattern0": [_vp, _vp],
    "dfm2g_ilu_set_pattern_k": [_vp, _vp, _i],
    "dfm2g_ilu_copy_value": [_vp, _vp],
    "dfm2g_ilu_decompose": [_vp, _pi],
    "dfm2g_ilu_forward": [_vp, _i, _vp, _i],
    "dfm2g_ilu_backward": [_vp, _i, _vp, _i],
    "dfm2g_ilu_solve_precond": [_vp, _i, _vp, _i],
    "dfm2g_ilu_solve_precond_noalloc": [_vp, _i, _vp],
    "dfm2g_ilu_set_sweep_mode": [_vp, _i],
    "dfm2g_ilu_get_sweep_mode": [_vp, _pi],
    "dfm2g_ilu_last_schedule": [_vp, _i, _i, _pi],
    "dfm2g_ilu_get_pattern": [_vp, _vp, _vp],
    "dfm2g_ilu_info": [_vp, _pu, _psz],
    "dfm2g_ilu_get_row_start": [_vp, _vp],
    "dfm2g_ilu_get_values": [_vp, _vp, _vp, _i],
    "dfm2g_ilu_get_levels": [_vp, _i, _vp, _vp, _vp, _pu],
    "dfm2g_chain_partition": [_u, _vp, _vp, _vp, _vp, _i, _vp, _pu, _pu],
    "dfm2g_tile_partition": [_u, _vp, _vp, _vp, _vp, _i, _u, _u, _vp, _vp, _pu, _pu],
    "dfm2g_solve_pcg": [_vp, _vp, _vp, _vp, _d, _u, _vp, _u, _pu, _i, _pstats],
    "dfm2g_solve_cg": [_vp, _vp, _vp, _d, _u, _vp, _u, _pu, _i, _pstats],
    "dfm2g_solve_pbicgstab": [_vp, _vp, _vp, _vp, _d, _u, _vp, _u, _pu, _i, _pstats],
    "dfm2g_solve_pcg_mixed": [_vp, _vp, _vp, _vp, _d, _d, _u, _u, _i, _pstats],
    "dfm2g_solve_pcg_mixed_reliable": [_vp, _vp, _vp, _vp, _d, _d, _u, _i, _pstats],
    "dfm2g_tetmesh_create": [C.POINTER(_vp), _vp, _vp, _sz, _vp, _sz],
    "dfm2g_tetmesh_destroy": [_vp],
    "dfm2g_tetmesh_info": [_vp, _pu, _psz],
    "dfm2g_tetmesh_assemble_linear": [_vp, _vp, _vp, _d, _d, _vp, _vp, _vp, _i],
    "dfm2g_tetmesh_dLdE": [_vp, _vp, _d, _vp, _vp, _vp, _i],
    "dfm2g_tetmesh_assemble_poisson": [_vp, _vp, _d, _d, _vp, _vp, _i],
    "dfm2g_tetmesh_assemble_beuler": [_vp, _vp, _d, _d, _d, _vp, _d, _vp, _vp, _vp, _vp, _i],
    "dfm2g_tetmesh_assemble_newmark": [_vp, _vp, _d, _d, _d, _vp, _d, _d, _d, _vp, _vp, _vp, _vp, _i],
    "dfm2g_hexmesh_create": [C.POINTER(_vp), _vp, _vp, _sz, _vp, _sz],
    "dfm2g_hexmesh_destroy": [_vp],
    "dfm2g_hexmesh_assemble_linear": [_vp, _vp, _d, _d, _d, _vp, _vp, _vp, _i],
    "dfm2g_trimesh2_create": [C.POINTER(_vp), _vp, _vp, _sz, _vp, _sz],
    "dfm2g_trimesh2_destroy": [_vp],
    "dfm2g_trimesh2_assemble_poisson": [_vp, _vp, _d, _d, _vp, _vp, _i],
    "dfm2g_trimesh2_assemble_solid_linear": [_vp, _vp, _d, _d, _d, _d, _d, _vp, _vp, _i],
    "dfm2g_cloth_create": [C.POINTER(_vp), _vp, _vp, _sz, _vp, _sz, _vp, _sz],
    "dfm2g_cloth_destroy": [_vp],
    "dfm2g_cloth_info": [_vp, _pu, _pu],
    "dfm2g_cloth_merge": [_vp, _vp, _vp, _vp, _d, _d, _vp, C.POINTER(C.c_double), _i],
    "dfm2g_cloth_step": [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _d, _d, _vp, _d, _d, _d, _u, _i, _pstats, _i],
    "dfm2g_cloth_adjoint_terms": [_vp, _vp, _vp, _d, _d, _vp, _vp, _vp, _vp, _i],
    "dfm2g_cloth_rollout": [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _d, _d, _vp, _d, _d, _d, _u, _i, _u, _u, _pstats,
                            _i],
    "dfm2g_cloth_rollout_adjoint": [_vp, _vp, _vp, _vp, _vp, _vp, _pstats, _i],
    "dfm2g_dev_alloc": [C.POINTER(_vp), _sz],
    "dfm2g_dev_free": [_vp],
    "dfm2g_dev_copy": [_vp, _vp, _sz, _i],
    "dfm2g_vec_dot": [_vp, _vp, _sz, C.POINTER(C.c_double), _i],
    "dfm2g_vec_axpy": [_vp, _d, _vp, _sz, _i],
    "dfm2g_vec_scale_add": [_vp, _d, _vp, _sz, _i],
    "dfm2g_vec_set_zero": [_vp, _sz, _i],
    "dfm2g_profile_enable": [_i],
    "dfm2g_profile_reset": [],
    "dfm2g_profile_read": [_i, _pu, C.POINTER(C.c_double)],
    "dfm2g_launch_count": [C.POINTER(C.c_ulonglong)],
    "dfm2g_alloc_count": [C.POINTER(C.c_ulonglong)],
    "dfm2g_debug_wait_timeout": [_u],
    "dfm2g_debug_grid_barrier": [_u, _i],
    "dfm2g_debug_host_failure": [_i],
}

PROF_KINDS = ["spmv", "update", "fill", "fwd", "bwd", "dot", "pupdate", "outer"]
_RESTYPE = {"dfm2g_status_string": C.c_char_p, "dfm2g_last_error": C.c_char_p}

_LIB = None


def load() -> C.CDLL:
    """Load libdfm2g.so; raises if it is missing (no CPU fallback exists)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is not built; run `python -m delfem2_gb300.build` first "
                           "(the CUDA library is the only implementation)")
    lib = C.CDLL(LIB_PATH)
    for name, argtypes in SIGNATURES.items():
        f = getattr(lib, name)
        f.argtypes = argtypes
        f.restype = _RESTYPE.get(name, C.c_int)
    _LIB = lib
    return lib


def last_error() -> str:
    return load().dfm2g_last_error().decode(errors="replace")


def check(status: int, where: str, allow=()) -> int:
    if status != OK and status not in allow:
        raise Dfm2gError(status, where, last_error())
    return status


def call(name: str, *args, allow=()) -> int:
    return check(getattr(load(), name)(*args), name, allow)
