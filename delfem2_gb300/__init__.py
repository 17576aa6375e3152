"""delfem2_gb300: GB300-native (sm_103a) drop-in for DelFEM2's implicit-FEM
linear-solve path (3x3 block-CSR assembly -> ILU(0) -> Solve_PCG).

The compute is libdfm2g.so (CUDA C ABI, include/dfm2g.h); this package is the
Python mirror of the reference's interface over it. There is no CPU fallback.
"""
from . import _native  # noqa: F401
from ._native import Dfm2gError, SolveStats  # noqa: F401
from .fem import HexMesh, TetMesh, TriMesh2, lame  # noqa: F401
from .ls import (CMatrixSparse, CPreconditionerILU, JArray_PSuP_MeshElem, Merge,  # noqa: F401
                 MeshTet3D_VoxelGrid, Solve_CG, Solve_PBiCGStab, Solve_PCG, Solve_PCG_Mixed, setRHS_Zero)
from .problem import StaticElasticProblem, voxel_problem_arrays  # noqa: F401
