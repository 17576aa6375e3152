"""Static linear-elasticity problems on voxel tet meshes (the callers of the path).

This is the sequence of a DelFEM2 application such as
examples_oldgl_glfw/618_Fem3Tet/main.cpp:234-319: mesh -> JArray_PSuP_MeshElem
-> CMatrixSparse::Initialize/SetPattern -> CPreconditionerILU::SetPattern0 ->
setZero -> per-element assembly -> SetFixedBC / setRHS_Zero -> CopyValue ->
Decompose -> Solve_PCG, run on the device through libdfm2g.
"""
from __future__ import annotations

import numpy as np

from .fem import TetMesh
from .ls import (CMatrixSparse, CPreconditionerILU, JArray_PSuP_MeshElem, MeshTet3D_VoxelGrid, Solve_PCG,
                 Solve_PCG_Mixed, setRHS_Zero)


def young_log_uniform(ntet: int, lo: float, hi: float, seed: int) -> np.ndarray:
    """Per-tet Young's modulus, log-uniform in [lo, hi] (numpy PCG64, seeded)."""
    rng = np.random.default_rng(seed)
    return np.exp(rng.uniform(np.log(lo), np.log(hi), ntet))


def voxel_problem_arrays(nx: int, ny: int, nz: int, h: float, young=None, seed: int = 0,
                         e_range=(0.1, 10.0)):
    """Mesh, pattern, z=0 clamp flags and per-tet E for an nx x ny x nz voxel block of spacing h."""
    xyz, tet = MeshTet3D_VoxelGrid(nx, ny, nz, h)
    np_ = xyz.size // 3
    ind, psup = JArray_PSuP_MeshElem(tet, 4, np_)
    bc = np.zeros(np_ * 3, np.int32)
    bc[np.repeat(xyz[2::3] == 0.0, 3)] = 1
    ntet = tet.size // 4
    if young is None:
        young = young_log_uniform(ntet, e_range[0], e_range[1], seed)
    elif np.isscalar(young):
        young = np.full(ntet, float(young))
    return dict(xyz=xyz, tet=tet, psup_ind=ind, psup=psup, bc=bc, young=np.asarray(young, np.float64),
                np=np_, ntet=ntet)


class StaticElasticProblem:
    """K u = f for a clamped voxel block, assembled, factored and solved on the GPU."""

    def __init__(self, arrays: dict, nu: float = 0.3, rho: float = 1.0, g=(0.0, 0.0, -1e-3)):
        self.a = arrays
        self.nu, self.rho, self.g = nu, rho, tuple(g)
        self.K = CMatrixSparse()
        self.K.Initialize(arrays["np"], 3, True)
        self.K.SetPattern(arrays["psup_ind"], arrays["psup"])
        self.mesh = TetMesh(self.K, arrays["xyz"], arrays["tet"])
        self.ilu = CPreconditionerILU()
        self.ilu.SetPattern0(self.K)
        self.ndof = arrays["np"] * 3

    def assemble(self, young=None, b=None):
        """K, b for the given per-tet E (default: the arrays' E); returns b (numpy or torch)."""
        young = self.a["young"] if young is None else young
        if b is None:
            b = np.zeros(self.ndof, np.float64)
        else:
            b.fill_(0.0) if hasattr(b, "fill_") else b.fill(0.0)
        on_device = hasattr(b, "is_cuda") and b.is_cuda
        if on_device and isinstance(young, np.ndarray):
            import torch
            key = (young.ctypes.data, young.size, str(b.device))
            if getattr(self, "_young_key", None) != key:
                self._young_dev = torch.from_numpy(young).to(b.device)
                self._young_key = key
            young = self._young_dev
        self.K.setZero()
        self.mesh.assemble_linear(young, self.nu, self.rho, self.g, b)
        self.K.SetFixedBC(self.a["bc"])
        bc = self.a["bc"]
        if hasattr(b, "is_cuda") and b.is_cuda:
            import torch
            bc = torch.from_numpy(bc).to(b.device)
        setRHS_Zero(b, bc)
        return b

    def assemble_stiffness(self, young):
        """K(E) with the clamp applied (no load); young: numpy or CUDA tensor of per-tet E."""
        import torch
        dev = young.device if hasattr(young, "device") else None
        if dev is not None and dev.type == "cuda":
            scratch = getattr(self, "_scratch_b", None)
            if scratch is None or scratch.device != dev:
                self._scratch_b = torch.zeros(self.ndof, dtype=torch.float64, device=dev)
            b = self._scratch_b
            b.zero_()
        else:
            b = np.zeros(self.ndof)
        self.K.setZero()
        self.mesh.assemble_linear(young, self.nu, 0.0, (0.0, 0.0, 0.0), b)
        self.K.SetFixedBC(self.a["bc"])

    def free_mask(self, like):
        """1 on free DOFs, 0 on clamped ones, as a tensor/array like `like`."""
        m = (self.a["bc"] == 0).astype(np.float64)
        if hasattr(like, "device"):
            import torch
            return torch.from_numpy(m).to(like.device)
        return m

    def factor(self) -> bool:
        self.ilu.CopyValue(self.K)
        return self.ilu.Decompose()

    def solve_fp64(self, b, tol=1e-10, max_iter=1000, stats=None):
        """Solve_PCG on a copy of b; returns (x, history)."""
        r = b.clone() if hasattr(b, "clone") else b.copy()
        x = r.new_zeros(r.shape) if hasattr(r, "new_zeros") else np.zeros_like(r)
        hist = Solve_PCG(r, x, tol, max_iter, self.K, self.ilu, stats)
        return x, hist

    def solve_mixed(self, b, tol=1e-10, inner_tol=1e-4, max_iter=100000, method="restart"):
        x = b.new_zeros(b.shape) if hasattr(b, "new_zeros") else np.zeros_like(b)
        st = Solve_PCG_Mixed(b, x, tol, self.K, self.ilu, inner_tol=inner_tol, max_iter=max_iter, method=method)
        return x, st
