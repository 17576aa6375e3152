"""Python mirror of DelFEM2's sparse linear-solve API, backed by libdfm2g.

Names, argument meaning and error behaviour follow the reference:
  CMatrixSparse      include/delfem2/ls_block_sparse.h:24-204
  Merge              include/delfem2/ls_block_sparse.h:260-310
  CPreconditionerILU include/delfem2/ls_ilu_block_sparse.h:21-60
  Solve_PCG/Solve_CG include/delfem2/lsitrsol.h:35-148
Vectors may be numpy arrays (host memory, copied in/out per call) or CUDA
torch tensors (device memory, used in place on torch's current stream).
Vectors that the reference overwrites (MatVec's y, SolvePrecond's vec,
Solve_PCG's r and x) are overwritten in place here too.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N


def _is_torch(a) -> bool:
    return type(a).__module__.startswith("torch")


def _vec(a, dtype, writable: bool):
    """(pointer, mem flag, keepalive) for a numpy array or torch tensor."""
    if a is None:
        return None, N.MEM_HOST, None
    if _is_torch(a):
        import torch
        tdt = {np.float64: torch.float64, np.float32: torch.float32, np.int32: torch.int32,
               np.uint32: torch.int32}[np.dtype(dtype).type]
        if a.dtype != tdt and not (np.dtype(dtype) == np.uint32 and a.dtype == torch.int32):
            raise TypeError(f"expected a {tdt} tensor, got {a.dtype}")
        if not a.is_contiguous():
            raise ValueError("tensor must be contiguous")
        if a.is_cuda:
            N.load().dfm2g_set_stream(C.c_void_p(torch.cuda.current_stream(a.device).cuda_stream))
            return C.c_void_p(a.data_ptr()), N.MEM_DEVICE, a
        a = a.numpy()
    if not isinstance(a, np.ndarray):
        if writable:
            raise TypeError("output vectors must be numpy arrays or torch tensors")
        a = np.asarray(a)
    if a.dtype != np.dtype(dtype):
        if writable:
            raise TypeError(f"expected dtype {np.dtype(dtype)}, got {a.dtype}")
        a = a.astype(dtype)
    if not a.flags["C_CONTIGUOUS"]:
        if writable:
            raise ValueError("array must be C-contiguous")
        a = np.ascontiguousarray(a)
    return C.c_void_p(a.ctypes.data), N.MEM_HOST, a


def _same_mem(*flags):
    fl = {f for f in flags if f is not None}
    if len(fl) > 1:
        raise ValueError("mixing host and device vectors in one call is not supported")
    return fl.pop() if fl else N.MEM_HOST


# ---------------------------------------------------------------------------
def MeshTet3D_VoxelGrid(nx: int, ny: int, nz: int, scale: float = 1.0):
    """Lattice mesh of (nx,ny,nz) voxels, 6 tets each (gridvoxel.cpp:194-271)."""
    np_ = (nx + 1) * (ny + 1) * (nz + 1)
    xyz = np.zeros(np_ * 3, np.float64)
    tet = np.zeros(nx * ny * nz * 24, np.uint32)
    N.call("dfm2g_mesh_tet_voxel_grid", nx, ny, nz, scale, xyz.ctypes.data, tet.ctypes.data)
    return xyz, tet


def JArray_PSuP_MeshElem(elem, nnoel: int, np_: int):
    """Node adjacency without self, rows sorted (msh_topology_uniform.cpp:301-316 + JArray_Sort)."""
    elem = np.ascontiguousarray(elem, np.uint32)
    ind = np.zeros(np_ + 1, np.uint32)
    n = C.c_size_t(0)
    N.call("dfm2g_psup_count", elem.ctypes.data, elem.size // nnoel, nnoel, np_, ind.ctypes.data, C.byref(n))
    psup = np.zeros(max(n.value, 1), np.uint32)
    N.call("dfm2g_psup_fill", elem.ctypes.data, elem.size // nnoel, nnoel, np_, ind.ctypes.data, psup.ctypes.data)
    return ind, psup[: n.value]


# ---------------------------------------------------------------------------
class CMatrixSparse:
    """Device-resident CMatrixSparse<double> with ndim x ndim blocks (ndim 1, 2 or 3)."""

    def __init__(self):
        self._h = None
        self.nrowblk = 0
        self.ndim = 0

    def Initialize(self, nblk: int, ndim: int, is_dia: bool = True):
        if not is_dia:
            raise ValueError("only matrices with a diagonal block array are supported")
        self._free()
        h = C.c_void_p()
        N.call("dfm2g_bsr_create", C.byref(h), nblk, ndim)
        self._h = h
        self.nrowblk = nblk
        self.ndim = ndim

    def SetPattern(self, colind, rowptr):
        """colind: row offsets (nblk+1); rowptr: column ids (reference naming)."""
        ci = np.ascontiguousarray(colind, np.uint32)
        rp = np.ascontiguousarray(rowptr, np.uint32)
        rp_buf = rp if rp.size else np.zeros(1, np.uint32)
        N.call("dfm2g_bsr_set_pattern", self._h, ci.ctypes.data, ci.size, rp_buf.ctypes.data, rp.size)

    def setZero(self):
        N.call("dfm2g_bsr_set_zero", self._h)

    @property
    def nnz(self) -> int:
        n = C.c_size_t()
        N.call("dfm2g_bsr_info", self._h, None, C.byref(n))
        return n.value

    def set_values(self, val_crs, val_dia):
        pc, mc, kc = _vec(val_crs, np.float64, False)
        pd, md, kd = _vec(val_dia, np.float64, False)
        N.call("dfm2g_bsr_set_values", self._h, pc, pd, _same_mem(mc if pc else None, md if pd else None))

    def get_values(self):
        bb = self.ndim * self.ndim
        vc = np.zeros(self.nnz * bb, np.float64)
        vd = np.zeros(self.nrowblk * bb, np.float64)
        N.call("dfm2g_bsr_get_values", self._h, vc.ctypes.data if vc.size else None, vd.ctypes.data, N.MEM_HOST)
        return vc, vd

    @property
    def val_crs(self):
        return self.get_values()[0]

    @property
    def val_dia(self):
        return self.get_values()[1]

    def SetFixedBC(self, bc):
        p, m, k = _vec(bc, np.int32, False)
        N.call("dfm2g_bsr_set_fixed_bc", self._h, p, m)

    def AddDia(self, eps: float):
        N.call("dfm2g_bsr_add_dia", self._h, float(eps))

    def MatVec(self, y, alpha: float, x, beta: float):
        """y = alpha*K*x + beta*y (in place); float32 vectors use the FP32 mirror."""
        dt = np.float32 if (getattr(y, "dtype", None) in (np.float32,) or str(getattr(y, "dtype", "")) == "torch.float32") else np.float64
        py, my, ky = _vec(y, dt, True)
        px, mx, kx = _vec(x, dt, False)
        N.call("dfm2g_bsr_matvec", self._h, N.F32 if dt == np.float32 else N.F64, py, float(alpha), px,
               float(beta), _same_mem(my, mx))

    def update_f32(self):
        N.call("dfm2g_bsr_update_f32", self._h)

    def _free(self):
        if self._h is not None:
            N.load().dfm2g_bsr_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self._free()
        except Exception:
            pass


def Merge(mat: CMatrixSparse, elem, emat):
    """Merge<nno,nno,ndim,ndim,double> for a batch: elem (nelem, nno), emat (nelem, nno, nno, ndim, ndim).

    Raises Dfm2gError(ERR_MISSING_SLOT) where the reference returns false."""
    elem = np.ascontiguousarray(elem, np.uint32)
    if elem.ndim == 1:
        elem = elem.reshape(1, -1)
    nelem, nno = elem.shape
    em = np.ascontiguousarray(emat, np.float64).reshape(nelem, nno, nno, mat.ndim, mat.ndim)
    N.call("dfm2g_bsr_merge", mat._h, nelem, nno, elem.ctypes.data, em.ctypes.data, N.MEM_HOST)


def setRHS_Zero(b, bc, iflag_nonzero: int = 0):
    """Zero b where bc != 0 (vecxitrsol.cpp:286-296 with iflag_nonzero = 0)."""
    if iflag_nonzero != 0:
        raise ValueError("only iflag_nonzero == 0 is supported")
    pb, mb, kb = _vec(b, np.float64, True)
    pf, mf, kf = _vec(bc, np.int32, False)
    N.call("dfm2g_vec_zero_bc", pb, pf, len(b), _same_mem(mb, mf))


# ---------------------------------------------------------------------------
class CPreconditionerILU:
    """Device-resident CPreconditionerILU<double> (ILU(0) or ILU(k); the matrix's block size)."""

    def __init__(self):
        h = C.c_void_p()
        N.call("dfm2g_ilu_create", C.byref(h))
        self._h = h
        self.nblk = 0
        self.ndim = 0

    def SetPattern0(self, mat: CMatrixSparse):
        N.call("dfm2g_ilu_set_pattern0", self._h, mat._h)
        self.nblk = mat.nrowblk
        self.ndim = mat.ndim
        self._nnz = mat.nnz

    def Initialize_ILUk(self, mat: CMatrixSparse, fill_level: int):
        """Level-of-fill ILU(k) pattern (ls_ilu_block_sparse.cpp:849-999); 0 is
        SetPattern0, -1 keeps every fill."""
        N.call("dfm2g_ilu_set_pattern_k", self._h, mat._h, int(fill_level))
        self.nblk = mat.nrowblk
        self.ndim = mat.ndim
        nnz = C.c_size_t(0)
        N.call("dfm2g_ilu_info", self._h, None, C.byref(nnz))
        self._nnz = nnz.value

    def CopyValue(self, mat: CMatrixSparse):
        N.call("dfm2g_ilu_copy_value", self._h, mat._h)

    def Decompose(self) -> bool:
        """Returns False when more than 10 pivots are singular (like the reference)."""
        ns = C.c_int(0)
        st = N.call("dfm2g_ilu_decompose", self._h, C.byref(ns), allow=(N.ERR_SINGULAR_PIVOT,))
        self.n_singular = ns.value
        return st == N.OK

    def _sweep(self, name, vec):
        dt = np.float32 if str(getattr(vec, "dtype", "")) in ("float32", "torch.float32") else np.float64
        p, m, k = _vec(vec, dt, True)
        N.call(name, self._h, N.F32 if dt == np.float32 else N.F64, p, m)

    def ForwardSubstitution(self, vec):
        self._sweep("dfm2g_ilu_forward", vec)

    def BackwardSubstitution(self, vec):
        self._sweep("dfm2g_ilu_backward", vec)

    def SolvePrecond(self, vec):
        self._sweep("dfm2g_ilu_solve_precond", vec)

    def set_sweep_mode(self, mode: int):
        N.call("dfm2g_ilu_set_sweep_mode", self._h, mode)

    def sweep_mode(self) -> int:
        m = C.c_int(0)
        N.call("dfm2g_ilu_get_sweep_mode", self._h, C.byref(m))
        return m.value

    def last_schedule(self, fp64: bool, backward: bool) -> int:
        """Schedule the last forward/backward sweep in FP64 or FP32 ran (-1: none yet)."""
        m = C.c_int(0)
        N.call("dfm2g_ilu_last_schedule", self._h, N.F64 if fp64 else N.F32, int(backward), C.byref(m))
        return m.value

    def row_start(self):
        """Row offsets of the ILU pattern (the matrix's for ILU(0))."""
        rs = np.zeros(self.nblk + 1, np.uint32)
        N.call("dfm2g_ilu_get_row_start", self._h, rs.ctypes.data)
        return rs

    def pattern(self):
        col = np.zeros(max(self._nnz, 1), np.uint32)
        dia = np.zeros(max(self.nblk, 1), np.uint32)
        N.call("dfm2g_ilu_get_pattern", self._h, col.ctypes.data, dia.ctypes.data)
        return col[: self._nnz], dia[: self.nblk]

    def values(self):
        bb = self.ndim * self.ndim
        vc = np.zeros(max(self._nnz * bb, 1), np.float64)
        vd = np.zeros(max(self.nblk * bb, 1), np.float64)
        N.call("dfm2g_ilu_get_values", self._h, vc.ctypes.data, vd.ctypes.data, N.MEM_HOST)
        return vc[: self._nnz * bb], vd[: self.nblk * bb]

    def levels(self, backward: bool = False):
        n = self.nblk
        level = np.zeros(max(n, 1), np.uint32)
        order = np.zeros(max(n, 1), np.uint32)
        lstart = np.zeros(n + 1, np.uint32)
        nl = C.c_uint(0)
        N.call("dfm2g_ilu_get_levels", self._h, int(backward), level.ctypes.data, order.ctypes.data,
               lstart.ctypes.data, C.byref(nl))
        return level[:n], order[:n], lstart[: nl.value + 1]

    def __del__(self):
        try:
            if self._h is not None:
                N.load().dfm2g_ilu_destroy(self._h)
                self._h = None
        except Exception:
            pass


# ---------------------------------------------------------------------------
def Solve_PCG(r_vec, x_vec, conv_ratio_tol: float, max_nitr: int, mat: CMatrixSparse,
              ilu: CPreconditionerILU, stats: N.SolveStats | None = None):
    """Solve_PCG (lsitrsol.h:80-148): returns the absolute residual history."""
    pr, mr, kr = _vec(r_vec, np.float64, True)
    px, mx, kx = _vec(x_vec, np.float64, True)
    cap = int(max_nitr) + 2
    hist = np.zeros(cap, np.float64)
    nh = C.c_uint(0)
    N.call("dfm2g_solve_pcg", mat._h, ilu._h, pr, px, float(conv_ratio_tol), int(max_nitr), hist.ctypes.data,
           cap, C.byref(nh), _same_mem(mr, mx), C.byref(stats) if stats is not None else None,
           allow=(N.ERR_NOT_CONVERGED,))
    return list(hist[: min(nh.value, cap)])


def Solve_CG(r_vec, u_vec, conv_ratio_tol: float, max_iteration: int, mat: CMatrixSparse,
             stats: N.SolveStats | None = None):
    """Solve_CG (lsitrsol.h:35-74): returns the relative residual history."""
    pr, mr, kr = _vec(r_vec, np.float64, True)
    px, mx, kx = _vec(u_vec, np.float64, True)
    cap = int(max_iteration) + 2
    hist = np.zeros(cap, np.float64)
    nh = C.c_uint(0)
    N.call("dfm2g_solve_cg", mat._h, pr, px, float(conv_ratio_tol), int(max_iteration), hist.ctypes.data, cap,
           C.byref(nh), _same_mem(mr, mx), C.byref(stats) if stats is not None else None,
           allow=(N.ERR_NOT_CONVERGED,))
    return list(hist[: min(nh.value, cap)])


def Solve_PBiCGStab(r_vec, x_vec, conv_ratio_tol: float, max_niter: int, mat: CMatrixSparse,
                    ilu: CPreconditionerILU, stats: N.SolveStats | None = None):
    """Solve_PBiCGStab (vecxitrsol.h:350-437): x = 0, r overwritten with the final
    residual; returns the RELATIVE residual history (one entry per iteration)."""
    pr, mr, kr = _vec(r_vec, np.float64, True)
    px, mx, kx = _vec(x_vec, np.float64, True)
    cap = int(max_niter) + 2
    hist = np.zeros(cap, np.float64)
    nh = C.c_uint(0)
    N.call("dfm2g_solve_pbicgstab", mat._h, ilu._h, pr, px, float(conv_ratio_tol), int(max_niter),
           hist.ctypes.data, cap, C.byref(nh), _same_mem(mr, mx), C.byref(stats) if stats is not None else None,
           allow=(N.ERR_NOT_CONVERGED,))
    return list(hist[: min(nh.value, cap)])


RELIABLE_REFRESH = 0.1  # |r| drop between FP64 residual refreshes of the reliable-update solver


def Solve_PCG_Mixed(b_vec, x_vec, tol: float, mat: CMatrixSparse, ilu: CPreconditionerILU,
                    inner_tol: float = 1e-4, max_iter: int = 100000, max_outer: int = 100,
                    allow_not_converged: bool = False, method: str = "restart",
                    refresh: float = RELIABLE_REFRESH) -> N.SolveStats:
    """FP32-inner / FP64-refinement PCG until |b - K x| / |b| < tol (b unchanged).

    method="reliable": one FP32 PCG whose residual is refreshed in FP64 each time
    it has dropped by the factor `refresh` (Krylov state kept; at 3.24M DOF a
    refresh every 0.1 keeps the FP32 iteration count at the FP64 one);
    method="restart": classic iterative refinement, a fresh FP32 PCG to
    `inner_tol` per FP64 step."""
    pb, mb, kb = _vec(b_vec, np.float64, False)
    px, mx, kx = _vec(x_vec, np.float64, True)
    st = N.SolveStats()
    allow = (N.ERR_NOT_CONVERGED,) if allow_not_converged else ()
    if method == "reliable":
        N.call("dfm2g_solve_pcg_mixed_reliable", mat._h, ilu._h, pb, px, float(tol), float(refresh),
               int(max_iter), _same_mem(mb, mx), C.byref(st), allow=allow)
    elif method == "restart":
        N.call("dfm2g_solve_pcg_mixed", mat._h, ilu._h, pb, px, float(tol), float(inner_tol), int(max_iter),
               int(max_outer), _same_mem(mb, mx), C.byref(st), allow=allow)
    else:
        raise ValueError(f"unknown method {method!r}")
    return st
