"""Implicit cloth on the device: the reference's cloth functions, plus the
time adjoint with checkpoint-and-recompute.

  SetClothShape_Square            include/delfem2/cloth_internal.h:331-403
  MergeLinSys_Cloth               include/delfem2/femcloth.h:48-114
  StepTime_InternalDynamicsILU    include/delfem2/cloth_internal.h:179-269
(element functions WdWddW_CST, fem_stvk.cpp:267-374, and WdWddW_Bend,
fem_quadratic_bending.cpp:49-107). Membrane moduli are per triangle:
(lambda, myu) = (E nu/((1+nu)(1-2nu)), E/(2(1+nu))). The contact terms of
the reference's step are not part of this path (its example passes a
no-contact object).

Vectors are numpy arrays (host, copied per call) or CUDA torch tensors
(device, used in place on torch's current stream).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .ls import CMatrixSparse, CPreconditionerILU, JArray_PSuP_MeshElem, _same_mem, _vec

PCG_F64 = 0    # Solve_PCG in FP64, as the reference
PCG_MIXED = 1  # FP32 PCG with FP64 reliable updates


def SetClothShape_Square(ndiv: int, cloth_size: float = 1.0):
    """(xyz0, bc_flag, tri, quad) of the square sheet; bc_flag pins the edge
    x = 0 as the reference does (cloth_internal.h:397-402)."""
    h = cloth_size / ndiv
    m = ndiv + 1
    ix, iy = np.meshgrid(np.arange(m), np.arange(m), indexing="ij")
    xyz0 = np.stack([ix * h, iy * h, np.zeros_like(ix, dtype=np.float64)], -1).reshape(-1).astype(np.float64)
    I, J = np.meshgrid(np.arange(ndiv), np.arange(ndiv), indexing="ij")
    I, J = I.ravel(), J.ravel()

    def vid(x, y):
        return (x * m + y).astype(np.uint32)

    tri = np.stack([vid(I, J), vid(I + 1, J), vid(I, J + 1), vid(I + 1, J + 1), vid(I, J + 1), vid(I + 1, J)],
                   -1).reshape(-1)
    q0 = np.stack([vid(I, J), vid(I + 1, J + 1), vid(I + 1, J), vid(I, J + 1)], -1)
    A, B = np.meshgrid(np.arange(ndiv), np.arange(ndiv - 1), indexing="ij")
    A, B = A.ravel(), B.ravel()
    q1 = np.stack([vid(A + 1, B), vid(A, B + 2), vid(A + 1, B + 1), vid(A, B + 1)], -1)
    A, B = np.meshgrid(np.arange(ndiv - 1), np.arange(ndiv), indexing="ij")
    A, B = A.ravel(), B.ravel()
    q2 = np.stack([vid(A, B + 1), vid(A + 2, B), vid(A + 1, B), vid(A + 1, B + 1)], -1)
    quad = np.concatenate([q0, q1, q2]).reshape(-1)
    bc = np.zeros(m * m * 3, np.int32)
    bc[: m * 3] = 1
    return xyz0, bc, tri.astype(np.uint32), quad.astype(np.uint32)


def pin_two_corners(ndiv: int):
    """bc flags pinning the two corners of the edge x = 0 (vertices 0, ndiv)."""
    bc = np.zeros((ndiv + 1) ** 2 * 3, np.int32)
    bc[0:3] = 1
    bc[ndiv * 3:ndiv * 3 + 3] = 1
    return bc


class Cloth:
    """A triangle sheet bound to a 3x3 block matrix whose pattern is the
    vertex adjacency of the bending quads (which covers every triangle)."""

    def __init__(self, xyz0, tri, quad, mat: CMatrixSparse | None = None):
        self.xyz0 = np.ascontiguousarray(xyz0, np.float64)
        self.tri = np.ascontiguousarray(tri, np.uint32)
        self.quad = np.ascontiguousarray(quad, np.uint32)
        self.np = self.xyz0.size // 3
        self.ntri = self.tri.size // 3
        self.nquad = self.quad.size // 4
        if mat is None:
            mat = CMatrixSparse()
            mat.Initialize(self.np, 3, True)
            ind, psup = JArray_PSuP_MeshElem(self.quad, 4, self.np)
            mat.SetPattern(ind, psup)
        self.mat = mat
        self.ilu = CPreconditionerILU()
        self.ilu.SetPattern0(mat)
        h = C.c_void_p()
        N.call("dfm2g_cloth_create", C.byref(h), mat._h, self.xyz0.ctypes.data, self.np, self.tri.ctypes.data,
               self.ntri, self.quad.ctypes.data, self.nquad)
        self._h = h

    @property
    def ncolor(self):
        a, b = C.c_uint(), C.c_uint()
        N.call("dfm2g_cloth_info", self._h, C.byref(a), C.byref(b))
        return a.value, b.value

    def MergeLinSys_Cloth(self, xyz, young_tri, nu: float, stiff_bend: float, dW) -> float:
        """K += ddW (PD-projected), dW += grad W (in place); returns W."""
        px, mx, kx = _vec(xyz, np.float64, False)
        py, my, ky = _vec(young_tri, np.float64, False)
        pd, md, kd = _vec(dW, np.float64, True)
        W = C.c_double(0.0)
        N.call("dfm2g_cloth_merge", self._h, self.mat._h, px, py, float(nu), float(stiff_bend), pd, C.byref(W),
               _same_mem(mx, my, md))
        return W.value

    def StepTime_InternalDynamicsILU(self, xyz, uvw, bc, young_tri, nu: float, stiff_bend: float, gravity,
                                     mass_point: float, dt: float, tol: float = 1e-4, max_iter: int = 100,
                                     solver: int = PCG_F64) -> N.SolveStats:
        """One backward-Euler step; xyz and uvw are updated in place."""
        px, mx, kx = _vec(xyz, np.float64, True)
        pv, mv, kv = _vec(uvw, np.float64, True)
        pb, mb, kb = _vec(bc, np.int32, False)
        py, my, ky = _vec(young_tri, np.float64, False)
        g3 = (C.c_double * 3)(*[float(v) for v in gravity])
        st = N.SolveStats()
        N.call("dfm2g_cloth_step", self._h, self.mat._h, self.ilu._h, px, pv, pb, py, float(nu), float(stiff_bend),
               g3, float(mass_point), float(dt), float(tol), int(max_iter), int(solver), C.byref(st),
               _same_mem(mx, mv, mb, my))
        return st

    def adjoint_terms(self, xyz, young_tri, nu: float, stiff_bend: float, mu, dx, xbar, Ebar):
        """xbar += -H mu - grad(mu^T A dx); Ebar += -(mu.dW + mu^T A dx)/E per triangle."""
        args = [_vec(xyz, np.float64, False), _vec(young_tri, np.float64, False), _vec(mu, np.float64, False),
                _vec(dx, np.float64, False), _vec(xbar, np.float64, True), _vec(Ebar, np.float64, True)]
        N.call("dfm2g_cloth_adjoint_terms", self._h, args[0][0], args[1][0], float(nu), float(stiff_bend),
               args[2][0], args[3][0], args[4][0], args[5][0], _same_mem(*[a[1] for a in args]))

    def rollout(self, xyz, uvw, bc, young_tri, nu, stiff_bend, gravity, mass_point, dt, tol, max_iter, nsteps,
                ckpt_every=10, solver=PCG_F64) -> N.SolveStats:
        """nsteps steps in place, keeping checkpoints every ckpt_every steps."""
        px, mx, kx = _vec(xyz, np.float64, True)
        pv, mv, kv = _vec(uvw, np.float64, True)
        pb, mb, kb = _vec(bc, np.int32, False)
        py, my, ky = _vec(young_tri, np.float64, False)
        g3 = (C.c_double * 3)(*[float(v) for v in gravity])
        st = N.SolveStats()
        N.call("dfm2g_cloth_rollout", self._h, self.mat._h, self.ilu._h, px, pv, pb, py, float(nu),
               float(stiff_bend), g3, float(mass_point), float(dt), float(tol), int(max_iter), int(solver),
               int(nsteps), int(ckpt_every), C.byref(st), _same_mem(mx, mv, mb, my))
        return st

    def rollout_adjoint(self, xbar, vbar, dLdE) -> N.SolveStats:
        """Reverse of the last rollout: xbar, vbar from dL/d(x_N, v_N) to
        dL/d(x_0, v_0) in place; dLdE (per triangle) overwritten."""
        px, mx, kx = _vec(xbar, np.float64, True)
        pv, mv, kv = _vec(vbar, np.float64, True)
        pe, me, ke = _vec(dLdE, np.float64, True)
        st = N.SolveStats()
        N.call("dfm2g_cloth_rollout_adjoint", self._h, self.mat._h, self.ilu._h, px, pv, pe, C.byref(st),
               _same_mem(mx, mv, me))
        return st

    def __del__(self):
        try:
            if self._h is not None:
                N.load().dfm2g_cloth_destroy(self._h)
                self._h = None
        except Exception:
            pass


class ClothRollout:
    """Settings of a multi-step rollout and the differentiable map
    E (per triangle) -> final positions, as a torch.autograd.Function."""

    def __init__(self, cloth: Cloth, bc, nu=0.3, stiff_bend=1e-3, gravity=(0.0, 0.0, -10.0), mass_point=None,
                 dt=0.01, tol=1e-8, max_iter=1000, nsteps=100, ckpt_every=10, solver=PCG_F64):
        self.cloth = cloth
        self.bc = np.ascontiguousarray(bc, np.int32)
        self.nu, self.stiff, self.g = nu, stiff_bend, tuple(gravity)
        self.mass = (1.0 / cloth.np) if mass_point is None else mass_point
        self.dt, self.tol, self.max_iter = dt, tol, max_iter
        self.nsteps, self.every, self.solver = nsteps, ckpt_every, solver

    def forward(self, young_tri, xyz=None, uvw=None):
        """Final (xyz, uvw) from (xyz, uvw) (default: rest, zero velocity)."""
        x = np.array(self.cloth.xyz0 if xyz is None else xyz, np.float64)
        v = np.zeros_like(x) if uvw is None else np.array(uvw, np.float64)
        st = self.cloth.rollout(x, v, self.bc, young_tri, self.nu, self.stiff, self.g, self.mass, self.dt, self.tol,
                                self.max_iter, self.nsteps, self.every, self.solver)
        return x, v, st

    def apply(self, young):
        """torch: x_N = rollout(young); backward through the checkpointed adjoint."""
        return _ClothFn.apply(young, self)


def _cloth_fn():
    import torch

    class ClothFn(torch.autograd.Function):
        @staticmethod
        def forward(ctx, young, ro: ClothRollout):
            dev = young.device
            y = young.detach().to(torch.float64).contiguous()
            x = torch.as_tensor(ro.cloth.xyz0, dtype=torch.float64, device=dev).clone()
            v = torch.zeros_like(x)
            bc = torch.as_tensor(ro.bc, device=dev)
            ro.cloth.rollout(x, v, bc, y, ro.nu, ro.stiff, ro.g, ro.mass, ro.dt, ro.tol, ro.max_iter, ro.nsteps,
                             ro.every, ro.solver)
            ctx.ro = ro
            ctx.dev = dev
            return x

        @staticmethod
        def backward(ctx, gx):
            import torch
            xbar = gx.detach().to(torch.float64).contiguous().clone()
            vbar = torch.zeros_like(xbar)
            dLdE = torch.zeros(ctx.ro.cloth.ntri, dtype=torch.float64, device=ctx.dev)
            ctx.ro.cloth.rollout_adjoint(xbar, vbar, dLdE)
            return dLdE, None

    return ClothFn


class _LazyFn:
    _fn = None

    @classmethod
    def apply(cls, *a):
        if cls._fn is None:
            cls._fn = _cloth_fn()
        return cls._fn.apply(*a)


_ClothFn = _LazyFn
