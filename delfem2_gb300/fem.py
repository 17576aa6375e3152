"""Element assembly on the device: linear tets (static, backward-Euler,
stiffness-warped and Newmark-beta elasticity with the adjoint element term,
3x3 blocks; scalar Poisson, 1x1 blocks), trilinear hexahedra (static
elasticity, 3x3 blocks) and 2-D linear triangles (scalar Poisson, 1x1 blocks;
static linear solid, 2x2 blocks).

TetMesh mirrors the per-element loops of MergeLinSys_SolidLinear_Static_MeshTet3D
(include/delfem2/fem_solidlinear.h:192-237, per-tet Young's modulus) and
MergeLinSys_Poission_MeshTet3D (include/delfem2/fem_poisson.h:128-162);
TriMesh2 those of MergeLinSys_Poission_MeshTri2D (fem_poisson.h:92-127) and
MergeLinSys_SolidLinear_Static_MeshTri2D (fem_solidlinear.h:155-187). The
assembly runs as colour-scheduled, atomic-free CUDA kernels.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .ls import CMatrixSparse, _same_mem, _vec


def lame(E, nu):
    """(lambda, myu) from Young's modulus and Poisson's ratio."""
    return E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu)), E / (2.0 * (1.0 + nu))


class TetMesh:
    """Element->slot map and colouring of a tet mesh against K's pattern."""

    def __init__(self, mat: CMatrixSparse, xyz, tet):
        self.xyz = np.ascontiguousarray(xyz, np.float64)
        self.tet = np.ascontiguousarray(tet, np.uint32)
        self.np = self.xyz.size // 3
        self.ntet = self.tet.size // 4
        h = C.c_void_p()
        N.call("dfm2g_tetmesh_create", C.byref(h), mat._h, self.xyz.ctypes.data, self.np, self.tet.ctypes.data,
               self.ntet)
        self._h = h
        self.mat = mat

    @property
    def ncolor(self) -> int:
        n = C.c_uint()
        N.call("dfm2g_tetmesh_info", self._h, C.byref(n), None)
        return n.value

    def assemble_linear(self, young, nu: float, rho: float, g, b, disp=None):
        """K += K_e(E_e); b += rho g vol/4 - K_e u_e (b in place)."""
        py, my, ky = _vec(young, np.float64, False)
        pb, mb, kb = _vec(b, np.float64, True)
        pd, md, kd = _vec(disp, np.float64, False) if disp is not None else (None, None, None)
        g3 = (C.c_double * 3)(*[float(v) for v in g])
        N.call("dfm2g_tetmesh_assemble_linear", self._h, self.mat._h, py, float(nu), float(rho), g3, pd, pb,
               _same_mem(my, mb, md))

    def assemble_poisson(self, alpha: float, source: float, b, val=None):
        """Scalar K += K_e, b += source vol/4 - K_e val_e (b in place; the matrix has 1x1 blocks)."""
        pb, mb, kb = _vec(b, np.float64, True)
        pv, mv, kv = _vec(val, np.float64, False) if val is not None else (None, None, None)
        N.call("dfm2g_tetmesh_assemble_poisson", self._h, self.mat._h, float(alpha), float(source), pv, pb,
               _same_mem(mb, mv))

    def assemble_beuler(self, myu: float, lam: float, rho: float, g, dt: float, disp, velo, b, rot=None):
        """Backward-Euler step matrix (stiffness-warped with rot, np x 3 x 3): K += K_e + rho vol/(4 dt^2) I,
        b += r_e / dt (MergeLinSys_SolidLinear_BEuler_MeshTet3D / MergeLinSys_SolidStiffwarp_BEuler_MeshTet3D)."""
        pu, mu, _ = _vec(disp, np.float64, False)
        pv, mv, _ = _vec(velo, np.float64, False)
        pr, mr, _ = _vec(rot, np.float64, False) if rot is not None else (None, None, None)
        pb, mb, _ = _vec(b, np.float64, True)
        g3 = (C.c_double * 3)(*[float(v) for v in g])
        N.call("dfm2g_tetmesh_assemble_beuler", self._h, self.mat._h, float(myu), float(lam), float(rho), g3,
               float(dt), pu, pv, pr, pb, _same_mem(mu, mv, mr, mb))

    def assemble_newmark(self, myu: float, lam: float, rho: float, g, dt: float, gamma: float, beta: float, disp,
                         velo, acc, b):
        """Newmark-beta matrix K += M_e + beta dt^2 K_e, b += r_e (MergeLinSys_SolidLinear_NewmarkBeta_MeshTet3D)."""
        pu, mu, _ = _vec(disp, np.float64, False)
        pv, mv, _ = _vec(velo, np.float64, False)
        pa, ma, _ = _vec(acc, np.float64, False)
        pb, mb, _ = _vec(b, np.float64, True)
        g3 = (C.c_double * 3)(*[float(v) for v in g])
        N.call("dfm2g_tetmesh_assemble_newmark", self._h, self.mat._h, float(myu), float(lam), float(rho), g3,
               float(dt), float(gamma), float(beta), pu, pv, pa, pb, _same_mem(mu, mv, ma, mb))

    def dLdE(self, nu: float, u, lam, out):
        """out[e] = -lam_e^T (dK_e/dE_e) u_e."""
        pu, mu, ku = _vec(u, np.float64, False)
        pl, ml, kl = _vec(lam, np.float64, False)
        po, mo, ko = _vec(out, np.float64, True)
        N.call("dfm2g_tetmesh_dLdE", self._h, None, float(nu), pu, pl, po, _same_mem(mu, ml, mo))

    def __del__(self):
        try:
            if self._h is not None:
                N.load().dfm2g_tetmesh_destroy(self._h)
                self._h = None
        except Exception:
            pass


class HexMesh:
    """Element->slot map and colouring of a trilinear-hex (Q1) mesh against a 3x3-block matrix's pattern."""

    def __init__(self, mat: CMatrixSparse, xyz, hexa):
        self.xyz = np.ascontiguousarray(xyz, np.float64)
        self.hex = np.ascontiguousarray(hexa, np.uint32)
        self.np = self.xyz.size // 3
        self.nhex = self.hex.size // 8
        h = C.c_void_p()
        N.call("dfm2g_hexmesh_create", C.byref(h), mat._h, self.xyz.ctypes.data, self.np, self.hex.ctypes.data,
               self.nhex)
        self._h = h
        self.mat = mat

    def assemble_linear(self, myu: float, lam: float, rho: float, g, b, disp=None):
        """K += K_e, b += int(rho g N) - K_e u_e (elemMatRes_LinearSolidGravity3_Static_Q1 per hex)."""
        pb, mb, _ = _vec(b, np.float64, True)
        pd, md, _ = _vec(disp, np.float64, False) if disp is not None else (None, None, None)
        g3 = (C.c_double * 3)(*[float(v) for v in g])
        N.call("dfm2g_hexmesh_assemble_linear", self._h, self.mat._h, float(myu), float(lam), float(rho), g3, pd, pb,
               _same_mem(mb, md))

    def __del__(self):
        try:
            if self._h is not None:
                N.load().dfm2g_hexmesh_destroy(self._h)
                self._h = None
        except Exception:
            pass


class TriMesh2:
    """Element->slot map and colouring of a 2-D triangle mesh against the pattern of a 1x1- or 2x2-block matrix."""

    def __init__(self, mat: CMatrixSparse, xy, tri):
        self.xy = np.ascontiguousarray(xy, np.float64)
        self.tri = np.ascontiguousarray(tri, np.uint32)
        self.np = self.xy.size // 2
        self.ntri = self.tri.size // 3
        h = C.c_void_p()
        N.call("dfm2g_trimesh2_create", C.byref(h), mat._h, self.xy.ctypes.data, self.np, self.tri.ctypes.data,
               self.ntri)
        self._h = h
        self.mat = mat

    def assemble_poisson(self, alpha: float, source: float, b, val=None):
        """Scalar K += K_e, b += source area/3 - K_e val_e (1x1 blocks)."""
        pb, mb, kb = _vec(b, np.float64, True)
        pv, mv, kv = _vec(val, np.float64, False) if val is not None else (None, None, None)
        N.call("dfm2g_trimesh2_assemble_poisson", self._h, self.mat._h, float(alpha), float(source), pv, pb,
               _same_mem(mb, mv))

    def assemble_solid_linear(self, myu: float, lam: float, rho: float, g, b, disp=None):
        """K += K_e, b += area rho g/3 - K_e u_e (2x2 blocks; g = (gx, gy))."""
        pb, mb, kb = _vec(b, np.float64, True)
        pd, md, kd = _vec(disp, np.float64, False) if disp is not None else (None, None, None)
        N.call("dfm2g_trimesh2_assemble_solid_linear", self._h, self.mat._h, float(myu), float(lam), float(rho),
               float(g[0]), float(g[1]), pd, pb, _same_mem(mb, md))

    def __del__(self):
        try:
            if self._h is not None:
                N.load().dfm2g_trimesh2_destroy(self._h)
                self._h = None
        except Exception:
            pass
