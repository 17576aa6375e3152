"""numpy front-end over the two CPU oracles (TEST INFRASTRUCTURE ONLY).

* ``port()``: the plain-C restatement ``dfm2_oracle.c`` (builds anywhere).
* ``reference()``: ``ref_driver.cpp`` over the unmodified DelFEM2 headers
  (built only where the reference source tree exists).

Both expose the same functions; arrays are numpy, indices uint32, values f64.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libdfm2ref.so")

_u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")


def build(reference_tree: str | None = None, quiet: bool = True) -> None:
    """Compile the restatement, and the reference driver when its tree exists."""
    env = dict(os.environ)
    if reference_tree:
        env["REF"] = reference_tree
    out = subprocess.run(["make", "-C", HERE, "all"], env=env, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if not quiet:
        print(out.stdout)


def _optr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class Oracle:
    """One of the two CPU implementations, selected by symbol prefix."""

    def __init__(self, so_path: str, prefix: str):
        self.lib = C.CDLL(so_path)
        self.prefix = prefix
        self.kind = "reference" if prefix == "ref_" else "port"

    def _f(self, name):
        return getattr(self.lib, self.prefix + name)

    # ---- mesh + pattern -------------------------------------------------
    def voxel_tet_mesh(self, nx, ny, nz, scale=1.0):
        np_ = (nx + 1) * (ny + 1) * (nz + 1)
        nt = nx * ny * nz * 6
        xyz = np.zeros(np_ * 3, np.float64)
        tet = np.zeros(nt * 4, np.uint32)
        f = self._f("voxel_tet_mesh")
        f.argtypes = [C.c_uint32] * 3 + [C.c_double, _f64p, _u32p]
        f(nx, ny, nz, scale, xyz, tet)
        return xyz, tet

    def psup(self, elem, nnoel, np_):
        elem = np.ascontiguousarray(elem, np.uint32)
        nelem = elem.size // nnoel
        ind = np.zeros(np_ + 1, np.uint32)
        fc = self._f("psup_count")
        fc.argtypes = [_u32p, C.c_size_t, C.c_uint32, C.c_size_t, _u32p]
        fc.restype = C.c_size_t
        n = fc(elem, nelem, nnoel, np_, ind)
        psup = np.zeros(max(n, 1), np.uint32)
        ff = self._f("psup_fill")
        ff.argtypes = [_u32p, C.c_size_t, C.c_uint32, C.c_size_t, _u32p, _u32p]
        ff(elem, nelem, nnoel, np_, ind, psup)
        return ind, psup[:n]

    # ---- matrix ----------------------------------------------------------
    def matvec(self, row_start, col, vcrs, vdia, y, alpha, x, beta):
        nblk = row_start.size - 1
        if vcrs.dtype == np.float32:
            f = self._f("bsr_matvec_f32")
            f.argtypes = [C.c_uint32, _u32p, _u32p, _f32p, _f32p, _f32p, C.c_float, _f32p, C.c_float]
        else:
            f = self._f("bsr_matvec")
            f.argtypes = [C.c_uint32, _u32p, _u32p, _f64p, _f64p, _f64p, C.c_double, _f64p, C.c_double]
        y = y.copy()
        f(nblk, row_start, _nz(col), _nz(vcrs), vdia, y, alpha, x, beta)
        return y

    def merge(self, row_start, col, vcrs, vdia, nodes, emat):
        nblk = row_start.size - 1
        f = self._f("merge")
        f.argtypes = [C.c_uint32, _u32p, _u32p, _f64p, _f64p, C.c_uint32, _u32p, _f64p, _u32p]
        f.restype = C.c_int
        buf = np.full(nblk, 0xFFFFFFFF, np.uint32)
        nodes = np.ascontiguousarray(nodes, np.uint32)
        return f(nblk, row_start, _nz(col), _nz(vcrs), vdia, nodes.size, nodes,
                 np.ascontiguousarray(emat, np.float64).ravel(), buf)

    def set_fixed_bc(self, row_start, col, vcrs, vdia, bc):
        nblk = row_start.size - 1
        f = self._f("set_fixed_bc")
        f.argtypes = [C.c_uint32, _u32p, _u32p, _f64p, _f64p, _i32p]
        f(nblk, row_start, _nz(col), _nz(vcrs), vdia, np.ascontiguousarray(bc, np.int32))

    def rhs_zero(self, b, bc):
        f = self._f("rhs_zero")
        f.argtypes = [_f64p, _i32p, C.c_size_t]
        f(b, np.ascontiguousarray(bc, np.int32), b.size)

    def emat_tet_linear(self, P, myu, lam):
        f = self._f("emat_tet_linear")
        f.argtypes = [_f64p, C.c_double, C.c_double, _f64p, _f64p]
        emat = np.zeros(144, np.float64)
        vol = np.zeros(1, np.float64)
        f(np.ascontiguousarray(P, np.float64).ravel(), myu, lam, emat, vol)
        return emat.reshape(4, 4, 3, 3), float(vol[0])

    def assemble_tet_linear(self, row_start, col, vcrs, vdia, b, xyz, tet, young, nu, rho, g,
                            disp=None):
        nblk = row_start.size - 1
        f = self._f("assemble_tet_linear")
        f.argtypes = [C.c_uint32, _u32p, _u32p, _f64p, _f64p, _f64p, _f64p, _u32p, C.c_size_t,
                      _f64p, C.c_double, C.c_double, _f64p, C.c_void_p]
        f.restype = C.c_int
        g = np.ascontiguousarray(g, np.float64)
        return f(nblk, row_start, _nz(col), _nz(vcrs), vdia, b, xyz, tet, tet.size // 4,
                 np.ascontiguousarray(young, np.float64), nu, rho, g, _optr(disp))

    def tet_dLdE(self, xyz, tet, young, nu, u, lam):
        f = self.lib.orc_tet_dLdE  # restatement only (the reference has no adjoint)
        f.argtypes = [_f64p, _u32p, C.c_size_t, _f64p, C.c_double, _f64p, _f64p, _f64p]
        out = np.zeros(tet.size // 4, np.float64)
        f(xyz, tet, tet.size // 4, np.ascontiguousarray(young, np.float64), nu, u, lam, out)
        return out

    # ---- ILU -------------------------------------------------------------
    def ilu_pattern0(self, row_start, col):
        nblk = row_start.size - 1
        f = self._f("ilu_pattern0")
        f.argtypes = [C.c_uint32, _u32p, _u32p, _u32p, _u32p]
        col_out = np.zeros(max(col.size, 1), np.uint32)
        dia = np.zeros(nblk, np.uint32)
        f(nblk, row_start, _nz(col), col_out, dia)
        return col_out[: col.size], dia

    def ilu_copy_value(self, row_start, col_ilu, col_mat, mat_vcrs, mat_vdia):
        nblk = row_start.size - 1
        f = self._f("ilu_copy_value")
        f.argtypes = [C.c_uint32, _u32p, _u32p, _f64p, _f64p, _u32p, _f64p, _f64p]
        vcrs = np.zeros(max(mat_vcrs.size, 9), np.float64)
        vdia = np.zeros(nblk * 9, np.float64)
        f(nblk, row_start, _nz(col_ilu), vcrs, vdia, _nz(col_mat), _nz(mat_vcrs), mat_vdia)
        return vcrs[: mat_vcrs.size], vdia

    def ilu_pattern_k(self, row_start, col_in, lev_fill):
        """Initialize_ILUk's pattern: (row_start, col, dia_ind) of the ILU(k)."""
        nblk = row_start.size - 1
        f = self._f("ilu_pattern_k")
        f.argtypes = [C.c_uint32, _u32p, _u32p, C.c_int, _u32p, C.c_void_p, C.c_size_t, _u32p]
        f.restype = C.c_size_t
        rs = np.zeros(nblk + 1, np.uint32)
        dia = np.zeros(max(nblk, 1), np.uint32)
        n = f(nblk, row_start, _nz(col_in), int(lev_fill), rs, None, 0, dia)
        col = np.zeros(max(n, 1), np.uint32)
        f(nblk, row_start, _nz(col_in), int(lev_fill), rs, col.ctypes.data, col.size, dia)
        return rs, col[:n], dia[:nblk]

    def ilu_copy_value_k(self, mrow_start, col_mat, mat_vcrs, mat_vdia, lev_fill, irow_start, col_ilu):
        nblk = mrow_start.size - 1
        f = self._f("ilu_copy_value_k")
        f.argtypes = [C.c_uint32, _u32p, _u32p, _f64p, _f64p, C.c_int, _u32p, _u32p, _f64p, _f64p]
        vcrs = np.zeros(max(col_ilu.size * 9, 9), np.float64)
        vdia = np.zeros(nblk * 9, np.float64)
        f(nblk, mrow_start, _nz(col_mat), _nz(mat_vcrs), mat_vdia, int(lev_fill), irow_start, _nz(col_ilu), vcrs,
          vdia)
        return vcrs[: col_ilu.size * 9], vdia

    def ilu_decompose(self, row_start, col, dia, vcrs, vdia):
        """In place; returns (status, n_singular) with status 0 on success."""
        nblk = row_start.size - 1
        f = self._f("ilu_decompose")
        f.argtypes = [C.c_uint32, _u32p, _u32p, _u32p, _f64p, _f64p, _i32p]
        f.restype = C.c_int
        ns = np.zeros(1, np.int32)
        st = f(nblk, row_start, _nz(col), dia, _nz(vcrs), vdia, ns)
        return st, int(ns[0])

    def ilu_forward(self, row_start, col, dia, vcrs, vdia, vec):
        f = self._f("ilu_forward")
        f.argtypes = [C.c_uint32, _u32p, _u32p, _u32p, _f64p, _f64p, _f64p]
        v = np.array(vec, np.float64)
        f(row_start.size - 1, row_start, _nz(col), dia, _nz(vcrs), vdia, v)
        return v

    def ilu_backward(self, row_start, col, dia, vcrs, vec):
        f = self._f("ilu_backward")
        f.argtypes = [C.c_uint32, _u32p, _u32p, _u32p, _f64p, _f64p]
        v = np.array(vec, np.float64)
        f(row_start.size - 1, row_start, _nz(col), dia, _nz(vcrs), v)
        return v

    def ilu_levels(self, row_start, col, dia, backward=False):
        """Level sets (restatement only; the reference sweeps serially)."""
        nblk = row_start.size - 1
        f = self.lib.orc_ilu_levels
        f.argtypes = [C.c_uint32, _u32p, _u32p, _u32p, C.c_int, _u32p, _u32p, _u32p]
        f.restype = C.c_uint32
        level = np.zeros(nblk, np.uint32)
        order = np.zeros(nblk, np.uint32)
        lstart = np.zeros(nblk + 1, np.uint32)
        nlev = f(nblk, row_start, _nz(col), dia, int(backward), level, order, lstart)
        return level, order, lstart[: nlev + 1]

    # ---- Krylov ------------------------------------------------------------
    def solve_pcg(self, row_start, col, vcrs, vdia, ilu_col, dia, ilu_vcrs, ilu_vdia, r, tol,
                  max_iter):
        """Returns (x, r_final, hist) for Solve_PCG on a copy of r."""
        nblk = row_start.size - 1
        f = self._f("solve_pcg")
        f.argtypes = [C.c_uint32, _u32p, _u32p, _f64p, _f64p, _u32p, _u32p, _f64p, _f64p, _f64p,
                      _f64p, C.c_double, C.c_uint32, _f64p, C.c_uint32]
        f.restype = C.c_uint32
        r = np.array(r, np.float64)
        x = np.zeros_like(r)
        cap = max_iter + 2
        hist = np.zeros(cap, np.float64)
        nh = f(nblk, row_start, _nz(col), _nz(vcrs), vdia, _nz(ilu_col), dia, _nz(ilu_vcrs),
               ilu_vdia, r, x, tol, max_iter, hist, cap)
        return x, r, hist[:nh]

    def solve_pcg_k(self, row_start, col, vcrs, vdia, ilu_row_start, ilu_col, dia, ilu_vcrs, ilu_vdia, r, tol,
                    max_iter):
        """Solve_PCG with an ILU whose pattern has its own row offsets (ILU(k))."""
        nblk = row_start.size - 1
        f = self._f("solve_pcg_k")
        f.argtypes = [C.c_uint32, _u32p, _u32p, _f64p, _f64p, _u32p, _u32p, _u32p, _f64p, _f64p, _f64p,
                      _f64p, C.c_double, C.c_uint32, _f64p, C.c_uint32]
        f.restype = C.c_uint32
        r = np.array(r, np.float64)
        x = np.zeros_like(r)
        cap = max_iter + 2
        hist = np.zeros(cap, np.float64)
        nh = f(nblk, row_start, _nz(col), _nz(vcrs), vdia, ilu_row_start, _nz(ilu_col), dia, _nz(ilu_vcrs),
               ilu_vdia, r, x, tol, max_iter, hist, cap)
        return x, r, hist[:nh]

    def solve_pbicgstab(self, row_start, col, vcrs, vdia, ilu_row_start, ilu_col, dia, ilu_vcrs, ilu_vdia, r,
                        tol, max_iter):
        """Returns (x, r_final, hist) for Solve_PBiCGStab on a copy of r (relative history)."""
        nblk = row_start.size - 1
        f = self._f("solve_pbicgstab")
        f.argtypes = [C.c_uint32, _u32p, _u32p, _f64p, _f64p, _u32p, _u32p, _u32p, _f64p, _f64p, _f64p,
                      _f64p, C.c_double, C.c_uint32, _f64p, C.c_uint32]
        f.restype = C.c_uint32
        r = np.array(r, np.float64)
        x = np.zeros_like(r)
        cap = max_iter + 2
        hist = np.zeros(cap, np.float64)
        nh = f(nblk, row_start, _nz(col), _nz(vcrs), vdia, ilu_row_start, _nz(ilu_col), dia, _nz(ilu_vcrs),
               ilu_vdia, r, x, tol, max_iter, hist, cap)
        return x, r, hist[:nh]

    def solve_cg(self, row_start, col, vcrs, vdia, r, tol, max_iter):
        nblk = row_start.size - 1
        f = self._f("solve_cg")
        f.argtypes = [C.c_uint32, _u32p, _u32p, _f64p, _f64p, _f64p, _f64p, C.c_double,
                      C.c_uint32, _f64p, C.c_uint32]
        f.restype = C.c_uint32
        r = np.array(r, np.float64)
        x = np.zeros_like(r)
        hist = np.zeros(max_iter + 2, np.float64)
        nh = f(nblk, row_start, _nz(col), _nz(vcrs), vdia, r, x, tol, max_iter, hist, hist.size)
        return x, r, hist[:nh]


    # ---- scalar (ndim 1) and 2x2 (ndim 2) blocks; ndim 3 runs the 3x3 code --------
    def nd_matvec(self, ndim, row_start, col, vcrs, vdia, y, alpha, x, beta):
        nblk = row_start.size - 1
        f = self._f("nd_matvec")
        f.argtypes = [C.c_uint32, C.c_uint32, _u32p, _u32p, _f64p, _f64p, _f64p, C.c_double, _f64p, C.c_double]
        y = np.array(y, np.float64)
        f(nblk, ndim, row_start, _nz(col), _nz(vcrs), vdia, y, alpha, np.ascontiguousarray(x, np.float64), beta)
        return y

    def nd_merge(self, ndim, row_start, col, vcrs, vdia, nodes, emat):
        """Merges one element in place; returns 0, or 1 on a missing slot."""
        nblk = row_start.size - 1
        f = self._f("nd_merge")
        f.argtypes = [C.c_uint32, C.c_uint32, _u32p, _u32p, _f64p, _f64p, C.c_uint32, _u32p, _f64p, _u32p]
        f.restype = C.c_int
        buf = np.full(nblk, 0xFFFFFFFF, np.uint32)
        nodes = np.ascontiguousarray(nodes, np.uint32)
        return f(nblk, ndim, row_start, _nz(col), _nz(vcrs), vdia, nodes.size, nodes,
                 np.ascontiguousarray(emat, np.float64).ravel(), buf)

    def nd_set_fixed_bc(self, ndim, row_start, col, vcrs, vdia, bc):
        nblk = row_start.size - 1
        f = self._f("nd_set_fixed_bc")
        f.argtypes = [C.c_uint32, C.c_uint32, _u32p, _u32p, _f64p, _f64p, _i32p]
        f(nblk, ndim, row_start, _nz(col), _nz(vcrs), vdia, np.ascontiguousarray(bc, np.int32))

    def nd_ilu_copy_value(self, ndim, mrow_start, col_mat, mat_vcrs, mat_vdia, lev_fill, irow_start, col_ilu):
        """CopyValue into the given ILU pattern; returns (ilu_vcrs, ilu_vdia)."""
        nblk = mrow_start.size - 1
        bb = ndim * ndim
        f = self._f("nd_ilu_copy_value")
        f.argtypes = [C.c_uint32, C.c_uint32, _u32p, _u32p, _f64p, _f64p, C.c_int, _u32p, _u32p, _f64p, _f64p]
        vc = np.zeros(max(int(irow_start[-1]) * bb, 1), np.float64)
        vd = np.zeros(max(nblk * bb, 1), np.float64)
        f(nblk, ndim, mrow_start, _nz(col_mat), _nz(mat_vcrs), _nz(mat_vdia), int(lev_fill), irow_start,
          _nz(col_ilu), vc, vd)
        return vc[: int(irow_start[-1]) * bb], vd[: nblk * bb]

    def nd_ilu_decompose(self, ndim, row_start, col, dia_ind, vcrs, vdia):
        """Returns (status, vcrs, vdia) of Decompose on copies of the values."""
        nblk = row_start.size - 1
        f = self._f("nd_ilu_decompose")
        f.argtypes = [C.c_uint32, C.c_uint32, _u32p, _u32p, _u32p, _f64p, _f64p, C.POINTER(C.c_int)]
        f.restype = C.c_int
        vc, vd = np.array(vcrs, np.float64), np.array(vdia, np.float64)
        ns = C.c_int(0)
        st = f(nblk, ndim, row_start, _nz(col), _nz(dia_ind), _nz(vc), _nz(vd), C.byref(ns))
        return st, vc, vd

    def nd_ilu_forward(self, ndim, row_start, col, dia_ind, vcrs, vdia, vec):
        nblk = row_start.size - 1
        f = self._f("nd_ilu_forward")
        f.argtypes = [C.c_uint32, C.c_uint32, _u32p, _u32p, _u32p, _f64p, _f64p, _f64p]
        v = np.array(vec, np.float64)
        f(nblk, ndim, row_start, _nz(col), _nz(dia_ind), _nz(vcrs), _nz(vdia), _nz(v))
        return v

    def nd_ilu_backward(self, ndim, row_start, col, dia_ind, vcrs, vec):
        nblk = row_start.size - 1
        f = self._f("nd_ilu_backward")
        f.argtypes = [C.c_uint32, C.c_uint32, _u32p, _u32p, _u32p, _f64p, _f64p]
        v = np.array(vec, np.float64)
        f(nblk, ndim, row_start, _nz(col), _nz(dia_ind), _nz(vcrs), _nz(v))
        return v

    def _nd_solve(self, name, ndim, row_start, col, vcrs, vdia, ilu_row_start, ilu_col, dia, ilu_vcrs, ilu_vdia, r,
                  tol, max_iter):
        nblk = row_start.size - 1
        f = self._f(name)
        f.argtypes = [C.c_uint32, C.c_uint32, _u32p, _u32p, _f64p, _f64p, _u32p, _u32p, _u32p, _f64p, _f64p, _f64p,
                      _f64p, C.c_double, C.c_uint32, _f64p, C.c_uint32]
        f.restype = C.c_uint32
        r = np.array(r, np.float64)
        x = np.zeros_like(r)
        hist = np.zeros(max_iter + 2, np.float64)
        nh = f(nblk, ndim, row_start, _nz(col), _nz(vcrs), vdia, ilu_row_start, _nz(ilu_col), _nz(dia),
               _nz(ilu_vcrs), ilu_vdia, r, x, tol, max_iter, hist, hist.size)
        return x, r, hist[:nh]

    def nd_solve_pcg(self, ndim, *args):
        """(row_start, col, vcrs, vdia, ilu_row_start, ilu_col, dia, ilu_vcrs, ilu_vdia, r, tol, max_iter)
        -> (x, r_final, hist): Solve_PCG (absolute history)."""
        return self._nd_solve("nd_solve_pcg", ndim, *args)

    def nd_solve_pbicgstab(self, ndim, *args):
        """Same arguments as nd_solve_pcg -> (x, r_final, hist): Solve_PBiCGStab (relative history)."""
        return self._nd_solve("nd_solve_pbicgstab", ndim, *args)

    def assemble_poisson_tet(self, row_start, col, xyz, tet, alpha, source, val=None):
        """MergeLinSys_Poission_MeshTet3D into a zeroed scalar matrix: (vcrs, vdia, b)."""
        nblk = row_start.size - 1
        f = self._f("assemble_poisson_tet")
        f.argtypes = [C.c_uint32, _u32p, _u32p, _f64p, _f64p, _f64p, C.c_double, C.c_double, _f64p, _u32p,
                      C.c_size_t, C.c_void_p]
        f.restype = C.c_int
        vc = np.zeros(max(col.size, 1), np.float64)
        vd = np.zeros(nblk, np.float64)
        b = np.zeros(nblk, np.float64)
        tet = np.ascontiguousarray(tet, np.uint32)
        v = None if val is None else np.ascontiguousarray(val, np.float64)
        st = f(nblk, row_start, _nz(col), vc, vd, b, alpha, source, np.ascontiguousarray(xyz, np.float64), tet,
               tet.size // 4, _optr(v))
        assert st == 0, "element block missing from the pattern"
        return vc[: col.size], vd, b

    def assemble_tri2(self, ndim, row_start, col, xy, tri, param, val=None):
        """Scalar Poisson (ndim 1, param = (alpha, source)) or 2-D linear solid (ndim 2, param = (myu, lambda,
        rho, gx, gy)) over a 2-D triangle mesh into a zeroed matrix: (vcrs, vdia, b)."""
        nblk = row_start.size - 1
        bb = ndim * ndim
        f = self._f("assemble_tri2")
        f.argtypes = [C.c_uint32, C.c_uint32, _u32p, _u32p, _f64p, _f64p, _f64p, _f64p, _f64p, _u32p, C.c_size_t,
                      C.c_void_p]
        f.restype = C.c_int
        vc = np.zeros(max(col.size * bb, 1), np.float64)
        vd = np.zeros(nblk * bb, np.float64)
        b = np.zeros(nblk * ndim, np.float64)
        tri = np.ascontiguousarray(tri, np.uint32)
        v = None if val is None else np.ascontiguousarray(val, np.float64)
        st = f(nblk, ndim, row_start, _nz(col), vc, vd, b, np.ascontiguousarray(param, np.float64),
               np.ascontiguousarray(xy, np.float64), tri, tri.size // 3, _optr(v))
        assert st == 0, "element block missing from the pattern"
        return vc[: col.size * bb], vd, b


    # ---- dynamic linear tets (3x3 blocks) -----------------------------------------
    def assemble_tet_beuler(self, row_start, col, xyz, tet, myu, lam, rho, g, dt, disp, velo, rot=None):
        """BEuler (rot None) or stiffness-warped BEuler tet assembly into a zeroed matrix: (vcrs, vdia, b)."""
        nblk = row_start.size - 1
        f = self._f("assemble_tet_beuler")
        f.argtypes = [C.c_uint32, _u32p, _u32p, _f64p, _f64p, _f64p, C.c_double, C.c_double, C.c_double, _f64p,
                      C.c_double, _f64p, _u32p, C.c_size_t, _f64p, _f64p, C.c_void_p]
        f.restype = C.c_int
        vc = np.zeros(max(col.size * 9, 1), np.float64)
        vd = np.zeros(nblk * 9, np.float64)
        b = np.zeros(nblk * 3, np.float64)
        tet = np.ascontiguousarray(tet, np.uint32)
        r = None if rot is None else np.ascontiguousarray(rot, np.float64)
        st = f(nblk, row_start, _nz(col), vc, vd, b, myu, lam, rho, np.ascontiguousarray(g, np.float64), dt,
               np.ascontiguousarray(xyz, np.float64), tet, tet.size // 4, np.ascontiguousarray(disp, np.float64),
               np.ascontiguousarray(velo, np.float64), _optr(r))
        assert st == 0
        return vc[: col.size * 9], vd, b

    def assemble_tet_newmark(self, row_start, col, xyz, tet, myu, lam, rho, g, dt, gamma, beta, disp, velo, acc):
        """Newmark-beta tet assembly (initial iteration) into a zeroed matrix: (vcrs, vdia, b)."""
        nblk = row_start.size - 1
        f = self._f("assemble_tet_newmark")
        f.argtypes = [C.c_uint32, _u32p, _u32p, _f64p, _f64p, _f64p, C.c_double, C.c_double, C.c_double, _f64p,
                      C.c_double, C.c_double, C.c_double, _f64p, _u32p, C.c_size_t, _f64p, _f64p, _f64p]
        f.restype = C.c_int
        vc = np.zeros(max(col.size * 9, 1), np.float64)
        vd = np.zeros(nblk * 9, np.float64)
        b = np.zeros(nblk * 3, np.float64)
        tet = np.ascontiguousarray(tet, np.uint32)
        st = f(nblk, row_start, _nz(col), vc, vd, b, myu, lam, rho, np.ascontiguousarray(g, np.float64), dt, gamma,
               beta, np.ascontiguousarray(xyz, np.float64), tet, tet.size // 4,
               *[np.ascontiguousarray(v, np.float64) for v in (disp, velo, acc)])
        assert st == 0
        return vc[: col.size * 9], vd, b


    # ---- trilinear hexahedra (Q1) ------------------------------------------------
    def emat_hex_q1(self, P, myu, lam, rho, g, disp):
        f = self._f("emat_hex_q1")
        f.argtypes = [_f64p, C.c_double, C.c_double, C.c_double, _f64p, _f64p, _f64p, _f64p]
        emat = np.zeros(8 * 8 * 9, np.float64)
        eres = np.zeros(24, np.float64)
        f(np.ascontiguousarray(P, np.float64).ravel(), myu, lam, rho, np.ascontiguousarray(g, np.float64),
          np.ascontiguousarray(disp, np.float64).ravel(), emat, eres)
        return emat.reshape(8, 8, 3, 3), eres.reshape(8, 3)

    def assemble_hex_q1(self, row_start, col, xyz, hexa, myu, lam, rho, g, disp=None):
        """Q1 hex assembly into a zeroed matrix: (vcrs, vdia, b)."""
        nblk = row_start.size - 1
        f = self._f("assemble_hex_q1")
        f.argtypes = [C.c_uint32, _u32p, _u32p, _f64p, _f64p, _f64p, C.c_double, C.c_double, C.c_double, _f64p,
                      _f64p, _u32p, C.c_size_t, C.c_void_p]
        f.restype = C.c_int
        vc = np.zeros(max(col.size * 9, 1), np.float64)
        vd = np.zeros(nblk * 9, np.float64)
        b = np.zeros(nblk * 3, np.float64)
        hexa = np.ascontiguousarray(hexa, np.uint32)
        d = None if disp is None else np.ascontiguousarray(disp, np.float64)
        st = f(nblk, row_start, _nz(col), vc, vd, b, myu, lam, rho, np.ascontiguousarray(g, np.float64),
               np.ascontiguousarray(xyz, np.float64), hexa, hexa.size // 8, _optr(d))
        assert st == 0
        return vc[: col.size * 9], vd, b

    # ---- deformers (reference only: oracle/ref_driver_deform.cpp) ---------------
    def arap_elements(self, xyz0, tri, xyz1, quat1):
        """Deformer_Arap's per-point elements: (ptr[np+1], idx, eM (9 n^2 each), eR (3 per entry))."""
        np_ = xyz0.size // 3
        tri = np.ascontiguousarray(tri, np.uint32)
        fs = self._f("arap_sizes")
        fs.argtypes = [C.c_uint32, C.c_uint32, _u32p, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
        ni, nm = C.c_uint64(), C.c_uint64()
        fs(np_, tri.size // 3, tri, C.byref(ni), C.byref(nm))
        ptr = np.zeros(np_ + 1, np.uint32)
        idx = np.zeros(ni.value, np.uint32)
        eM = np.zeros(nm.value, np.float64)
        eR = np.zeros(ni.value * 3, np.float64)
        f = self._f("arap_elements")
        f.argtypes = [C.c_uint32, _f64p, C.c_uint32, _u32p, _f64p, _f64p, _u32p, _u32p, _f64p, _f64p]
        f(np_, np.ascontiguousarray(xyz0, np.float64), tri.size // 3, tri, np.ascontiguousarray(xyz1, np.float64),
          np.ascontiguousarray(quat1, np.float64), ptr, idx, eM, eR)
        return ptr, idx, eM, eR

    def arap_deform(self, xyz0, tri, xyz1, quat1, bc):
        """One Deformer_Arap::Deform with ILU(0)-PCG: (new xyz1, history)."""
        np_ = xyz0.size // 3
        tri = np.ascontiguousarray(tri, np.uint32)
        x1 = np.array(xyz1, np.float64)
        q1 = np.array(quat1, np.float64)
        hist = np.zeros(1000, np.float64)
        f = self._f("arap_deform")
        f.argtypes = [C.c_uint32, _f64p, C.c_uint32, _u32p, _f64p, _f64p, _i32p, _f64p, C.c_uint32]
        f.restype = C.c_uint32
        nh = f(np_, np.ascontiguousarray(xyz0, np.float64), tri.size // 3, tri, x1, q1,
               np.ascontiguousarray(bc, np.int32), hist, hist.size)
        return x1, hist[:nh]

    def lap_deform(self, xyz0, tri, bc, xyz_def):
        """CDef_LaplacianLinear (ILU(20)): its matrix pattern, dual-Laplacian elements, ILU(20) pattern, and one
        Deform from xyz_def: dict(pat_start, pat_col, ptr, idx, eM, ilu_start, ilu_col, xyz_def, hist)."""
        np_ = xyz0.size // 3
        tri = np.ascontiguousarray(tri, np.uint32)
        fs = self._f("lap_sizes")
        fs.argtypes = [C.c_uint32, C.c_uint32, _u32p] + [C.POINTER(C.c_uint64)] * 4
        npat, ni, nm, nilu = (C.c_uint64() for _ in range(4))
        fs(np_, tri.size // 3, tri, C.byref(npat), C.byref(ni), C.byref(nm), C.byref(nilu))
        out = dict(pat_start=np.zeros(np_ + 1, np.uint32), pat_col=np.zeros(npat.value, np.uint32),
                   ptr=np.zeros(np_ + 1, np.uint32), idx=np.zeros(ni.value, np.uint32),
                   eM=np.zeros(nm.value, np.float64), ilu_start=np.zeros(np_ + 1, np.uint32),
                   ilu_col=np.zeros(nilu.value, np.uint32), xyz_def=np.array(xyz_def, np.float64))
        hist = np.zeros(1000, np.float64)
        f = self._f("lap_deform")
        f.argtypes = [C.c_uint32, _f64p, C.c_uint32, _u32p, _i32p, _f64p, _u32p, _u32p, _u32p, _u32p, _f64p, _u32p,
                      _u32p, _f64p, C.c_uint32]
        f.restype = C.c_uint32
        nh = f(np_, np.ascontiguousarray(xyz0, np.float64), tri.size // 3, tri, np.ascontiguousarray(bc, np.int32),
               out["xyz_def"], out["pat_start"], out["pat_col"], out["ptr"], out["idx"], out["eM"],
               out["ilu_start"], out["ilu_col"], hist, hist.size)
        out["hist"] = hist[:nh]
        return out


def hex_grid(nx: int, ny: int, nz: int, h: float, seed: int | None = None, jitter: float = 0.0):
    """A structured nx x ny x nz hex mesh of spacing h (node (ix,iy,iz) = ix*(ny+1)*(nz+1) + iy*(nz+1) + iz), each
    hex's nodes in ShapeFunc_Hex8's corner order; interior nodes moved by up to jitter*h when seeded."""
    ii, jj, kk = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), np.arange(nz + 1), indexing="ij")
    xyz = np.stack([ii, jj, kk], -1).reshape(-1, 3).astype(np.float64) * h
    if seed is not None and jitter > 0:
        rng = np.random.default_rng(seed)
        inner = ((ii > 0) & (ii < nx) & (jj > 0) & (jj < ny) & (kk > 0) & (kk < nz)).ravel()
        xyz[inner] += rng.uniform(-jitter * h, jitter * h, (int(inner.sum()), 3))

    def nid(i, j, k):
        return (i * (ny + 1) + j) * (nz + 1) + k

    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    i, j, k = i.ravel(), j.ravel(), k.ravel()
    hexa = np.stack([nid(i, j, k), nid(i + 1, j, k), nid(i + 1, j + 1, k), nid(i, j + 1, k),
                     nid(i, j, k + 1), nid(i + 1, j, k + 1), nid(i + 1, j + 1, k + 1), nid(i, j + 1, k + 1)], -1)
    return xyz.ravel(), hexa.astype(np.uint32).ravel()


def _nz(a):
    """Never hand a zero-length array to C (its data pointer may be NULL)."""
    if a.size == 0:
        return np.zeros(1, a.dtype)
    return a


_PORT = None
_REF = None


def port() -> Oracle:
    global _PORT
    if _PORT is None:
        if not os.path.exists(PORT_SO):
            build()
        _PORT = Oracle(PORT_SO, "orc_")
    return _PORT


def HAVE_REFERENCE_BUILD() -> bool:
    return os.path.exists(REF_SO)


def reference() -> Oracle:
    global _REF
    if _REF is None:
        if not os.path.exists(REF_SO):
            raise FileNotFoundError("reference driver not built (needs the DelFEM2 source tree)")
        _REF = Oracle(REF_SO, "ref_")
    return _REF
