"""numpy front-end over the cloth functions of the CPU oracles (TEST INFRASTRUCTURE ONLY).

Each function takes an `Oracle` (oracle.port() or oracle.reference()) and calls
its orc_/ref_ symbol of the same name.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .oracle import _f64p, _i32p, _nz, _u32p


def _fn(O, name, argtypes, restype=None):
    f = getattr(O.lib, O.prefix + name)
    f.argtypes = argtypes
    f.restype = restype
    return f


def cloth_square(O, ndiv: int, size: float = 1.0):
    """Mesh of SetClothShape_Square: (xyz0, tri, quad)."""
    np_ = (ndiv + 1) ** 2
    ntri = ndiv * ndiv * 2
    nquad = ndiv * ndiv + ndiv * (ndiv - 1) * 2
    xyz0 = np.zeros(np_ * 3)
    tri = np.zeros(ntri * 3, np.uint32)
    quad = np.zeros(max(nquad * 4, 1), np.uint32)
    _fn(O, "cloth_square", [C.c_uint32, C.c_double, _f64p, _u32p, _u32p])(ndiv, size, xyz0, tri, quad)
    return xyz0, tri, quad[: nquad * 4]


def make_pd_sim22(O, s2):
    s3 = np.zeros(3)
    _fn(O, "make_pd_sim22", [_f64p, _f64p])(np.ascontiguousarray(s2, np.float64), s3)
    return s3


def wdwddw_cst(O, Cm, c, lam, myu):
    W = np.zeros(1)
    dW = np.zeros(9)
    ddW = np.zeros(81)
    _fn(O, "wdwddw_cst", [_f64p, _f64p, C.c_double, C.c_double, _f64p, _f64p, _f64p])(
        np.ascontiguousarray(Cm, np.float64).ravel(), np.ascontiguousarray(c, np.float64).ravel(), lam, myu, W, dW,
        ddW)
    return float(W[0]), dW.reshape(3, 3), ddW.reshape(3, 3, 3, 3)


def wdwddw_bend(O, Cm, c, stiff):
    W = np.zeros(1)
    dW = np.zeros(12)
    ddW = np.zeros(144)
    _fn(O, "wdwddw_bend", [_f64p, _f64p, C.c_double, _f64p, _f64p, _f64p])(
        np.ascontiguousarray(Cm, np.float64).ravel(), np.ascontiguousarray(c, np.float64).ravel(), stiff, W, dW,
        ddW)
    return float(W[0]), dW.reshape(4, 3), ddW.reshape(4, 4, 3, 3)


def cloth_assemble(O, row_start, col, xyz0, xyz, tri, quad, young_tri, nu, stiff_bend):
    """Returns (W, vcrs, vdia, dW) for K = ddW, starting from zero."""
    nblk = row_start.size - 1
    vc, vd, dW = np.zeros(max(col.size * 9, 9)), np.zeros(nblk * 9), np.zeros(nblk * 3)
    f = _fn(O, "cloth_assemble", [C.c_uint32, _u32p, _u32p, _f64p, _f64p, _f64p, _f64p, _f64p, _u32p, C.c_size_t,
                                  _u32p, C.c_size_t, _f64p, C.c_double, C.c_double], C.c_double)
    W = f(nblk, row_start, _nz(col), vc, vd, dW, xyz0, xyz, tri, tri.size // 3, _nz(quad), quad.size // 4,
          np.ascontiguousarray(young_tri, np.float64), nu, stiff_bend)
    return W, vc[: col.size * 9], vd, dW


def cloth_step(O, row_start, col, xyz, uvw, xyz0, bc, tri, quad, young_tri, nu, stiff_bend, g, mass, dt, tol,
               max_iter):
    """One backward-Euler step on copies of (xyz, uvw); returns (xyz, uvw, history length)."""
    nblk = row_start.size - 1
    x, v = np.array(xyz, np.float64), np.array(uvw, np.float64)
    f = _fn(O, "cloth_step", [C.c_uint32, _u32p, _u32p, _f64p, _f64p, _f64p, _i32p, _u32p, C.c_size_t, _u32p,
                              C.c_size_t, _f64p, C.c_double, C.c_double, _f64p, C.c_double, C.c_double, C.c_double,
                              C.c_uint32], C.c_uint32)
    nh = f(nblk, row_start, _nz(col), x, v, xyz0, np.ascontiguousarray(bc, np.int32), tri, tri.size // 3,
           _nz(quad), quad.size // 4, np.ascontiguousarray(young_tri, np.float64), nu, stiff_bend,
           np.ascontiguousarray(g, np.float64), mass, dt, tol, max_iter)
    return x, v, nh
