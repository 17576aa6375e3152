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


def pd_sim22_jac(O, s2):
    J = np.zeros(9)
    _fn(O, "pd_sim22_jac", [_f64p, _f64p])(np.ascontiguousarray(s2, np.float64), J)
    return J.reshape(3, 3)


def adjoint_terms(O, xyz0, xyz, tri, quad, young_tri, nu, stiff_bend, mu, dx, xbar, Ebar):
    """In place: xbar += -H mu - grad(mu^T ddW dx); Ebar += -(mu.dW + mu^T ddW dx)/E."""
    f = _fn(O, "cloth_adjoint_terms", [_f64p, _f64p, _u32p, C.c_size_t, _u32p, C.c_size_t, _f64p, C.c_double,
                                       C.c_double, _f64p, _f64p, _f64p, _f64p])
    f(xyz0, np.ascontiguousarray(xyz, np.float64), tri, tri.size // 3, _nz(quad), quad.size // 4,
      np.ascontiguousarray(young_tri, np.float64), nu, stiff_bend, np.ascontiguousarray(mu, np.float64),
      np.ascontiguousarray(dx, np.float64), xbar, Ebar)


def step_matrix(O, row_start, col, xyz0, xyz, bc, tri, quad, young_tri, nu, stiff_bend, mass, dt):
    """The clamped A = M/dt^2 + ddW(x) of a step and its ILU(0) factors."""
    W, vc, vd, dW = cloth_assemble(O, row_start, col, xyz0, xyz, tri, quad, young_tri, nu, stiff_bend)
    for d in (0, 4, 8):
        vd[d::9] += mass / (dt * dt)
    O.set_fixed_bc(row_start, col, vc, vd, np.ascontiguousarray(bc, np.int32))
    icol, dia = O.ilu_pattern0(row_start, col)
    ivc, ivd = O.ilu_copy_value(row_start, icol, col, vc, vd)
    st, _ = O.ilu_decompose(row_start, icol, dia, ivc, ivd)
    assert st == 0
    return vc, vd, icol, dia, ivc, ivd


def rollout(O, row_start, col, xyz0, bc, tri, quad, young_tri, nu, stiff_bend, g, mass, dt, tol, max_iter, nsteps):
    """All positions x_0..x_N (from rest, zero velocity) and the final velocity."""
    x, v = xyz0.copy(), np.zeros_like(xyz0)
    xs = [x.copy()]
    for _ in range(nsteps):
        x, v, _ = cloth_step(O, row_start, col, x, v, xyz0, bc, tri, quad, young_tri, nu, stiff_bend, g, mass, dt,
                             tol, max_iter)
        xs.append(x.copy())
    return xs, v


def rollout_adjoint(O, row_start, col, xyz0, xs, bc, tri, quad, young_tri, nu, stiff_bend, mass, dt, tol, max_iter,
                    xbar, vbar):
    """FP64 CPU adjoint of `rollout` (all states kept): returns dL/dx_0,
    dL/dv_0, dL/dE from xbar = dL/dx_N, vbar = dL/dv_N. Per step, with
    mu = A^-1 P (xbar + vbar/dt): xbar <- xbar - H mu - grad(mu^T A dx),
    vbar <- M mu/dt on free DOFs."""
    xbar, vbar = np.array(xbar, np.float64), np.array(vbar, np.float64)
    Ebar = np.zeros(tri.size // 3)
    free = np.asarray(bc) == 0
    for k in range(len(xs) - 2, -1, -1):
        xk, xk1 = xs[k], xs[k + 1]
        vc, vd, icol, dia, ivc, ivd = step_matrix(O, row_start, col, xyz0, xk, bc, tri, quad, young_tri, nu,
                                                  stiff_bend, mass, dt)
        dxbar = np.where(free, xbar + vbar / dt, 0.0)
        dx = np.where(free, xk1 - xk, 0.0)
        mu, _, _ = O.solve_pcg(row_start, col, vc, vd, icol, dia, ivc, ivd, dxbar, tol, max_iter)
        adjoint_terms(O, xyz0, xk, tri, quad, young_tri, nu, stiff_bend, mu, dx, xbar, Ebar)
        vbar = np.where(free, mass * mu / dt, vbar)
    return xbar, vbar, Ebar
