"""Scalar (ndim 1) and 2x2 (ndim 2) block systems shared by the oracle tests,
the GPU tests and tests/golden/make_golden.py.

* Poisson on tets (ndim 1): the n^3 voxel block (6 tets per voxel, unit cube),
  alpha = 1, source = 1; nodes on z = 0 fixed at 0 and on z = 1 fixed at 1,
  the fixed values lifted into the right-hand side through the assembly's
  `val` argument (as 618_Fem3Tet/main.cpp:56-139 does with aVal).
* Poisson on triangles (ndim 1): the cloth square's triangle mesh in the xy
  plane, the same boundary values on y = 0 / y = 1.
* 2-D linear solid (ndim 2): the same triangle mesh, myu = 1, lambda = 2,
  rho = 1, g = (0, -1), the x = 0 edge clamped.
"""
import numpy as np

POISSON = dict(alpha=1.0, source=1.0)
SOLID2 = dict(myu=1.0, lam=2.0, rho=1.0, gx=0.0, gy=-1.0)


def poisson_tet(O, n=8):
    xyz, tet = O.voxel_tet_mesh(n, n, n, 1.0 / n)
    np_ = xyz.size // 3
    ind, psup = O.psup(tet, 4, np_)
    z = xyz.reshape(-1, 3)[:, 2]
    bc = ((z < 1e-9) | (z > 1 - 1e-9)).astype(np.int32)
    val = np.where(z > 1 - 1e-9, 1.0, 0.0)
    vc, vd, b = O.assemble_poisson_tet(ind, psup, xyz, tet, POISSON["alpha"], POISSON["source"], val)
    O.nd_set_fixed_bc(1, ind, psup, vc, vd, bc)
    b[bc != 0] = 0.0
    return dict(ndim=1, xyz=xyz, elem=tet, nnoel=4, ind=ind, psup=psup, vc=vc, vd=vd, b=b, bc=bc, val=val)


def tri_mesh(ndiv):
    """The cloth square's nodes (xy) and triangles, from the restatement of SetClothShape_Square."""
    from oracle import port
    from oracle.cloth import cloth_square
    xyz0, tri, _ = cloth_square(port(), ndiv, 1.0)
    xy = np.ascontiguousarray(xyz0.reshape(-1, 3)[:, :2]).ravel()
    return xy, tri


def poisson_tri2(O, ndiv=16):
    xy, tri = tri_mesh(ndiv)
    np_ = xy.size // 2
    ind, psup = O.psup(tri, 3, np_)
    y = xy.reshape(-1, 2)[:, 1]
    bc = ((y < 1e-9) | (y > 1 - 1e-9)).astype(np.int32)
    val = np.where(y > 1 - 1e-9, 1.0, 0.0)
    vc, vd, b = O.assemble_tri2(1, ind, psup, xy, tri, (POISSON["alpha"], POISSON["source"]), val)
    O.nd_set_fixed_bc(1, ind, psup, vc, vd, bc)
    b[bc != 0] = 0.0
    return dict(ndim=1, xy=xy, elem=tri, nnoel=3, ind=ind, psup=psup, vc=vc, vd=vd, b=b, bc=bc, val=val)


def solid_tri2(O, ndiv=16):
    xy, tri = tri_mesh(ndiv)
    np_ = xy.size // 2
    ind, psup = O.psup(tri, 3, np_)
    x = xy.reshape(-1, 2)[:, 0]
    bc = np.repeat((x < 1e-9).astype(np.int32), 2)
    s = SOLID2
    vc, vd, b = O.assemble_tri2(2, ind, psup, xy, tri, (s["myu"], s["lam"], s["rho"], s["gx"], s["gy"]))
    O.nd_set_fixed_bc(2, ind, psup, vc, vd, bc)
    b[bc != 0] = 0.0
    return dict(ndim=2, xy=xy, elem=tri, nnoel=3, ind=ind, psup=psup, vc=vc, vd=vd, b=b, bc=bc, val=None)


SYSTEMS = {"poisson_tet": poisson_tet, "poisson_tri2": poisson_tri2, "solid_tri2": solid_tri2}


def factor(O, s, k):
    """ILU(k) pattern (Initialize_ILUk), CopyValue and Decompose: (row_start, col, dia, vcrs, vdia)."""
    rs, col, dia = O.ilu_pattern_k(s["ind"], s["psup"], k)
    ivc, ivd = O.nd_ilu_copy_value(s["ndim"], s["ind"], s["psup"], s["vc"], s["vd"], k, rs, col)
    st, ivc, ivd = O.nd_ilu_decompose(s["ndim"], rs, col, dia, ivc, ivd)
    assert st == 0
    return rs, col, dia, ivc, ivd
