"""Inputs of the dynamic linear-tet assemblers (backward Euler, stiffness-
warped backward Euler, Newmark-beta) shared by the oracle tests, the GPU tests
and tests/golden/make_golden.py: the 5^3 voxel block (unit cube), seeded
displacements, velocities, accelerations and per-node rotations (Rodrigues'
formula of a seeded axis and angle), as 603_Fem3DStiffwarp and 618_Fem3Tet
drive them."""
import numpy as np

MAT = dict(myu=1.0, lam=2.0, rho=1.5, g=np.array([0.0, 0.0, -9.8]), dt=0.01, gamma=0.6, beta=0.3)


def rotations(np_, seed=4):
    rng = np.random.default_rng(seed)
    out = np.zeros((np_, 3, 3))
    for k in range(np_):
        w = rng.standard_normal(3)
        w /= np.linalg.norm(w)
        th = rng.uniform(0.0, np.pi)
        W = np.array([[0, -w[2], w[1]], [w[2], 0, -w[0]], [-w[1], w[0], 0]])
        out[k] = np.eye(3) + np.sin(th) * W + (1 - np.cos(th)) * W @ W
    return out.ravel()


def inputs(O, n=5):
    xyz, tet = O.voxel_tet_mesh(n, n, n, 1.0 / n)
    np_ = xyz.size // 3
    ind, psup = O.psup(tet, 4, np_)
    rng = np.random.default_rng(3)
    return dict(xyz=xyz, tet=tet, ind=ind, psup=psup, u=0.01 * rng.standard_normal(np_ * 3),
                v=0.1 * rng.standard_normal(np_ * 3), acc=rng.standard_normal(np_ * 3), rot=rotations(np_))


def assemble(O, s, kind):
    m = MAT
    if kind == "newmark":
        return O.assemble_tet_newmark(s["ind"], s["psup"], s["xyz"], s["tet"], m["myu"], m["lam"], m["rho"], m["g"],
                                      m["dt"], m["gamma"], m["beta"], s["u"], s["v"], s["acc"])
    return O.assemble_tet_beuler(s["ind"], s["psup"], s["xyz"], s["tet"], m["myu"], m["lam"], m["rho"], m["g"],
                                 m["dt"], s["u"], s["v"], s["rot"] if kind == "warp" else None)


KINDS = ("beuler", "warp", "newmark")


def hex_inputs(O, nx=4, ny=3, nz=5):
    """A jittered nx x ny x nz hex grid (spacing 1/4, interior nodes moved by up to 0.2 of it) with a seeded
    displacement: distorted hexes, where the quadrature rule matters."""
    from oracle.oracle import hex_grid
    xyz, hexa = hex_grid(nx, ny, nz, 0.25, seed=2, jitter=0.2)
    np_ = xyz.size // 3
    ind, psup = O.psup(hexa, 8, np_)
    return dict(xyz=xyz, hex=hexa, ind=ind, psup=psup, u=0.01 * np.random.default_rng(1).standard_normal(np_ * 3))


def assemble_hex(O, s):
    m = MAT
    return O.assemble_hex_q1(s["ind"], s["psup"], s["xyz"], s["hex"], m["myu"], m["lam"], m["rho"], m["g"], s["u"])
