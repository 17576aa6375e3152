"""Cloth part of the CPU oracle pinned against the reference.

* against tests/golden/cloth.npz, recorded from the compiled reference
  (WdWddW_CST, MakePositiveDefinite_Sim22, WdWddW_Bend, MergeLinSys_Cloth and
  StepTime_InternalDynamicsILU), on every machine;
* directly against the reference driver where it is built;
* element derivatives against central differences of the element energy.
"""
import numpy as np
import pytest

from conftest import golden, rel_err
from oracle import HAVE_REFERENCE_BUILD
from oracle import cloth as CL


@pytest.fixture(scope="module")
def G():
    return golden("cloth")


def test_mesh_matches_golden(port, G):
    xyz0, tri, quad = CL.cloth_square(port, 16)
    assert np.array_equal(xyz0, G["xyz0"]) and np.array_equal(tri, G["tri"]) and np.array_equal(quad, G["quad"])
    ind, psup = port.psup(quad, 4, xyz0.size // 3)
    assert np.array_equal(ind, G["ind"]) and np.array_equal(psup, G["psup"])
    # sizes of the 256x256-vertex sheet of the cloth workload
    n = 255
    assert ((n + 1) ** 2, 2 * n * n, n * n + 2 * n * (n - 1)) == (65536, 130050, 194565)


def test_elements_match_golden(port, G):
    for i in range(G["cst_C"].shape[0]):
        W, dW, ddW = CL.wdwddw_cst(port, G["cst_C"][i], G["cst_c"][i], *G["cst_lm"][i])
        assert abs(W - G["cst_W"][i]) <= 1e-13 * abs(G["cst_W"][i]) + 1e-300
        assert rel_err(dW, G["cst_dW"][i]) < 1e-13
        assert rel_err(ddW, G["cst_ddW"][i]) < 1e-13
    for i in range(G["bend_C"].shape[0]):
        W, dW, ddW = CL.wdwddw_bend(port, G["bend_C"][i], G["bend_c"][i], 1e-3)
        assert abs(W - G["bend_W"][i]) <= 1e-13 * abs(G["bend_W"][i])
        assert rel_err(dW, G["bend_dW"][i]) < 1e-13
        assert rel_err(ddW, G["bend_ddW"][i]) < 1e-13
    for s2, s3 in zip(G["pd_s2"], G["pd_s3"]):
        assert np.allclose(CL.make_pd_sim22(port, s2), s3, rtol=1e-13, atol=1e-15)


def test_assemble_matches_golden(port, G):
    W, vc, vd, dW = CL.cloth_assemble(port, G["ind"], G["psup"], G["xyz0"], G["asm_xyz"], G["tri"], G["quad"],
                                      G["young_rand"], 0.3, 1e-3)
    assert abs(W - float(G["asm_W"])) < 1e-13 * abs(float(G["asm_W"]))
    for a, b in ((vc, G["asm_vc"]), (vd, G["asm_vd"]), (dW, G["asm_dW"])):
        assert rel_err(a, b) < 1e-13


@pytest.mark.parametrize("tag", ["own", "rand"])
def test_steps_match_golden(port, G, tag):
    """StepTime_InternalDynamicsILU with its own (uniform E, 1e-4, 100) and the
    per-triangle-E step with PCG to 1e-8: ten steps each from rest."""
    young = np.full(G["tri"].size // 3, 1e3) if tag == "own" else G["young_rand"]
    tol, mi = (1e-4, 100) if tag == "own" else (1e-8, 1000)
    x, v = G["xyz0"].copy(), np.zeros_like(G["xyz0"])
    mass = 1.0 / (x.size // 3)
    for k in range(G[f"step_{tag}_x"].shape[0]):
        x, v, nh = CL.cloth_step(port, G["ind"], G["psup"], x, v, G["xyz0"], G["bc"], G["tri"], G["quad"], young,
                                 0.3, 1e-3, np.array([0, 0, -10.0]), mass, 0.01, tol, mi)
        disp = G[f"step_{tag}_x"][k] - G["xyz0"]
        assert rel_err(x - G["xyz0"], disp) < 1e-10, k
        if tag == "rand":
            assert nh == G["step_rand_nhist"][k]
    assert rel_err(v, G[f"step_{tag}_v"]) < 1e-9
    # pinned corners never move
    fixed = G["bc"] != 0
    assert np.array_equal(x[fixed], G["xyz0"][fixed])


def test_element_gradients_are_energy_derivatives(port):
    rng = np.random.default_rng(3)
    h = 1e-6
    for _ in range(4):
        Cm = rng.standard_normal((3, 3))
        c = Cm + 0.2 * rng.standard_normal((3, 3))
        W, dW, ddW = CL.wdwddw_cst(port, Cm, c, 0.9, 0.6)
        fd = np.zeros((3, 3))
        for a in range(3):
            for d in range(3):
                cp, cm = c.copy(), c.copy()
                cp[a, d] += h
                cm[a, d] -= h
                fd[a, d] = (CL.wdwddw_cst(port, Cm, cp, 0.9, 0.6)[0] - CL.wdwddw_cst(port, Cm, cm, 0.9, 0.6)[0]) / (
                    2 * h)
        assert rel_err(dW, fd) < 1e-6
        Cq = rng.standard_normal((4, 3))
        cq = Cq + 0.2 * rng.standard_normal((4, 3))
        W, dW, ddW = CL.wdwddw_bend(port, Cq, cq, 1e-2)
        # quadratic bending (fem_quadratic_bending.cpp:84-106): constant H, dW = H c
        # and the reported W = c.H.c (twice the energy whose gradient dW is)
        Hm = ddW.transpose(0, 2, 1, 3).reshape(12, 12)
        u = cq.ravel()
        assert rel_err(Hm @ u, dW.ravel()) < 1e-12
        assert abs(u @ Hm @ u - W) < 1e-12 * abs(W)
        # a planar rest pair (0 and 1 on either side of the edge 2-3) has zero
        # bending force at rest: H C = 0
        Q, _ = np.linalg.qr(rng.standard_normal((3, 3)))
        Cp = np.array([[0.3, 0.7, 0.0], [0.6, -0.8, 0.0], [0.0, 0.0, 0.0], [1.0, 0.0, 0.0]]) @ Q.T
        assert np.abs(CL.wdwddw_bend(port, Cp, Cp, 1e-2)[1]).max() < 1e-14


def test_pd_projection_is_positive_semidefinite(port):
    rng = np.random.default_rng(9)
    for _ in range(200):
        s3 = CL.make_pd_sim22(port, rng.standard_normal(3))
        S = np.array([[s3[0], s3[2]], [s3[2], s3[1]]])
        assert np.linalg.eigvalsh(S).min() > -1e-12


@pytest.mark.skipif(not HAVE_REFERENCE_BUILD(), reason="reference source tree not available")
def test_port_equals_reference_directly(port):
    from oracle import reference
    R = reference()
    rng = np.random.default_rng(21)
    for _ in range(50):
        Cm = rng.standard_normal((3, 3))
        c = Cm + 0.3 * rng.standard_normal((3, 3))
        for a, b in zip(CL.wdwddw_cst(port, Cm, c, 1.3, 0.7), CL.wdwddw_cst(R, Cm, c, 1.3, 0.7)):
            assert rel_err(a, b) < 1e-13
    ndiv = 9
    x0, tri, quad = CL.cloth_square(port, ndiv)
    xr, tr, qr = CL.cloth_square(R, ndiv)
    assert np.array_equal(x0, xr) and np.array_equal(tri, tr) and np.array_equal(quad, qr)
    np_ = x0.size // 3
    ind, psup = port.psup(quad, 4, np_)
    bc = np.zeros(np_ * 3, np.int32)
    bc[0:3] = 1
    bc[ndiv * 3:ndiv * 3 + 3] = 1
    young = np.exp(rng.uniform(np.log(5e2), np.log(2e3), tri.size // 3))
    xa, va = x0.copy(), np.zeros_like(x0)
    xb, vb = x0.copy(), np.zeros_like(x0)
    for _ in range(4):
        xa, va, na = CL.cloth_step(port, ind, psup, xa, va, x0, bc, tri, quad, young, 0.3, 1e-3, [0, 0, -10.0],
                                   1.0 / np_, 0.01, 1e-8, 1000)
        xb, vb, nb = CL.cloth_step(R, ind, psup, xb, vb, x0, bc, tri, quad, young, 0.3, 1e-3, [0, 0, -10.0],
                                   1.0 / np_, 0.01, 1e-8, 1000)
        assert na == nb
    assert rel_err(xa - x0, xb - x0) < 1e-12 and rel_err(va, vb) < 1e-12


# ---- adjoint (no reference counterpart): the oracle's terms against central
# differences of the reference-pinned element functions ----

def _fd(f, x, h):
    x = np.array(x, np.float64)
    out = []
    for i in range(x.size):
        xp, xm = x.copy(), x.copy()
        xp.flat[i] += h
        xm.flat[i] -= h
        out.append((np.asarray(f(xp)) - np.asarray(f(xm))) / (2 * h))
    return np.array(out)


def test_pd_jacobian_matches_differences(port):
    rng = np.random.default_rng(4)
    branches = set()
    for _ in range(300):
        s = rng.standard_normal(3)
        b, e = 0.5 * (s[0] + s[1]), np.hypot(0.5 * (s[0] - s[1]), s[2])
        if min(abs(b - e), abs(b + e)) < 1e-3:
            continue  # too close to a branch switch for differences
        branches.add((b - e > 0, b + e < 0))
        J = CL.pd_sim22_jac(port, s)
        fd = _fd(lambda v: CL.make_pd_sim22(port, v), s, 1e-7).T
        assert np.abs(J - fd).max() < 1e-6 * max(1.0, np.abs(fd).max())
    assert len(branches) == 3  # kept, zeroed and rank-1 cases all met


def _sheet(port, ndiv, rng, amp):
    x0, tri, quad = CL.cloth_square(port, ndiv)
    ind, psup = port.psup(quad, 4, x0.size // 3)
    x = x0 + amp / ndiv * rng.standard_normal(x0.size)
    return x0, tri, quad, ind, psup, x


def test_adjoint_terms_match_differences(port):
    rng = np.random.default_rng(8)
    x0, tri, quad, ind, psup, x = _sheet(port, 3, rng, 0.3)
    young = rng.uniform(500, 2000, tri.size // 3)
    nu, kb = 0.3, 1e-3
    mu, dx = rng.standard_normal(x.size), rng.standard_normal(x.size)
    xbar, Ebar = np.zeros(x.size), np.zeros(tri.size // 3)
    CL.adjoint_terms(port, x0, x, tri, quad, young, nu, kb, mu, dx, xbar, Ebar)

    def grad(xx, E=young):
        return CL.cloth_assemble(port, ind, psup, x0, xx, tri, quad, E, nu, kb)[3]

    def phi(xx, E=young):
        _, vc, vd, _ = CL.cloth_assemble(port, ind, psup, x0, xx, tri, quad, E, nu, kb)
        Ad = port.matvec(ind, psup, vc, vd, np.zeros_like(dx), 1.0, dx, 0.0)
        return mu @ Ad

    h = 1e-6 / 3
    Hmu = (grad(x + h * mu) - grad(x - h * mu)) / (2 * h)
    gphi = _fd(phi, x, h)
    want = -Hmu - gphi
    assert rel_err(xbar, want) < 1e-6
    # per-triangle modulus: d/dE_t of (mu . dW + mu^T A dx)
    for t in range(0, tri.size // 3, 3):
        def s(E):
            yy = young.copy()
            yy[t] = E
            return mu @ grad(x, yy) + phi(x, yy)
        hE = 1e-4 * young[t]
        fd = (s(young[t] + hE) - s(young[t] - hE)) / (2 * hE)
        assert abs(Ebar[t] + fd) < 1e-6 * max(abs(fd), np.abs(Ebar).max())


def test_rollout_adjoint_matches_differences(port):
    """dL/dE of L = |x_N - x*|^2 / 2 over three backward-Euler steps (PCG to
    1e-14 so that the discrete map is the differentiated one)."""
    rng = np.random.default_rng(12)
    ndiv = 4
    x0, tri, quad = CL.cloth_square(port, ndiv)
    np_ = x0.size // 3
    ind, psup = port.psup(quad, 4, np_)
    bc = np.zeros(np_ * 3, np.int32)
    bc[0:3] = 1
    bc[ndiv * 3:ndiv * 3 + 3] = 1
    young = rng.uniform(50, 200, tri.size // 3)
    target = x0 + 0.05 * rng.standard_normal(x0.size)
    args = dict(nu=0.3, stiff_bend=1e-3, mass=1.0 / np_, dt=0.01, tol=1e-14, max_iter=2000)

    def loss(E):
        xs, v = CL.rollout(port, ind, psup, x0, bc, tri, quad, E, args["nu"], args["stiff_bend"], [0, 0, -10.0],
                           args["mass"], args["dt"], args["tol"], args["max_iter"], 3)
        return 0.5 * np.sum((xs[-1] - target) ** 2), xs

    L, xs = loss(young)
    xbar, vbar, Ebar = CL.rollout_adjoint(port, ind, psup, x0, xs, bc, tri, quad, young, args["nu"],
                                          args["stiff_bend"], args["mass"], args["dt"], args["tol"],
                                          args["max_iter"], xs[-1] - target, np.zeros_like(x0))
    for t in rng.choice(tri.size // 3, 6, replace=False):
        h = 1e-5 * young[t]
        yp, ym = young.copy(), young.copy()
        yp[t] += h
        ym[t] -= h
        fd = (loss(yp)[0] - loss(ym)[0]) / (2 * h)
        assert abs(Ebar[t] - fd) < 1e-5 * np.abs(Ebar).max(), (t, Ebar[t], fd)
