"""The CPU oracle (plain-C restatement) pinned against the reference.

* against the golden fixtures recorded from the compiled reference
  (tests/golden/make_golden.py), on every machine;
* directly against the reference driver where it is built (this container).
"""
import numpy as np
import pytest

from conftest import golden, rel_err
from oracle import HAVE_REFERENCE_BUILD

NU, RHO, G = 0.3, 1.0, [0.0, 0.0, -1e-3]


def build_system(O, nx, ny, nz, h, young):
    xyz, tet = O.voxel_tet_mesh(nx, ny, nz, h)
    np_ = xyz.size // 3
    ind, psup = O.psup(tet, 4, np_)
    vc, vd, b = np.zeros(psup.size * 9), np.zeros(np_ * 9), np.zeros(np_ * 3)
    assert O.assemble_tet_linear(ind, psup, vc, vd, b, xyz, tet, young, NU, RHO, G) == 0
    bc = np.zeros(np_ * 3, np.int32)
    bc[np.repeat(xyz[2::3] == 0.0, 3)] = 1
    O.set_fixed_bc(ind, psup, vc, vd, bc)
    O.rhs_zero(b, bc)
    col, dia = O.ilu_pattern0(ind, psup)
    ivc, ivd = O.ilu_copy_value(ind, col, psup, vc, vd)
    st, ns = O.ilu_decompose(ind, col, dia, ivc, ivd)
    assert st == 0
    return dict(xyz=xyz, tet=tet, ind=ind, psup=psup, vc=vc, vd=vd, b=b, bc=bc, col=col, dia=dia, ivc=ivc,
                ivd=ivd)


def test_port_matches_tiny_golden(port):
    g = golden("tiny")
    s = build_system(port, 3, 2, 2, 1.0 / 3, g["young"])
    for k in ("xyz", "tet", "ind", "psup", "bc", "col", "dia"):
        assert np.array_equal(s[k], g[k]), k  # integer / exact data: bit-exact
    for k in ("vc", "vd", "b", "ivc", "ivd"):
        assert rel_err(s[k], g[k]) < 1e-13, k
    x, r, hist = port.solve_pcg(s["ind"], s["psup"], s["vc"], s["vd"], s["col"], s["dia"], s["ivc"], s["ivd"],
                                s["b"], 1e-10, 1000)
    assert len(hist) == len(g["hist"])
    assert rel_err(x, g["x"]) < 1e-11
    assert rel_err(hist, g["hist"]) < 1e-9
    fwd = port.ilu_forward(s["ind"], s["col"], s["dia"], s["ivc"], s["ivd"], g["vec"])
    assert rel_err(fwd, g["fwd"]) < 1e-13
    both = port.ilu_backward(s["ind"], s["col"], s["dia"], s["ivc"], fwd)
    assert rel_err(both, g["precond"]) < 1e-13
    mv = port.matvec(s["ind"], s["psup"], s["vc"], s["vd"], np.zeros_like(g["vec"]), 1.0, g["vec"], 0.0)
    assert rel_err(mv, g["matvec"]) < 1e-13


@pytest.mark.parametrize("name", ["cfg1", "cfg1e"])
def test_port_matches_config1_golden(port, name):
    import hashlib
    g = golden(name)
    ntet = 16 ** 3 * 6
    if name == "cfg1":
        young = np.ones(ntet)
    else:
        young = np.exp(np.random.default_rng(0).uniform(np.log(0.1), np.log(10.0), ntet))
    s = build_system(port, 16, 16, 16, 1 / 16, young)
    h = hashlib.sha256()
    h.update(s["ind"].tobytes())
    h.update(s["psup"].tobytes())
    assert h.hexdigest() == str(g["pattern_sha"])
    assert rel_err(s["b"], g["b"]) < 1e-13
    x, r, hist = port.solve_pcg(s["ind"], s["psup"], s["vc"], s["vd"], s["col"], s["dia"], s["ivc"], s["ivd"],
                                s["b"], 1e-10, 1000)
    assert len(hist) - 1 == int(g["n_iter"])  # 81 / 126 iterations, as the reference
    assert rel_err(x, g["x"]) < 1e-10


def test_levels_are_a_valid_schedule(port):
    s = build_system(port, 4, 3, 3, 0.25, np.ones(4 * 3 * 3 * 6))
    n = s["ind"].size - 1
    for backward in (False, True):
        level, order, lstart = port.ilu_levels(s["ind"], s["col"], s["dia"], backward)
        assert np.array_equal(np.sort(order), np.arange(n))
        for i in range(n):
            lo, hi = (s["dia"][i], s["ind"][i + 1]) if backward else (s["ind"][i], s["dia"][i])
            deps = s["col"][lo:hi]
            assert all(level[j] < level[i] for j in deps)
            assert level[i] == (max(level[deps]) + 1 if deps.size else 0)
        # (level, row) ascending
        key = level[order].astype(np.int64) * (n + 1) + order
        assert np.all(np.diff(key) > 0)
        # voxel ordering: forward level = ix + iy + iz
        if not backward:
            ix, iy, iz = np.unravel_index(np.arange(n), (5, 4, 4))
            assert np.array_equal(level, ix + iy + iz)


def test_adjoint_element_term_is_the_energy_derivative(port):
    """-lam^T (K_e/E_e) u_e equals d/dE_e of -lam^T K(E) u (finite difference on a tiny mesh)."""
    xyz, tet = port.voxel_tet_mesh(2, 2, 1, 0.5)
    np_ = xyz.size // 3
    ind, psup = port.psup(tet, 4, np_)
    rng = np.random.default_rng(5)
    young = np.exp(rng.uniform(-1, 1, tet.size // 4))
    u, lam = rng.standard_normal(np_ * 3), rng.standard_normal(np_ * 3)

    def energy(E):
        vc, vd, b = np.zeros(psup.size * 9), np.zeros(np_ * 9), np.zeros(np_ * 3)
        port.assemble_tet_linear(ind, psup, vc, vd, b, xyz, tet, E, NU, RHO, [0, 0, 0])
        Ku = port.matvec(ind, psup, vc, vd, np.zeros(np_ * 3), 1.0, u, 0.0)
        return -lam @ Ku

    d = port.tet_dLdE(xyz, tet, young, NU, u, lam)
    for e in (0, 3, 7):
        Ep, Em = young.copy(), young.copy()
        Ep[e] += 1e-6
        Em[e] -= 1e-6
        fd = (energy(Ep) - energy(Em)) / 2e-6
        assert abs(fd - d[e]) < 1e-6 * max(1.0, abs(d[e]))


@pytest.mark.skipif(not HAVE_REFERENCE_BUILD(), reason="reference source tree not available")
def test_port_equals_reference_directly(port):
    from oracle import reference
    R = reference()
    rng = np.random.default_rng(1)
    for dims in [(2, 2, 2), (3, 4, 2), (5, 3, 4)]:
        nx, ny, nz = dims
        young = np.exp(rng.uniform(np.log(0.1), np.log(10), nx * ny * nz * 6))
        a = build_system(port, nx, ny, nz, 1.0 / nx, young)
        b = build_system(R, nx, ny, nz, 1.0 / nx, young)
        for k in ("xyz", "tet", "ind", "psup", "col", "dia"):
            assert np.array_equal(a[k], b[k]), (dims, k)
        for k in ("vc", "vd", "b", "ivc", "ivd"):
            assert rel_err(a[k], b[k]) < 1e-13, (dims, k)
        xa = port.solve_pcg(a["ind"], a["psup"], a["vc"], a["vd"], a["col"], a["dia"], a["ivc"], a["ivd"], a["b"],
                            1e-10, 500)
        xb = R.solve_pcg(b["ind"], b["psup"], b["vc"], b["vd"], b["col"], b["dia"], b["ivc"], b["ivd"], b["b"],
                         1e-10, 500)
        assert len(xa[2]) == len(xb[2])
        assert rel_err(xa[0], xb[0]) < 1e-11
        # max-iteration exhaustion appends the final |r| (lsitrsol.h:142-147)
        ya = port.solve_pcg(a["ind"], a["psup"], a["vc"], a["vd"], a["col"], a["dia"], a["ivc"], a["ivd"], a["b"],
                            1e-30, 3)
        yb = R.solve_pcg(b["ind"], b["psup"], b["vc"], b["vd"], b["col"], b["dia"], b["ivc"], b["ivd"], b["b"],
                         1e-30, 3)
        assert len(ya[2]) == len(yb[2]) == 5 and ya[2][-1] == ya[2][-2]
        # Solve_CG
        ca = port.solve_cg(a["ind"], a["psup"], a["vc"], a["vd"], a["b"], 1e-8, 2000)
        cb = R.solve_cg(b["ind"], b["psup"], b["vc"], b["vd"], b["b"], 1e-8, 2000)
        # unpreconditioned CG amplifies ulp-level differences in K; the reference's
        # own cross-back-end test allows +-10 iterations (test_cpp/eigen/ls_sparse_test.cpp:172-173)
        assert abs(len(ca[2]) - len(cb[2])) <= 10 and rel_err(ca[0], cb[0]) < 1e-6
        # MatVec with beta != 0 and the f32 instantiation
        x = rng.standard_normal(a["b"].size)
        y0 = rng.standard_normal(a["b"].size)
        assert rel_err(port.matvec(a["ind"], a["psup"], a["vc"], a["vd"], y0, 0.7, x, -1.3),
                       R.matvec(b["ind"], b["psup"], b["vc"], b["vd"], y0, 0.7, x, -1.3)) < 1e-14
        f = lambda v: v.astype(np.float32)  # noqa: E731
        assert rel_err(port.matvec(a["ind"], a["psup"], f(a["vc"]), f(a["vd"]), f(y0), 0.5, f(x), 2.0),
                       R.matvec(b["ind"], b["psup"], f(b["vc"]), f(b["vd"]), f(y0), 0.5, f(x), 2.0)) < 1e-6


@pytest.mark.skipif(not HAVE_REFERENCE_BUILD(), reason="reference source tree not available")
def test_merge_and_missing_slot_match_reference(port):
    from oracle import reference
    R = reference()
    xyz, tet = port.voxel_tet_mesh(2, 2, 2, 0.5)
    np_ = xyz.size // 3
    ind, psup = port.psup(tet, 4, np_)
    rng = np.random.default_rng(3)
    emat = rng.standard_normal(16 * 9)
    outs = []
    for O in (port, R):
        vc, vd = np.zeros(psup.size * 9), np.zeros(np_ * 9)
        assert O.merge(ind, psup, vc, vd, tet[4:8], emat) == 0
        outs.append((vc, vd))
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])
    far = np.array([0, np_ - 1, 1, 2], np.uint32)  # node 0 and the far corner are not adjacent
    for O in (port, R):
        vc, vd = np.zeros(psup.size * 9), np.zeros(np_ * 9)
        assert O.merge(ind, psup, vc, vd, far, emat) == 1
