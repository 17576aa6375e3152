"""Implicit cloth on the GPU against the oracle (pinned to the reference).

Tolerances (FP64 throughout unless stated):
  assembly (K, dW, W) vs the oracle              1e-12 relative;
  ten steps, PCG to 1e-8, vs the golden run     1e-7 relative displacement
    (two 1e-8 solves differ by their error, iterate order is the same);
  the reference's own step settings (1e-4, 100)  1e-6;
  mixed-precision steps vs FP64 steps            1e-6;
  adjoint element terms vs the oracle            1e-11;
  rollout gradient vs the oracle CPU adjoint     1e-8 (solves to 1e-14);
  rollout gradient vs central differences        1e-5 of max |dL/dE|.
"""
import numpy as np
import pytest

from conftest import golden, rel_err
from oracle import cloth as CL

pytestmark = pytest.mark.gpu

NU, KB, G3, DT = 0.3, 1e-3, (0.0, 0.0, -10.0), 0.01


def _cloth(ndiv):
    from delfem2_gb300 import cloth as DC
    xyz0, _, tri, quad = DC.SetClothShape_Square(ndiv, 1.0)
    return DC.Cloth(xyz0, tri, quad), DC.pin_two_corners(ndiv)


def test_mesh_matches_oracle(gpu, port):
    from delfem2_gb300 import cloth as DC
    for ndiv in (1, 2, 7, 16):
        a = DC.SetClothShape_Square(ndiv, 1.0)
        b = CL.cloth_square(port, ndiv)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[2], b[1]) and np.array_equal(a[3], b[2])


def test_merge_matches_oracle(gpu, port):
    G = golden("cloth")
    c, _ = _cloth(16)
    c.mat.setZero()
    dW = np.zeros(c.np * 3)
    W = c.MergeLinSys_Cloth(G["asm_xyz"], G["young_rand"], NU, KB, dW)
    vc, vd = c.mat.get_values()
    assert abs(W - float(G["asm_W"])) < 1e-12 * abs(float(G["asm_W"]))
    assert rel_err(vc, G["asm_vc"]) < 1e-12 and rel_err(vd, G["asm_vd"]) < 1e-12
    assert rel_err(dW, G["asm_dW"]) < 1e-12
    tc, qc = c.ncolor
    assert 1 <= tc <= 16 and 1 <= qc <= 32


@pytest.mark.parametrize("tag", ["rand", "own"])
def test_steps_match_golden(gpu, tag):
    G = golden("cloth")
    c, bc = _cloth(16)
    assert np.array_equal(bc, G["bc"])
    young = G["young_rand"] if tag == "rand" else np.full(c.ntri, 1e3)
    tol, mi = (1e-8, 1000) if tag == "rand" else (1e-4, 100)
    x, v = c.xyz0.copy(), np.zeros(c.np * 3)
    for k in range(G[f"step_{tag}_x"].shape[0]):
        st = c.StepTime_InternalDynamicsILU(x, v, bc, young, NU, KB, G3, 1.0 / c.np, DT, tol, mi)
        ref = G[f"step_{tag}_x"][k] - c.xyz0
        assert rel_err(x - c.xyz0, ref) < (1e-7 if tag == "rand" else 1e-6), k
        if tag == "rand":
            assert abs(int(st.iterations) - int(G["step_rand_nhist"][k] - 1)) <= 1
    assert np.array_equal(x[bc != 0], c.xyz0[bc != 0])


def test_mixed_steps_close_to_fp64(gpu):
    from delfem2_gb300 import cloth as DC
    G = golden("cloth")
    c, bc = _cloth(16)
    res = []
    for solver in (DC.PCG_F64, DC.PCG_MIXED):
        x, v = c.xyz0.copy(), np.zeros(c.np * 3)
        for _ in range(5):
            c.StepTime_InternalDynamicsILU(x, v, bc, G["young_rand"], NU, KB, G3, 1.0 / c.np, DT, 1e-10, 2000,
                                           solver)
        res.append(x - c.xyz0)
    assert rel_err(res[1], res[0]) < 1e-6


def test_adjoint_terms_match_oracle(gpu, port):
    rng = np.random.default_rng(5)
    c, _ = _cloth(9)
    x = c.xyz0 + 0.3 / 9 * rng.standard_normal(c.np * 3)
    young = rng.uniform(500, 2000, c.ntri)
    mu, dx = rng.standard_normal(c.np * 3), rng.standard_normal(c.np * 3)
    xb0, eb0 = rng.standard_normal(c.np * 3), rng.standard_normal(c.ntri)
    xb, eb = xb0.copy(), eb0.copy()
    c.adjoint_terms(x, young, NU, KB, mu, dx, xb, eb)
    xr, er = xb0.copy(), eb0.copy()
    CL.adjoint_terms(port, c.xyz0, x, c.tri, c.quad, young, NU, KB, mu, dx, xr, er)
    assert rel_err(xb - xb0, xr - xb0) < 1e-11
    assert rel_err(eb - eb0, er - eb0) < 1e-11


def _small_problem(ndiv=5, seed=12):
    rng = np.random.default_rng(seed)
    c, bc = _cloth(ndiv)
    young = rng.uniform(50, 200, c.ntri)
    target = c.xyz0 + 0.05 * rng.standard_normal(c.np * 3)
    return c, bc, young, target


def test_rollout_gradient_matches_oracle_and_differences(gpu, port):
    c, bc, young, target = _small_problem()
    nsteps, every = 5, 2  # segments [0,2) [2,4) [4,5)
    mass = 1.0 / c.np
    x, v = c.xyz0.copy(), np.zeros(c.np * 3)
    c.rollout(x, v, bc, young, NU, KB, G3, mass, DT, 1e-14, 3000, nsteps, every)
    xbar, vbar, gE = x - target, np.zeros(c.np * 3), np.zeros(c.ntri)
    c.rollout_adjoint(xbar, vbar, gE)
    ind, psup = port.psup(c.quad, 4, c.np)
    xs, _ = CL.rollout(port, ind, psup, c.xyz0, bc, c.tri, c.quad, young, NU, KB, G3, mass, DT, 1e-14, 3000, nsteps)
    assert rel_err(x - c.xyz0, xs[-1] - c.xyz0) < 1e-10
    xr, vr, er = CL.rollout_adjoint(port, ind, psup, c.xyz0, xs, bc, c.tri, c.quad, young, NU, KB, mass, DT, 1e-14,
                                    3000, xs[-1] - target, np.zeros(c.np * 3))
    assert rel_err(gE, er) < 1e-8
    assert rel_err(xbar, xr) < 1e-8 and rel_err(vbar, vr) < 1e-8

    def loss(E):
        xx, vv = c.xyz0.copy(), np.zeros(c.np * 3)
        c.rollout(xx, vv, bc, E, NU, KB, G3, mass, DT, 1e-14, 3000, nsteps, 0)
        return 0.5 * np.sum((xx - target) ** 2)

    rng = np.random.default_rng(1)
    for t in rng.choice(c.ntri, 8, replace=False):
        h = 1e-5 * young[t]
        yp, ym = young.copy(), young.copy()
        yp[t] += h
        ym[t] -= h
        fd = (loss(yp) - loss(ym)) / (2 * h)
        assert abs(gE[t] - fd) < 1e-5 * np.abs(gE).max(), (t, gE[t], fd)


def test_checkpoint_interval_does_not_change_the_gradient(gpu):
    """Recomputed segments replay the forward run exactly (deterministic
    kernels), so every checkpoint interval gives the same bits."""
    c, bc, young, target = _small_problem(4, 3)
    out = []
    for every in (1, 3, 7, 20):
        x, v = c.xyz0.copy(), np.zeros(c.np * 3)
        c.rollout(x, v, bc, young, NU, KB, G3, 1.0 / c.np, DT, 1e-10, 500, 7, every)
        xbar, vbar, gE = x - target, np.zeros(c.np * 3), np.zeros(c.ntri)
        c.rollout_adjoint(xbar, vbar, gE)
        out.append(gE)
    for g in out[1:]:
        assert np.array_equal(g, out[0])


def test_torch_autograd_function(gpu):
    import torch
    from delfem2_gb300 import cloth as DC
    c, bc, young, target = _small_problem(4, 9)
    ro = DC.ClothRollout(c, bc, nu=NU, stiff_bend=KB, gravity=G3, dt=DT, tol=1e-12, max_iter=2000, nsteps=4,
                         ckpt_every=2)
    E = torch.tensor(young, device="cuda", requires_grad=True)
    xN = ro.apply(E)
    L = 0.5 * torch.sum((xN - torch.tensor(target, device="cuda")) ** 2)
    L.backward()
    x, v, _ = ro.forward(young)
    assert rel_err(xN.detach().cpu().numpy() - c.xyz0, x - c.xyz0) < 1e-12
    xbar, vbar, gE = x - target, np.zeros(c.np * 3), np.zeros(c.ntri)
    c.rollout_adjoint(xbar, vbar, gE)  # reverses the host-side rollout of ro.forward
    assert rel_err(E.grad.cpu().numpy(), gE) < 1e-12


def test_cloth_errors_are_reported(gpu):
    from delfem2_gb300 import _native as N
    c, bc = _cloth(3)
    with pytest.raises(N.Dfm2gError):
        c.rollout_adjoint(np.zeros(c.np * 3), np.zeros(c.np * 3), np.zeros(c.ntri))  # no rollout yet
    x, v = c.xyz0.copy(), np.zeros(c.np * 3)
    with pytest.raises(N.Dfm2gError):
        c.StepTime_InternalDynamicsILU(x, v, bc, np.full(c.ntri, 1e3), NU, KB, G3, 1.0 / c.np, 0.0)  # dt = 0
