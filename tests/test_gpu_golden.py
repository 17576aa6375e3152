"""Large configurations against samples recorded from the reference's own
Solve_PCG run to 1e-12 (tests/golden/make_golden.py): pattern hash (bit-exact),
iteration count to 1e-10, sampled solution entries and norms."""
import hashlib

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu

CONFIGS = {
    # name: (nx, ny, nz, h, E range, seed)
    "cfg2": (64, 64, 64, 1 / 64, (0.1, 10.0), 2),
    "cfg4": (48, 48, 48, 1 / 48, (0.5, 2.0), 4),
    "cfg3": (128, 128, 64, 1 / 128, (0.1, 10.0), 3),
}


def iterations_to(hist, tol):
    h = np.asarray(hist)
    return int(np.nonzero(h / h[0] < tol)[0][0])


@pytest.fixture(scope="module", params=list(CONFIGS))
def big(request, gpu):
    import torch
    import delfem2_gb300 as D
    nx, ny, nz, h, er, seed = CONFIGS[request.param]
    a = D.voxel_problem_arrays(nx, ny, nz, h, seed=seed, e_range=er)
    P = D.StaticElasticProblem(a)
    b = P.assemble(b=torch.zeros(a["np"] * 3, dtype=torch.float64, device="cuda"))
    assert P.factor()
    yield request.param, a, P, b
    del P
    torch.cuda.empty_cache()


def test_pattern_and_inputs_match_reference(big):
    name, a, P, b = big
    g = golden(name)
    hsh = hashlib.sha256()
    hsh.update(a["psup_ind"].tobytes())
    hsh.update(a["psup"].tobytes())
    assert hsh.hexdigest() == str(g["pattern_sha"])
    bn = b.cpu().numpy()
    assert abs(np.linalg.norm(bn) - float(g["b_norm"])) < 1e-12 * float(g["b_norm"])
    vc, vd = P.K.get_values()
    ksum = np.abs(vc).sum() + np.abs(vd).sum()
    assert abs(ksum - float(g["K_abs_sum"])) < 1e-11 * float(g["K_abs_sum"])


def test_fp64_solve_matches_reference(big):
    import torch
    import delfem2_gb300 as D
    name, a, P, b = big
    g = golden(name)
    r = b.clone()
    x = torch.zeros_like(b)
    hist = D.Solve_PCG(r, x, 1e-12, 5000, P.K, P.ilu)
    # iteration count to 1e-10 of the same algorithm: within 2 of the reference
    assert abs(iterations_to(hist, 1e-10) - iterations_to(g["hist"], 1e-10)) <= 2
    xs = x.cpu().numpy()[g["idx"]]
    assert np.abs(xs - g["x_sample"]).max() <= 1e-8 * np.abs(g["x_sample"]).max()
    assert abs(float(torch.linalg.norm(x)) - float(g["x_norm"])) <= 1e-9 * float(g["x_norm"])


@pytest.mark.parametrize("method", ["reliable", "restart"])
def test_mixed_solve_agrees_with_reference_to_1e8(big, method):
    import torch
    import delfem2_gb300 as D
    name, a, P, b = big
    g = golden(name)
    x = torch.zeros_like(b)
    st = D.Solve_PCG_Mixed(b, x, 1e-10, P.K, P.ilu, inner_tol=1e-4, method=method)
    assert st.rel_residual < 1e-10
    xs = x.cpu().numpy()[g["idx"]]
    err = np.abs(xs - g["x_sample"]).max() / np.abs(g["x_sample"]).max()
    print(f"{name} {method}: mixed {st.iterations} inner / {st.outer} outer, rel res {st.rel_residual:.2e}, "
          f"sample err vs reference {err:.2e}")
    assert err <= 1e-8
