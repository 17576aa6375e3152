"""Solve_PBiCGStab (include/delfem2/vecxitrsol.h:350-437) in the CPU oracle,
pinned against the reference on a non-symmetric system (each off-diagonal
block of the 8^3 tet K scaled by a seeded factor in [0.7, 1.3]): the fixture
tests/golden/bicgstab.npz, and directly where the reference is built.
Relative-residual history and x identical to 1e-12 (same operation order)."""
import numpy as np
import pytest

from conftest import golden, rel_err
from oracle import HAVE_REFERENCE_BUILD
from test_oracle import build_system


def nonsymmetric_system(O, seed=11):
    young = np.exp(np.random.default_rng(5).uniform(np.log(0.1), np.log(10.0), 8 ** 3 * 6))
    s = build_system(O, 8, 8, 8, 1.0 / 8, young)
    rng = np.random.default_rng(seed)
    vc = s["vc"] * (1.0 + 0.3 * rng.uniform(-1.0, 1.0, s["vc"].size // 9).repeat(9))
    vd = s["vd"].copy()
    O.set_fixed_bc(s["ind"], s["psup"], vc, vd, s["bc"])
    return s, vc, vd


def _factor(O, s, vc, vd, k):
    rs, col, dia = O.ilu_pattern_k(s["ind"], s["psup"], k)
    ivc, ivd = O.ilu_copy_value_k(s["ind"], s["psup"], vc, vd, k, rs, col)
    assert O.ilu_decompose(rs, col, dia, ivc, ivd)[0] == 0
    return rs, col, dia, ivc, ivd


@pytest.mark.parametrize("k", [0, 1])
@pytest.mark.parametrize("tol", [1e-10, 1e-6])
def test_port_matches_golden(port, k, tol):
    G = golden("bicgstab")
    s, vc, vd = nonsymmetric_system(port)
    f = _factor(port, s, vc, vd, k)
    x, r, hist = port.solve_pbicgstab(s["ind"], s["psup"], vc, vd, *f, s["b"], tol, 1000)
    tag = f"k{k}_t{int(-np.log10(tol))}"
    assert len(hist) == len(G[f"{tag}_hist"])
    assert rel_err(hist, G[f"{tag}_hist"]) < 1e-6
    assert rel_err(x, G[f"{tag}_x"]) < 1e-10
    assert hist[-1] < tol <= hist[-2]


def test_semantics_early_return_and_exhaustion(port):
    s, vc, vd = nonsymmetric_system(port)
    f = _factor(port, s, vc, vd, 0)
    x, r, hist = port.solve_pbicgstab(s["ind"], s["psup"], vc, vd, *f, np.zeros_like(s["b"]), 1e-10, 100)
    assert len(hist) == 1 and hist[0] == 0.0 and not x.any()  # |r0|^2 < 1e-60
    x, r, hist = port.solve_pbicgstab(s["ind"], s["psup"], vc, vd, *f, s["b"], 1e-30, 7)
    assert len(hist) == 6  # iterations 1 .. max_niter-1, no extra entry on exhaustion


@pytest.mark.skipif(not HAVE_REFERENCE_BUILD(), reason="reference source tree not available")
def test_port_equals_reference_directly(port):
    from oracle import reference
    R = reference()
    s, vc, vd = nonsymmetric_system(port, seed=12)
    f = _factor(port, s, vc, vd, 0)
    a = port.solve_pbicgstab(s["ind"], s["psup"], vc, vd, *f, s["b"], 1e-9, 500)
    b = R.solve_pbicgstab(s["ind"], s["psup"], vc, vd, *f, s["b"], 1e-9, 500)
    assert np.array_equal(a[2], b[2]) and np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
